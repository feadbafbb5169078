// Many plain-DMC steps (discrete weighting, Philox deviates) in one launch:
// the loop of DMC_Sim.propagate (pyvibdmc.py:710-876) between two events.
//
// The walkers live in shared memory.  CTA c of a cooperative grid of G CTAs
// holds a run [base_c, base_c + n_c) of the population in its logical
// (np.repeat) order.  A CTA is six mover warps and one reducer warp:
//   movers, step t:  move every walker of the run and evaluate V (the walker
//     draws from the Philox stream of its 64-bit lineage key, so nothing in
//     the move depends on other CTAs); barrier A with the reducer, which has
//     by then published step t-1's global results (vref_t, N_t, this CTA's
//     logical base, what to do next); weights and counts with vref_t; barrier
//     B (the CTA's per-thread sums handed to the reducer); scan of the counts
//     and the copies' gather index and lineage keys (copy r of walker i is the
//     next run's walker cnt[i] + r with key lineage_key(key_i, r, step)).
//   reducer, after barrier B of step t (while the movers move step t+1):
//     the CTA's sums into a 16-byte partial, grid arrival, wait for all G
//     arrivals (bounded), all partials reduced in the same fixed order in
//     every CTA (N', vref, guards, the largest CTA count, this CTA's base),
//     the history and control block (CTA 0), the next action; barrier A.
// So the grid-wide reduction of a step runs behind the next step's move.
// The action after step t, the same in every CTA:
//   go on with the copies where they are;
//   exchange: the largest CTA's run would take more warps than an even split
//     plus one, so the moved walkers of step t+1 are split evenly through
//     global memory (second grid barrier) before their weights;
//   overflow: a CTA's copies did not fit its buffer: step t's copies are split
//     evenly through global memory and step t+1 is moved again (the lineage
//     keys make the walk independent of where a walker is moved);
//   stop: the launch's last step, or a population whose even split does not
//     fit the buffers: step t's copies go to the output in logical order;
//   guard: a guard tripped at step t: its moved, unbranched walkers go to the
//     output, as the per-step kernels leave them.
// The walk is the per-step kernels' algorithm with another noise stream: a
// walker's deviates and branching uniform come from its lineage key (its
// logical index at the launch's start) instead of its logical index at every
// step.
#include <cmath>
#include <mutex>
#include "gbdmc_device.cuh"
#include "gbdmc_internal.cuh"
#include "gbdmc_stepcore.cuh"

namespace gbdmc {

constexpr int kRunMovers = 192;               // six mover warps
constexpr int kRunTPB = kRunMovers + 32;      // and the reducer warp
constexpr int kRunMaxCTA = 384;
constexpr unsigned kRunSpinLimit = 1u << 22;
constexpr unsigned kRunOverflowBit = 0x40u;   // a CTA's copies exceed its buffer (partial flag)

enum RunAction { kRunGoOn = 0, kRunExchange = 1, kRunOverflow = 2, kRunStop = 3, kRunGuard = 4 };

// A CTA's sums of one step: one 16-byte load per CTA in the reduction.
struct RunPart {
  int c;         // sum of the branch counts (the CTA's copies)
  unsigned df;   // deaths | flags << 24 (a CTA holds fewer than 2^24 walkers)
  double s0;     // sum of c V
};
static_assert(sizeof(RunPart) == 16, "RunPart is 16 bytes");
struct RunStats {  // only when the potential statistics are logged
  double s1, vmin, vmax, pad;
};

// A step's global results as the movers use them (published by the reducer).
struct RunRes {
  long long n;      // the population after the step (N')
  long long below;  // this CTA's logical base of its copies: the earlier CTAs' counts
  double vref;      // vref after the step
  int action;       // RunAction
  int pad;
};

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void red_release_add(unsigned* p, unsigned v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" : : "l"(p), "r"(v) : "memory");
}

// Bounded wait of one thread for a monotonic arrival counter to reach target.
__device__ __forceinline__ bool run_poll(const unsigned* arrive, unsigned target) {
  unsigned it = 0;
  while (ld_acquire(arrive) < target) {
    if (++it > kRunSpinLimit) return false;
    __nanosleep(32);
  }
  return true;
}

// Named barriers: all 224 threads (movers and reducer), the 192 movers.
__device__ __forceinline__ void bar_all() { asm volatile("bar.sync 1, 224;" ::: "memory"); }
__device__ __forceinline__ void bar_mov() { asm volatile("bar.sync 2, 192;" ::: "memory"); }

// Grid barrier of the movers (the exchanges): their writes released by thread
// 0's arrival after the movers' barrier, the others' acquired by its wait.
__device__ __forceinline__ bool mov_grid_barrier(unsigned* arrive, unsigned target) {
  __shared__ int s_ok;
  bar_mov();
  if (threadIdx.x == 0) {
    red_release_add(arrive, 1u);
    s_ok = run_poll(arrive, target) ? 1 : 0;
  }
  bar_mov();
  return s_ok != 0;
}

// Exclusive scan of cnt[0..n) in place by the movers, returns the total.
__device__ __forceinline__ int mov_scan(int* cnt, int n) {
  __shared__ int ws[kRunMovers / 32];
  __shared__ int s_run;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (threadIdx.x == 0) s_run = 0;
  bar_mov();
  for (int b = 0; b < n; b += kRunMovers) {
    const int i = b + threadIdx.x;
    const int c = i < n ? cnt[i] : 0;
    const int inc = warp_incl_scan(c);
    if (lane == 31) ws[wid] = inc;
    bar_mov();
    int off = s_run;
    for (int w = 0; w < wid; ++w) off += ws[w];
    if (i < n) cnt[i] = off + inc - c;
    bar_mov();
    if (threadIdx.x == kRunMovers - 1) s_run = off + inc;
    bar_mov();
  }
  return s_run;
}

struct RunArgs {
  int64_t step_end;  // stop before this step
  int kmax;          // and after at most this many steps
  int capc;          // walkers per CTA buffer
  RunPart* part;     // [2][G]
  RunStats* stat;    // [2][G]
  uint64_t* gkey;    // [ld] lineage keys of the exchanges
  uint64_t* gu;      // [ld] branching-uniform bits of the exchanges
  unsigned* sync;    // [0] partial arrivals, [1] exits, [2] exchange arrivals
};

// The CTA's shared walker state: buffer b of each double-buffered array is at
// base + b * stride (arithmetic, so that no array of pointers sits in local memory).
template <int A>
struct RunSm {
  double* x0;      // [2][3A][capc] coordinates (source / moved)
  double* v0;      // [2][capc] V of the walkers moved into buffer b
  uint64_t* key0;  // [2][capc] lineage keys: the run's, the next run's
  uint64_t* u;     // [capc] the moved walkers' branching-uniform bits
  int* who0;       // [2][capc] ancestor ids
  int* cnt;        // [capc] counts, then their exclusive scan
  int* src;        // [capc] the next run's walker i is the copy of slot src[i]
  int capc;
  __device__ __forceinline__ double* x(int b) const { return x0 + (size_t)b * 3 * A * capc; }
  __device__ __forceinline__ double* v(int b) const { return v0 + (size_t)b * capc; }
  __device__ __forceinline__ uint64_t* key(int b) const { return key0 + (size_t)b * capc; }
  __device__ __forceinline__ int* who(int b) const { return who0 + (size_t)b * capc; }
};

template <int PK, int A, int NM, bool STATS>
__global__ void __launch_bounds__(kRunTPB) k_run(const __grid_constant__ gbdmc_sim_t S, const gbdmc_walkers_t in,
                                                 gbdmc_walkers_t out, gbdmc_ctrl_t* ctrl, const RunArgs R) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int capc = R.capc, G = gridDim.x, c = blockIdx.x;
  const int tid = threadIdx.x, lane = tid & 31;
  const bool mover = tid < kRunMovers;
  RunSm<A> W;
  {
    double* d = reinterpret_cast<double*>(smem);
    W.capc = capc;
    W.x0 = d;
    W.v0 = d + (size_t)2 * 3 * A * capc;
    uint64_t* q = reinterpret_cast<uint64_t*>(W.v0 + 2 * capc);
    W.key0 = q;
    W.u = q + 2 * capc;
    int* ip = reinterpret_cast<int*>(q + 3 * capc);
    W.who0 = ip;
    W.cnt = ip + 2 * capc;
    W.src = ip + 3 * capc;
  }
  __shared__ int pc[kRunMovers], pd[kRunMovers];
  __shared__ unsigned pf[kRunMovers];
  __shared__ double ps[kRunMovers];
  __shared__ RunStats pst[STATS ? kRunMovers : 1];
  __shared__ RunRes res[2];
  __shared__ int s_abort;
  const int64_t ld = S.ld;
  const long long N0 = S.n0;
  const double n0 = (double)N0, w_hi = (n0 + n0 * 0.5) + 1.0;
  const bool track = in.who && out.who;
  const long long step0 = ctrl->step;
  const int status0 = *(volatile int*)&ctrl->status;
  const long long N_in = ctrl->n;
  const double vref_in = ctrl->vref;
  bool run = !status0 && step0 < R.step_end;
  if (run && (N_in < 0 || N_in > ld || (N_in + G - 1) / G > capc)) {
    // a start population whose even split does not fit the blocks' buffers (more
    // than the 1.5 n0 the population guard allows): refused, nothing is moved
    run = false;
    if (c == 0 && tid == 0) {
      ctrl->status = GBDMC_ST_OVERFLOW;
      ctrl->err_step = (int)step0;
    }
  }
  const long long Nst = N_in < 0 ? 0 : (N_in > ld ? ld : N_in);
  if (tid == 0) s_abort = 0;
  __syncthreads();
  if (!run) {
    // no step to run: the walkers pass through, so a queue of launches always
    // leaves the current walkers in the last launch's output
    for (int64_t g = (int64_t)c * kRunTPB + tid; g < Nst; g += (int64_t)G * kRunTPB) {
#pragma unroll
      for (int k = 0; k < 3 * A; ++k) out.x[k * ld + g] = in.x[k * ld + g];
      out.v[g] = in.v[g];
      if (track) out.who[g] = in.who[g];
      if (out.key) out.key[g] = in.key ? in.key[g] : (uint64_t)g;
    }
  } else if (mover) {
    // ------------------------------------------------------------ movers
    // the CTA's even share of the compact input, with its lineage keys (the
    // logical indices when the input has none)
    long long base = Nst * c / G;
    int n = (int)(Nst * (c + 1) / G - base);
    for (int i = tid; i < n; i += kRunMovers) {
      const int64_t g = base + i;
      const int j = (int)GBDMC_BC(i, 0, capc, kBcRunShared);
#pragma unroll
      for (int k = 0; k < 3 * A; ++k) W.x(0)[k * capc + j] = in.x[k * ld + g];
      W.who(0)[j] = track ? in.who[g] : 0;
      W.key(0)[j] = in.key ? in.key[g] : (uint64_t)g;
    }
    int sb = 0, kq = 0;         // source buffer of the run, its keys
    bool gather = false;        // the run's walker i is slot src[i] of buffer sb (else slot i)
    int mb = 0, n_prev = 0;     // the previous step: its moved buffer, run size and copies
    int tot_prev = 0;
    long long base_prev = 0, step = step0;
    unsigned nx = 0;            // exchange barriers passed
    bool moved = true;          // the run of this step has been moved
    for (unsigned t = 0;; ++t, ++step) {
      if ((long long)t > (long long)R.kmax + 1) break;  // never reached: the stop action ends the launch (the reducer checks the same)
      const bool prev_last = t > 0 && ((int)t >= R.kmax || step >= R.step_end);
      const int db = sb ^ 1;
      // 1. move and potential (no step to move after the launch's last step)
      if (!prev_last) {
        for (int i = tid; i < n; i += kRunMovers) {
          double x[3 * A], z[3 * A], gr[3 * A];
          const int j = gather ? (int)GBDMC_BC(W.src[i], 0, capc, kBcRunShared) : i;
          RngL rng(S.seed, (uint64_t)step, W.key(kq)[i], S.replica_id);
          gen_normals<NM, 3 * A>(rng, z);
          const double* xr = W.x(sb);
          double* xw = W.x(db);
#pragma unroll
          for (int k = 0; k < 3 * A; ++k) {
            x[k] = __dadd_rn(xr[k * capc + j], __dmul_rn(S.sigma[k / 3], z[k]));
            xw[k * capc + i] = x[k];
          }
          W.v(db)[i] = pes<PK, A, false>(x, S.pes, gr);
          W.u[i] = rng.bits53();
          if (track) W.who(db)[i] = W.who(sb)[j];
        }
      }
      int cur = db;  // the buffer with this step's moved walkers
      // 2. barrier A: the previous step's global results
      bar_all();
      const RunRes rp = t == 0 ? RunRes{Nst, base, vref_in, kRunGoOn, 0} : res[(t - 1) & 1];
      if (rp.action == kRunGuard) {
        // step t-1's moved, unbranched walkers (buffer mb), compact in logical order
        for (int i = tid; i < n_prev; i += kRunMovers) {
          const int64_t g = GBDMC_BC(base_prev + i, 0, ld, kBcRunOut);
#pragma unroll
          for (int k = 0; k < 3 * A; ++k) out.x[k * ld + g] = W.x(mb)[k * capc + i];
          out.v[g] = W.v(mb)[i];
          if (track) out.who[g] = W.who(mb)[i];
          if (out.key) out.key[g] = W.key(kq ^ 1)[i];
        }
        break;
      }
      if (rp.action == kRunStop || rp.action == kRunOverflow) {
        // step t-1's copies at their logical positions: the output, or the
        // exchange area from which every CTA loads an even share
        const bool stop = rp.action == kRunStop;
        for (int i = tid; i < n_prev; i += kRunMovers) {
          const int c0 = (i + 1 < n_prev ? W.cnt[i + 1] : tot_prev) - W.cnt[i];
          const int64_t g0 = rp.below + W.cnt[i];
          for (int r = 0; r < c0; ++r) {
            const int64_t go = GBDMC_BC(g0 + r, 0, ld, kBcRunOut);
#pragma unroll
            for (int k = 0; k < 3 * A; ++k) out.x[k * ld + go] = W.x(mb)[k * capc + i];
            out.v[go] = W.v(mb)[i];
            if (track) out.who[go] = W.who(mb)[i];
            const uint64_t kr = lineage_key(W.key(kq ^ 1)[i], r, (uint64_t)(step - 1));  // step t-1's copies
            if (!stop) R.gkey[go] = kr;
            else if (out.key) out.key[go] = kr;
          }
        }
        if (stop) break;
        if (!mov_grid_barrier(R.sync + 2, (unsigned)G * ++nx)) {
          if (tid == 0) atomicOr(&ctrl->status, GBDMC_ST_TIMEOUT);
          s_abort = 1;
          moved = false;
        } else {
          // the even share of step t-1's copies is this step's run; move it again
          base = rp.n * c / G;
          n = (int)(rp.n * (c + 1) / G - base);
          const int lb = db;  // neither step t-1's moved walkers (mb) nor needed any more
          for (int i = tid; i < n; i += kRunMovers) {
            const int64_t g = base + i;
            const int j = (int)GBDMC_BC(i, 0, capc, kBcRunShared);
#pragma unroll
            for (int k = 0; k < 3 * A; ++k) W.x(lb)[k * capc + j] = __ldcg(out.x + k * ld + g);
            W.who(lb)[j] = track ? __ldcg(out.who + g) : 0;
            W.key(kq)[j] = __ldcg(R.gkey + g);
          }
          bar_mov();
          sb = lb;
          gather = false;
          const int db2 = sb ^ 1;
          for (int i = tid; i < n; i += kRunMovers) {
            double x[3 * A], z[3 * A], gr[3 * A];
            RngL rng(S.seed, (uint64_t)step, W.key(kq)[i], S.replica_id);
            gen_normals<NM, 3 * A>(rng, z);
#pragma unroll
            for (int k = 0; k < 3 * A; ++k) {
              x[k] = __dadd_rn(W.x(sb)[k * capc + i], __dmul_rn(S.sigma[k / 3], z[k]));
              W.x(db2)[k * capc + i] = x[k];
            }
            W.v(db2)[i] = pes<PK, A, false>(x, S.pes, gr);
            W.u[i] = rng.bits53();
            if (track) W.who(db2)[i] = W.who(sb)[i];
          }
          cur = db2;
        }
      } else {
        base = rp.below;
        if (rp.action == kRunExchange) {
          // this step's moved walkers split evenly: through the exchange area
          for (int i = tid; i < n; i += kRunMovers) {
            const int64_t g = GBDMC_BC(base + i, 0, ld, kBcRunOut);
#pragma unroll
            for (int k = 0; k < 3 * A; ++k) out.x[k * ld + g] = W.x(cur)[k * capc + i];
            out.v[g] = W.v(cur)[i];
            if (track) out.who[g] = W.who(cur)[i];
            R.gkey[g] = W.key(kq)[i];
            R.gu[g] = W.u[i];
          }
          if (!mov_grid_barrier(R.sync + 2, (unsigned)G * ++nx)) {
            if (tid == 0) atomicOr(&ctrl->status, GBDMC_ST_TIMEOUT);
            s_abort = 1;
            moved = false;
          } else {
            base = rp.n * c / G;
            n = (int)(rp.n * (c + 1) / G - base);
            const int lb = cur ^ 1;
            for (int i = tid; i < n; i += kRunMovers) {
              const int64_t g = base + i;
              const int j = (int)GBDMC_BC(i, 0, capc, kBcRunShared);
#pragma unroll
              for (int k = 0; k < 3 * A; ++k) W.x(lb)[k * capc + j] = __ldcg(out.x + k * ld + g);
              W.v(lb)[j] = __ldcg(out.v + g);
              W.who(lb)[j] = track ? __ldcg(out.who + g) : 0;
              W.key(kq)[j] = __ldcg(R.gkey + g);
              W.u[j] = __ldcg(R.gu + g);
            }
            cur = lb;
          }
        }
      }
      // 3. weights and counts with this step's vref
      const double vref = rp.vref;
      int csum = 0, flag = 0;
      long long births = 0, deaths = 0;
      double s0 = 0.0;
      RunStats st = {0.0, INFINITY, -INFINITY, 0.0};
      if (moved) {
        bar_mov();
        for (int i = tid; i < n; i += kRunMovers) {
          const double v = W.v(cur)[i];
          if (STATS) {
            st.s1 += v;
            st.vmin = fmin(st.vmin, v);
            st.vmax = fmax(st.vmax, v);
          }
          const int cn = branch_count(v, vref, S.dt, (double)W.u[i] * 0x1.0p-53, w_hi, flag, births, deaths);
          W.cnt[i] = cn;
          csum += cn;
          s0 += cn == 1 ? v : (double)cn * v;
        }
      }
      pc[tid] = csum;
      pd[tid] = (int)deaths;
      pf[tid] = (unsigned)flag;
      ps[tid] = s0;
      if (STATS) pst[tid] = st;
      // 4. barrier B: the sums to the reducer
      bar_all();
      if (s_abort) {
        moved = true;
        continue;  // the reducer publishes the abort at the next barrier A
      }
      // 5. the copies' gather index and lineage keys (the next run)
      const int tot = mov_scan(W.cnt, n);
      for (int i = tid; i < n; i += kRunMovers) {
        const int c0 = (i + 1 < n ? W.cnt[i + 1] : tot) - W.cnt[i];
        const int j0 = W.cnt[i];
        for (int r = 0; r < c0; ++r) {
          const int j = j0 + r;
          if (j < capc) {  // a CTA's copies past its buffer: the overflow action follows
            W.src[j] = i;
            W.key(kq ^ 1)[j] = lineage_key(W.key(kq)[i], r, (uint64_t)step);
          }
        }
      }
      bar_mov();
      mb = cur;
      n_prev = n;
      tot_prev = tot;
      base_prev = base;
      sb = cur;
      kq ^= 1;
      gather = true;
      n = tot < capc ? tot : capc;
    }
  } else {
    // ----------------------------------------------------------- reducer
    long long N = Nst;  // the population moved at step t
    double vref = vref_in;
    long long step = step0;
    unsigned narr = 0;
    for (unsigned t = 0;; ++t, ++step) {
      if ((long long)t > (long long)R.kmax + 1) break;  // as the movers
      // barrier A of step t: the movers have read nothing of step t yet
      bar_all();
      if (t > 0) {
        const int act = res[(t - 1) & 1].action;
        if (act == kRunGuard || act == kRunStop) break;
      }
      // barrier B of step t: the movers' per-thread sums
      bar_all();
      const unsigned full = 0xffffffffu;
      int cc = 0, dd = 0;
      unsigned ff = 0;
      double q = 0.0;
      RunStats qs = {0.0, INFINITY, -INFINITY, 0.0};
#pragma unroll
      for (int w = 0; w < kRunMovers / 32; ++w) {
        const int k = lane + 32 * w;
        cc += pc[k];
        dd += pd[k];
        ff |= pf[k];
        q += ps[k];
        if (STATS) {
          qs.s1 += pst[k].s1;
          qs.vmin = fmin(qs.vmin, pst[k].vmin);
          qs.vmax = fmax(qs.vmax, pst[k].vmax);
        }
      }
      cc = (int)__reduce_add_sync(full, (unsigned)cc);
      dd = (int)__reduce_add_sync(full, (unsigned)dd);
      ff = __reduce_or_sync(full, ff);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) q += __shfl_xor_sync(full, q, o);
      if (STATS) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) qs.s1 += __shfl_xor_sync(full, qs.s1, o);
        qs.vmin = dkey_inv(warp_min_key(dkey(qs.vmin)));
        qs.vmax = dkey_inv(warp_max_key(dkey(qs.vmax)));
      }
      const int par = t & 1;
      bool ok = s_abort == 0;  // the movers gave up on an exchange barrier: no arrival
      if (lane == 0 && ok) {
        if (cc > capc) ff |= kRunOverflowBit;
        RunPart pp;
        pp.c = cc;
        pp.df = (unsigned)dd | (ff << 24);
        pp.s0 = q;
        R.part[par * G + c] = pp;
        if (STATS) R.stat[par * G + c] = qs;
        red_release_add(R.sync, 1u);
        ok = run_poll(R.sync, (unsigned)G * ++narr);
      } else if (ok) {
        ++narr;
      }
      ok = __shfl_sync(full, ok ? 1 : 0, 0) != 0;
      __syncwarp();  // lane 0's acquire of the arrivals orders the warp's loads of the partials
      // every CTA's partial: the same reduction in every CTA (all loads first)
      unsigned nn = 0, below = 0;
      int nd = 0, cmax = 0;
      unsigned f = 0;
      double q0 = 0.0;
      RunStats rs = {0.0, INFINITY, -INFINITY, 0.0};
      if (ok) {
        int4 rpv[kRunMaxCTA / 32];
        const int4* pp = reinterpret_cast<const int4*>(R.part + par * G);
#pragma unroll
        for (int k = 0; k < kRunMaxCTA / 32; ++k) {
          const int g = lane + 32 * k;
          rpv[k] = g < G ? __ldcg(pp + g) : make_int4(0, 0, 0, 0);
        }
#pragma unroll
        for (int k = 0; k < kRunMaxCTA / 32; ++k) {
          const int g = lane + 32 * k;
          const int4 r = rpv[k];
          const int rc = r.x;
          nn += (unsigned)rc;
          nd += (int)((unsigned)r.y & 0xFFFFFFu);
          f |= (unsigned)r.y >> 24;
          if (g < G) q0 += __hiloint2double(r.w, r.z);
          if (g < c) below += (unsigned)rc;
          cmax = rc > cmax ? rc : cmax;
          if (STATS && g < G) {
            const double2 a = __ldcg(reinterpret_cast<const double2*>(R.stat + par * G + g));
            const double2 b = __ldcg(reinterpret_cast<const double2*>(R.stat + par * G + g) + 1);
            rs.s1 += a.x;
            rs.vmin = fmin(rs.vmin, a.y);
            rs.vmax = fmax(rs.vmax, b.x);
          }
        }
      }
      if (STATS) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) rs.s1 += __shfl_xor_sync(full, rs.s1, o);
        rs.vmin = dkey_inv(warp_min_key(dkey(rs.vmin)));
        rs.vmax = dkey_inv(warp_max_key(dkey(rs.vmax)));
      }
      nn = __reduce_add_sync(full, nn);
      below = __reduce_add_sync(full, below);
      nd = (int)__reduce_add_sync(full, (unsigned)nd);
      cmax = (int)__reduce_max_sync(full, (unsigned)cmax);
      f = __reduce_or_sync(full, f);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) q0 += __shfl_xor_sync(full, q0, o);
      // 32-bit sums: exact while every block holds fewer than 2^31 / kRunMaxCTA
      // copies; a larger block count is a population past any guard (N' > 1.5 N0)
      const bool huge = cmax >= (int)(0x7fffffff / kRunMaxCTA);
      const long long Nn = huge ? (long long)INT32_MAX * 4 : (long long)nn;
      // the step's divisions, one SIMT division: <V> of the branched population
      // (lane 0), the population term (lane 1), the mean potential (lane 2)
      const double num = lane == 0 ? q0 : (lane == 1 ? (double)(Nn - N0) : rs.s1);
      const double den = lane == 0 ? (double)Nn : (lane == 1 ? n0 : (double)N);
      const double qq = num / den;
      const double vbar = __shfl_sync(full, qq, 0), corr = __shfl_sync(full, qq, 1);
      const double vmean = __shfl_sync(full, qq, 2);
      const double vr = vbar - S.alpha * corr;
      int st2 = ok ? (int)(f & 0x3Fu) : GBDMC_ST_TIMEOUT;
      if (!st2) {
        if ((double)Nn < n0 - n0 * 0.5) st2 |= GBDMC_ST_POP_LOW;
        if ((double)Nn > n0 + n0 * 0.5) st2 |= GBDMC_ST_POP_HIGH;
        if (Nn > ld) st2 |= GBDMC_ST_OVERFLOW;
      }
      const long long even = huge ? (long long)INT32_MAX : (long long)((nn + (unsigned)G - 1u) / (unsigned)G);
      const bool last = (int)t + 1 >= R.kmax || step + 1 >= R.step_end;
      // the largest CTA's copies against the warps of an even split plus one
      const long long lim = ((even + 31) / 32) * 32 + 32;
      int act = kRunGoOn;
      if (st2) act = kRunGuard;
      else if (last || even > capc) act = kRunStop;
      else if (f & kRunOverflowBit) act = kRunOverflow;
      else if ((long long)cmax > (lim < capc ? lim : (long long)capc)) act = kRunExchange;
      if (lane == 0) {
        if (c == 0 && step < S.hist.len && ok) {
          const int64_t h = step;
          if (STATS) {
            if (S.hist.vmin) S.hist.vmin[h] = rs.vmin;
            if (S.hist.vmax) S.hist.vmax[h] = rs.vmax;
            if (S.hist.vmean) S.hist.vmean[h] = vmean;
          }
          if (!st2) {
            if (S.hist.vref) S.hist.vref[h] = vr;
            if (S.hist.pop) S.hist.pop[h] = (double)Nn;
            if (S.hist.births) S.hist.births[h] = (int)(Nn - (N - nd));  // sum of max(c - 1, 0)
            if (S.hist.deaths) S.hist.deaths[h] = nd;
          }
        }
        if (c == 0) {
          if (st2) {  // as a failed per-step call leaves it: moved walkers, N, vref and step of the step
            ctrl->n = N;
            ctrl->vref = vref;
            ctrl->step = step;
            atomicOr(&ctrl->status, st2);
            ctrl->err_step = (int)step;
          } else if (act == kRunStop) {
            ctrl->n_prev = N;
            ctrl->n = Nn;
            ctrl->vref = vr;
            ctrl->step = step + 1;
          }
        }
        res[par] = RunRes{Nn, (long long)below, vr, act, 0};
      }
      N = Nn;
      vref = vr;
    }
  }
  // the last CTA out resets the barrier words for the next launch
  __syncthreads();
  if (tid == 0) {
    __threadfence();
    if (atomicAdd(&R.sync[1], 1u) == (unsigned)G - 1) {
      R.sync[0] = 0;
      R.sync[1] = 0;
      R.sync[2] = 0;
    }
  }
}

// The deviates and branching uniforms of walkers with the given lineage keys
// at one step, as the multi-step kernel draws them (for checking its
// trajectory with the per-step kernels on injected noise).
template <int NM, int A>
__global__ void k_lineage_noise(uint64_t seed, uint32_t replica, int64_t step, const uint64_t* __restrict__ keys,
                                int64_t n, double* __restrict__ normal, int64_t ldn, double* __restrict__ u) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    RngL rng(seed, (uint64_t)step, keys[i], replica);
    double z[3 * A];
    gen_normals<NM, 3 * A>(rng, z);
#pragma unroll
    for (int k = 0; k < 3 * A; ++k) normal[k * ldn + i] = z[k];
    u[i] = rng.uniform53();
  }
}

template <int NM>
static void lineage_noise_launch(const gbdmc_sim_t& S, const uint64_t* keys, int64_t n, int64_t step, double* normal,
                                 int64_t ldn, double* u, cudaStream_t s) {
  const int grid = (int)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096);
  if (S.natoms == 1)
    k_lineage_noise<NM, 1><<<grid, 256, 0, s>>>(S.seed, S.replica_id, step, keys, n, normal, ldn, u);
  else if (S.natoms == 3)
    k_lineage_noise<NM, 3><<<grid, 256, 0, s>>>(S.seed, S.replica_id, step, keys, n, normal, ldn, u);
  else
    k_lineage_noise<NM, 6><<<grid, 256, 0, s>>>(S.seed, S.replica_id, step, keys, n, normal, ldn, u);
}

// ------------------------------------------------------------ host side
// Per walker slot: two coordinate buffers, two V, two lineage keys, the
// branching-uniform bits, two ancestor ids, the count and the gather index.
static size_t run_smem_bytes(int A, int capc) {
  return (size_t)capc * (2 * 3 * A * sizeof(double) + 2 * sizeof(double) + 3 * sizeof(uint64_t) + 4 * sizeof(int));
}

struct RunShape {
  int grid, capc;
  size_t smem;
};

template <int PK, int A, int NM, bool STATS>
static int run_launch(const gbdmc_sim_t& S, const gbdmc_walkers_t& src, const gbdmc_walkers_t& dst,
                      gbdmc_ctrl_t* ctrl, const RunArgs& R, const RunShape& sh, cudaStream_t s) {
  auto kern = k_run<PK, A, NM, STATS>;
  static std::mutex mu;
  static size_t attr_set = 0;
  {
    std::lock_guard<std::mutex> lk(mu);
    if (sh.smem > attr_set) {
      if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh.smem) != cudaSuccess) {
        set_error("gbdmc_sim_run: %zu bytes of shared memory per block refused", sh.smem);
        return GBDMC_ERR_CUDA;
      }
      attr_set = sh.smem;
    }
  }
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kRunTPB, sh.smem) != cudaSuccess ||
      per_sm * num_sms() < sh.grid) {
    set_error("gbdmc_sim_run: %d co-resident blocks of %zu shared bytes do not fit", sh.grid, sh.smem);
    return GBDMC_ERR_CAPACITY;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)sh.grid);
  cfg.blockDim = dim3(kRunTPB);
  cfg.dynamicSmemBytes = sh.smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeCooperative;
  at[0].val.cooperative = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  if (cudaLaunchKernelEx(&cfg, kern, S, src, dst, ctrl, R) != cudaSuccess) {
    (void)cudaGetLastError();
    set_error("gbdmc_sim_run: cooperative launch of %d blocks failed", sh.grid);
    return GBDMC_ERR_CUDA;
  }
  return check_launch("gbdmc_sim_run");
}

template <int PK, int A>
static int run_dispatch(const gbdmc_sim_t& S, const gbdmc_walkers_t& src, const gbdmc_walkers_t& dst,
                        gbdmc_ctrl_t* ctrl, const RunArgs& R, const RunShape& sh, cudaStream_t s) {
  const bool stats = S.hist.vmin || S.hist.vmax || S.hist.vmean;
  if (S.noise_mode == GBDMC_NOISE_PHILOX32)
    return stats ? run_launch<PK, A, GBDMC_NOISE_PHILOX32, true>(S, src, dst, ctrl, R, sh, s)
                 : run_launch<PK, A, GBDMC_NOISE_PHILOX32, false>(S, src, dst, ctrl, R, sh, s);
  return stats ? run_launch<PK, A, GBDMC_NOISE_PHILOX64, true>(S, src, dst, ctrl, R, sh, s)
               : run_launch<PK, A, GBDMC_NOISE_PHILOX64, false>(S, src, dst, ctrl, R, sh, s);
}

// Grid and per-CTA buffers of a launch: about 96 walkers per CTA, at most one
// CTA per SM (and kRunMaxCTA); each CTA's buffers hold its even share of the
// largest population the guard allows (1.5 n0) with a margin.
static int run_shape(const gbdmc_sim_t& S, RunShape& sh) {
  const int A = S.natoms;
  int g = (int)((S.n0 + 95) / 96);
  const int lim = num_sms() < kRunMaxCTA ? num_sms() : kRunMaxCTA;
  g = g < 1 ? 1 : (g > lim ? lim : g);
  const int64_t capc = ((S.n0 * 3 / 2 + 1 + g - 1) / g + 64 + 31) / 32 * 32;
  const size_t smax = 200 * 1024;
  if (capc > (1 << 20) || run_smem_bytes(A, (int)capc) > smax) {
    set_error("gbdmc_sim_run: %lld walkers per block buffer do not fit shared memory (%zu bytes); use "
              "gbdmc_sim_step", (long long)capc, run_smem_bytes(A, (int)(capc > (1 << 20) ? 1 << 20 : capc)));
    return GBDMC_ERR_CAPACITY;
  }
  sh.grid = g;
  sh.capc = (int)capc;
  sh.smem = run_smem_bytes(A, (int)capc);
  return GBDMC_OK;
}

static size_t run_scratch_head() {
  return align256(sizeof(RunPart) * 2 * kRunMaxCTA) + align256(sizeof(RunStats) * 2 * kRunMaxCTA) +
         align256(4 * sizeof(unsigned));
}

GBDMC_BOUNDS_READER(bounds_read_run)

}  // namespace gbdmc

using namespace gbdmc;

extern "C" size_t gbdmc_sim_run_scratch_bytes(int64_t ld) {
  return run_scratch_head() + 2 * align256((size_t)(ld > 0 ? ld : 0) * sizeof(uint64_t));
}

extern "C" int gbdmc_sim_run(const gbdmc_sim_t* S, const gbdmc_walkers_t* src, const gbdmc_walkers_t* dst,
                             gbdmc_ctrl_t* ctrl, void* scratch, int64_t step_end, int32_t max_steps, void* stream) {
  const char* what = "gbdmc_sim_run";
  if (!S || !src || !dst || !ctrl || !scratch || !src->x || !dst->x || !dst->v) {
    set_error("%s: null argument", what);
    return GBDMC_ERR_ARG;
  }
  if (src->idx || src->x == dst->x || (src->who && src->who == dst->who) || (S->track_who && (!src->who || !dst->who))) {
    set_error("%s: src must be compact (idx NULL), src and dst separate, who in both when tracked", what);
    return GBDMC_ERR_ARG;
  }
  if (S->weighting != GBDMC_DISCRETE || S->trial.kind != GBDMC_TRIAL_NONE ||
      S->noise_mode == GBDMC_NOISE_INJECTED || S->pes.kind == GBDMC_PES_EXTERNAL) {
    set_error("%s: runs plain DMC with discrete weighting, Philox deviates and a built-in potential", what);
    return GBDMC_ERR_ARG;
  }
  if (S->n0 < 1 || S->ld < 1 || S->ld > (int64_t)INT32_MAX || S->natoms < 1 || S->pes.natoms != S->natoms) {
    set_error("%s: bad sizes (n0=%lld ld=%lld natoms=%d)", what, (long long)S->n0, (long long)S->ld, S->natoms);
    return GBDMC_ERR_ARG;
  }
  if (max_steps < 1) {
    set_error("%s: max_steps must be >= 1", what);
    return GBDMC_ERR_ARG;
  }
  RunShape sh;
  int rc = run_shape(*S, sh);
  if (rc) return rc;
  char* b = (char*)scratch;
  RunArgs R;
  R.step_end = step_end;
  // at most two grid barriers per step on a 32-bit arrival counter
  const int kcap = (int)((1u << 31) / (2u * (unsigned)sh.grid));
  R.kmax = max_steps < kcap ? max_steps : kcap;
  R.capc = sh.capc;
  R.part = (RunPart*)b;
  R.stat = (RunStats*)(b + align256(sizeof(RunPart) * 2 * kRunMaxCTA));
  R.sync = (unsigned*)(b + align256(sizeof(RunPart) * 2 * kRunMaxCTA) + align256(sizeof(RunStats) * 2 * kRunMaxCTA));
  R.gkey = (uint64_t*)(b + run_scratch_head());
  R.gu = (uint64_t*)(b + run_scratch_head() + align256((size_t)S->ld * sizeof(uint64_t)));
  cudaStream_t s = (cudaStream_t)stream;
  const int PK = S->pes.kind, A = S->natoms;
  if (PK == GBDMC_PES_HO && A == 1) return run_dispatch<GBDMC_PES_HO, 1>(*S, *src, *dst, ctrl, R, sh, s);
  if (PK == GBDMC_PES_HO && A == 3) return run_dispatch<GBDMC_PES_HO, 3>(*S, *src, *dst, ctrl, R, sh, s);
  if (PK == GBDMC_PES_H2O_LM && A == 3) return run_dispatch<GBDMC_PES_H2O_LM, 3>(*S, *src, *dst, ctrl, R, sh, s);
  if (PK == GBDMC_PES_H2O_PS && A == 3) return run_dispatch<GBDMC_PES_H2O_PS, 3>(*S, *src, *dst, ctrl, R, sh, s);
  if (PK == GBDMC_PES_DIMER && A == 6) return run_dispatch<GBDMC_PES_DIMER, 6>(*S, *src, *dst, ctrl, R, sh, s);
  set_error("%s: unsupported system (pes %d, atoms %d)", what, PK, A);
  return GBDMC_ERR_ARG;
}

// The output of a gbdmc_sim_run_host call written straight into the host's
// page-locked arrays over the host link: the control block, the ctrl->n
// walkers of dst (x, v, who, key) and the history of the steps run.
__global__ void k_export_host(const gbdmc_ctrl_t* __restrict__ ctrl, gbdmc_walkers_t dst, int64_t ld, int A3,
                              gbdmc_host_walkers_t host, gbdmc_ctrl_t* ctrl_host, gbdmc_history_t hist, int64_t step0,
                              int32_t max_steps, double* hist_host) {
  const int64_t n = ctrl->n;
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, nth = (int64_t)gridDim.x * blockDim.x;
  if (tid == 0) *ctrl_host = *ctrl;
  const int64_t m = n < ld ? (n < 0 ? 0 : n) : ld;
  for (int64_t i = tid; i < m; i += nth) {
    for (int k = 0; k < A3; ++k) host.x[k * host.ld + i] = dst.x[k * ld + i];
    if (host.v) host.v[i] = dst.v[i];
    if (host.who) host.who[i] = dst.who[i];
    if (host.key) host.key[i] = dst.key[i];
  }
  if (hist_host && hist.vref && hist.pop && step0 >= 0 && step0 < hist.len) {
    int64_t k = ctrl->step - step0;
    if (k > max_steps) k = max_steps;
    if (k > hist.len - step0) k = hist.len - step0;
    for (int64_t j = tid; j < k; j += nth) {
      hist_host[j] = hist.vref[step0 + j];
      hist_host[max_steps + j] = hist.pop[step0 + j];
    }
  }
}

extern "C" int gbdmc_sim_run_host(const gbdmc_sim_t* S, gbdmc_host_walkers_t* host, const gbdmc_walkers_t* dev_src,
                                  const gbdmc_walkers_t* dev_dst, gbdmc_ctrl_t* ctrl, gbdmc_ctrl_t* ctrl_host,
                                  void* scratch, int64_t step_end, int32_t max_steps, double* hist_host,
                                  void* stream) {
  const char* what = "gbdmc_sim_run_host";
  if (!S || !host || !host->x || !dev_src || !dev_dst || !ctrl || !ctrl_host || !dev_src->x || !dev_dst->x ||
      !dev_dst->v || host->ld < S->ld || max_steps < 1) {
    set_error("%s: null argument, host->ld below sim->ld, or max_steps < 1", what);
    return GBDMC_ERR_ARG;
  }
  const int64_t n = ctrl_host->n;
  if (n < 0 || n > S->ld || (host->who && (!dev_src->who || !dev_dst->who)) ||
      (host->key && (!dev_src->key || !dev_dst->key)) || (S->track_who && !host->who)) {
    set_error("%s: bad population (%lld) or missing device arrays for the host's who / key", what, (long long)n);
    return GBDMC_ERR_ARG;
  }
  gbdmc_walkers_t src = *dev_src, dst = *dev_dst;
  if (!host->key) src.key = dst.key = nullptr;  // the launch takes the logical indices
  const cudaStream_t s = (cudaStream_t)stream;
  const int A3 = 3 * S->natoms;
  cudaError_t e = cudaSuccess;
  if (host->ld == S->ld) {
    // the launch reads its input straight from the host arrays (page-locked
    // memory is addressable from the device under unified addressing)
    src.x = host->x;
    src.who = host->who ? host->who : src.who;
    src.key = host->key;
  } else if (n > 0) {
    const size_t dp = (size_t)S->ld * sizeof(double), hp = (size_t)host->ld * sizeof(double);
    e = cudaMemcpy2DAsync(src.x, dp, host->x, hp, (size_t)n * sizeof(double), A3, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && host->who)
      e = cudaMemcpyAsync(src.who, host->who, (size_t)n * sizeof(int32_t), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && host->key)
      e = cudaMemcpyAsync(src.key, host->key, (size_t)n * sizeof(uint64_t), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) {
      set_error("%s: host -> device copy: %s", what, cudaGetErrorString(e));
      return GBDMC_ERR_CUDA;
    }
  }
  const int64_t step0 = ctrl_host->step;
  int rc = gbdmc_sim_run(S, &src, &dst, ctrl, scratch, step_end, max_steps, stream);
  if (rc) return rc;
  k_export_host<<<2 * num_sms(), 256, 0, s>>>(ctrl, dst, S->ld, A3, *host, ctrl_host, S->hist, step0, max_steps,
                                              hist_host);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    set_error("%s: %s", what, cudaGetErrorString(e));
    return GBDMC_ERR_CUDA;
  }
  return GBDMC_OK;
}

extern "C" int gbdmc_lineage_noise(const gbdmc_sim_t* sim, const uint64_t* keys_dev, int64_t n, int64_t step,
                                   double* normal_dev, int64_t ld_noise, double* u_dev, void* stream) {
  if (!sim || n < 0 || ld_noise < n || (n > 0 && (!keys_dev || !normal_dev || !u_dev))) {
    set_error("gbdmc_lineage_noise: invalid arguments");
    return GBDMC_ERR_ARG;
  }
  if (sim->natoms != 1 && sim->natoms != 3 && sim->natoms != 6) {
    set_error("gbdmc_lineage_noise: %d atoms (1, 3 or 6)", sim->natoms);
    return GBDMC_ERR_ARG;
  }
  if (n == 0) return GBDMC_OK;
  const cudaStream_t s = (cudaStream_t)stream;
  if (sim->noise_mode == GBDMC_NOISE_PHILOX64)
    lineage_noise_launch<GBDMC_NOISE_PHILOX64>(*sim, keys_dev, n, step, normal_dev, ld_noise, u_dev, s);
  else
    lineage_noise_launch<GBDMC_NOISE_PHILOX32>(*sim, keys_dev, n, step, normal_dev, ld_noise, u_dev, s);
  return check_launch("gbdmc_lineage_noise");
}
