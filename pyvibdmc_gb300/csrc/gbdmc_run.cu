// Many plain-DMC steps (discrete weighting, Philox deviates) in one launch:
// the loop of DMC_Sim.propagate (pyvibdmc.py:710-876) between two events.
//
// The walkers of a step live in shared memory.  CTA c of a cooperative grid
// of G CTAs holds a run [base_c, base_c + n_c) of the population in its
// logical (np.repeat) order, the runs of the CTAs back to back.  One step:
//   1. every walker of the CTA moves (x + fl(sigma z) from Philox, keyed by
//      its logical index base_c + i as in k_move), its potential, weight and
//      count (pyvibdmc.py:540-547, :392-403); the CTA's 16-byte partial (sum
//      c, sum cV, deaths, guards; sum V / min / max when logging apart) goes
//      to global memory;
//   2. a grid barrier (bounded wait, GBDMC_ST_TIMEOUT on expiry);
//   3. warp 0 of every CTA reduces the G partials in the same fixed order, so
//      all CTAs hold the same N', vref' (calc_vref, :651-661), guards and
//      largest CTA count, and the CTA's new base is the earlier CTAs' counts;
//   4. the CTA's copies (np.repeat order) become its next run.  Normally they
//      stay in shared memory (the other half of a double buffer).  When the
//      largest CTA's copies would take more warps than an even split of N'
//      (or no double buffer fits), every CTA writes its copies to the output
//      at their logical positions, a second grid barrier follows, and every
//      CTA loads its even share of the new population back: the step's time
//      is that of the CTA with the most walkers, so the runs are split evenly
//      again before one of them grows by a warp.
// After the last step of the launch the copies go to the output, which then
// holds the branched population compact in logical order.  A step whose
// guards trip writes its moved, unbranched walkers to the output and stops,
// as the per-step kernels do.
// The deviates and branching uniforms are those of the per-step kernels
// (same Philox counters), so the trajectories agree; vref sums the CTA
// partials in another order (last-bit differences).
#include <cmath>
#include <mutex>
#include "gbdmc_device.cuh"
#include "gbdmc_internal.cuh"
#include "gbdmc_stepcore.cuh"

namespace gbdmc {

constexpr int kRunTPB = 192;
constexpr int kRunMaxCTA = 384;
constexpr unsigned kRunSpinLimit = 1u << 22;

// A CTA's sums of one step: one 16-byte load per CTA in the reduction.
struct RunPart {
  int c;         // sum of the branch counts (the CTA's copies)
  unsigned df;   // deaths | guard bits << 24 (a CTA holds fewer than 2^24 walkers)
  double s0;     // sum of c V
};
static_assert(sizeof(RunPart) == 16, "RunPart is 16 bytes");
struct RunStats {  // only when the potential statistics are logged
  double s1, vmin, vmax, pad;
};

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void red_release_add(unsigned* p, unsigned v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" : : "l"(p), "r"(v) : "memory");
}

// Grid barrier over a monotonic arrival counter: the CTA's writes are released
// by thread 0's arrival after the block barrier, the others' acquired by its
// wait before the next one.  Returns false if the wait ran out (the caller
// stops; the other CTAs' next waits run out as well).
__device__ __forceinline__ bool run_barrier(unsigned* arrive, unsigned target) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    red_release_add(arrive, 1u);
    int ok = 1;
    unsigned it = 0;
    while (ld_acquire(arrive) < target) {
      if (++it > kRunSpinLimit) {
        ok = 0;
        break;
      }
      __nanosleep(32);
    }
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// The two halves of the per-step barrier, apart so that a block's own work
// (the scan of its counts) runs while the other blocks arrive.  Thread 0
// arrives after writing the block's partial: the release orders that write
// before the arrival.  run_wait: bounded, false when the wait ran out.
__device__ __forceinline__ void run_arrive(unsigned* arrive) { red_release_add(arrive, 1u); }

__device__ __forceinline__ bool run_wait(const unsigned* arrive, unsigned target) {
  __shared__ int s_ok;
  if (threadIdx.x == 0) {
    int ok = 1;
    unsigned it = 0;
    while (ld_acquire(arrive) < target) {
      if (++it > kRunSpinLimit) {
        ok = 0;
        break;
      }
      __nanosleep(32);
    }
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// Exclusive scan of cnt[0..n) in place (chunks of the block), returns the total.
__device__ __forceinline__ int run_scan(int* cnt, int n) {
  __shared__ int ws[kRunTPB / 32];
  __shared__ int s_run;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (threadIdx.x == 0) s_run = 0;
  __syncthreads();
  for (int b = 0; b < n; b += kRunTPB) {
    const int i = b + threadIdx.x;
    const int c = i < n ? cnt[i] : 0;
    const int inc = warp_incl_scan(c);
    if (lane == 31) ws[wid] = inc;
    __syncthreads();
    int off = s_run;
    for (int w = 0; w < wid; ++w) off += ws[w];
    if (i < n) cnt[i] = off + inc - c;
    __syncthreads();
    if (threadIdx.x == kRunTPB - 1) s_run = off + inc;
    __syncthreads();
  }
  return s_run;
}

struct RunArgs {
  int64_t step_end;  // stop before this step
  int kmax;          // and after at most this many steps
  int capc;          // walkers per CTA buffer
  int dbuf;          // 1: two walker buffers per CTA (copies stay in shared memory)
  RunPart* part;     // [2][G]
  RunStats* stat;    // [2][G]
  unsigned* sync;    // [0] arrivals, [1] exits
};

// The CTA's sums of step 1, reduced over the block: valid in thread 0.
template <bool STATS>
__device__ __forceinline__ void run_block_sums(int& c, int& d, unsigned& f, double& s0, RunStats& st) {
  __shared__ int4 sh_i[kRunTPB / 32];
  __shared__ double sh_d[kRunTPB / 32][4];
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  c = (int)__reduce_add_sync(full, (unsigned)c);
  d = (int)__reduce_add_sync(full, (unsigned)d);
  f = __reduce_or_sync(full, f);
  if (STATS) {
    warp_sum2(s0, st.s1);
    st.vmin = dkey_inv(warp_min_key(dkey(st.vmin)));
    st.vmax = dkey_inv(warp_max_key(dkey(st.vmax)));
  } else {
    s0 = warp_sum(s0);
  }
  if (lane == 0) {
    sh_i[wid] = make_int4(c, d, (int)f, 0);
    sh_d[wid][0] = s0;
    if (STATS) {
      sh_d[wid][1] = st.s1;
      sh_d[wid][2] = st.vmin;
      sh_d[wid][3] = st.vmax;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int4 a = sh_i[0];
    s0 = sh_d[0][0];
    if (STATS) {
      st.s1 = sh_d[0][1];
      st.vmin = sh_d[0][2];
      st.vmax = sh_d[0][3];
    }
#pragma unroll
    for (int w = 1; w < kRunTPB / 32; ++w) {
      const int4 b = sh_i[w];
      a.x += b.x;
      a.y += b.y;
      a.z |= b.z;
      s0 += sh_d[w][0];
      if (STATS) {
        st.s1 += sh_d[w][1];
        st.vmin = fmin(st.vmin, sh_d[w][2]);
        st.vmax = fmax(st.vmax, sh_d[w][3]);
      }
    }
    c = a.x;
    d = a.y;
    f = (unsigned)a.z;
  }
}

template <int PK, int A, int NM, bool STATS>
__global__ void __launch_bounds__(kRunTPB) k_run(const __grid_constant__ gbdmc_sim_t S, const gbdmc_walkers_t in,
                                                 gbdmc_walkers_t out, gbdmc_ctrl_t* ctrl, const RunArgs R) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int capc = R.capc, G = gridDim.x, c = blockIdx.x, nbuf = R.dbuf ? 2 : 1;
  const int lane = threadIdx.x & 31;
  double* xsb = reinterpret_cast<double*>(smem);     // [nbuf][3A][capc]
  double* vs = xsb + (size_t)nbuf * 3 * A * capc;     // [capc]
  int* whob = reinterpret_cast<int*>(vs + capc);      // [nbuf][capc]
  int* cnt = whob + (size_t)nbuf * capc;              // [capc]
  int* src = cnt + capc;                              // [capc] the run's walker i is slot src[i] of its buffer
  __shared__ long long s_base, s_nc, s_nnew, s_N;
  __shared__ double s_vref;
  __shared__ int s_stop;  // 0 go on, 1 branch to the output and end, 2 guards tripped
  __shared__ int s_even;  // 1: every CTA takes its even share of the new population
  const int64_t ld = S.ld;
  const long long N0 = S.n0;
  const double n0 = (double)N0, w_hi = (n0 + n0 * 0.5) + 1.0;
  const bool track = in.who && out.who;
  long long step = ctrl->step;
  int status = *(volatile int*)&ctrl->status;
  const long long N_in = ctrl->n;
  if (!status && step < R.step_end && (N_in < 0 || N_in > ld || (N_in + G - 1) / G > capc)) {
    // a start population whose even split does not fit the blocks' buffers (more
    // than the 1.5 n0 the population guard allows): refused, nothing is moved
    status = GBDMC_ST_OVERFLOW;
    if (c == 0 && threadIdx.x == 0) {
      ctrl->status = GBDMC_ST_OVERFLOW;
      ctrl->err_step = (int)step;
    }
  }
  if (threadIdx.x == 0) {
    const long long N = N_in < 0 ? 0 : (N_in > ld ? ld : N_in);
    s_N = N;
    s_base = N * c / G;
    s_nc = N * (c + 1) / G - s_base;
    s_vref = ctrl->vref;
  }
  __syncthreads();
  if (status || step >= R.step_end) {
    // no step to run: the walkers pass through, so a queue of launches always
    // leaves the current walkers in the last launch's output
    const int64_t N = s_N;
    for (int64_t g = (int64_t)c * kRunTPB + threadIdx.x; g < N; g += (int64_t)G * kRunTPB) {
#pragma unroll
      for (int k = 0; k < 3 * A; ++k) out.x[k * ld + g] = in.x[k * ld + g];
      out.v[g] = in.v[g];
      if (track) out.who[g] = in.who[g];
    }
  } else {
    int rd = 0;          // the buffer holding the CTA's run
    bool gather = false;  // its walker i is slot src[i] (the copies of the last step) or slot i
    unsigned nbar = 0;    // grid barriers passed: every CTA takes the same ones (the same decisions)
    // the CTA's even share of the compact input
    for (int i = threadIdx.x; i < s_nc; i += kRunTPB) {
      const int64_t g = s_base + i;
      const int j = (int)GBDMC_BC(i, 0, capc, kBcRunShared);
#pragma unroll
      for (int k = 0; k < 3 * A; ++k) xsb[k * capc + j] = in.x[k * ld + g];
      whob[j] = track ? in.who[g] : 0;
    }
    for (unsigned t = 0;; ++t, ++step) {
      const long long base = s_base, nc = s_nc, N = s_N;
      const double vref = s_vref;
      // the moved walkers go to the other buffer (in place with one buffer, where
      // every step starts from an even share, gather false)
      const int wr = R.dbuf ? rd ^ 1 : rd;
      const double* xr = xsb + (size_t)rd * 3 * A * capc;
      double* xs = xsb + (size_t)wr * 3 * A * capc;
      const int* whor = whob + (size_t)rd * capc;
      int* whos = whob + (size_t)wr * capc;
      // 1. move, potential, weight, count
      int csum = 0, flag = 0;
      long long births = 0, deaths = 0;
      double s0 = 0.0;
      RunStats st = {0.0, INFINITY, -INFINITY, 0.0};
      for (int i = threadIdx.x; i < nc; i += kRunTPB) {
        double x[3 * A], z[3 * A], g[3 * A];
        const int j = gather ? (int)GBDMC_BC(src[i], 0, capc, kBcRunShared) : i;
        Rng rng(S.seed, (uint64_t)step, (uint64_t)(base + i), S.replica_id);
        gen_normals<NM, 3 * A>(rng, z);
#pragma unroll
        for (int k = 0; k < 3 * A; ++k) {
          x[k] = __dadd_rn(xr[k * capc + j], __dmul_rn(S.sigma[k / 3], z[k]));
          xs[k * capc + i] = x[k];
        }
        if (track) whos[i] = whor[j];
        const double v = pes<PK, A, false>(x, S.pes, g);
        vs[i] = v;
        if (STATS) {
          st.s1 += v;
          st.vmin = fmin(st.vmin, v);
          st.vmax = fmax(st.vmax, v);
        }
        const int cn = branch_count(v, vref, S.dt, rng.uniform53(), w_hi, flag, births, deaths);
        cnt[i] = cn;
        csum += cn;
        s0 += cn == 1 ? v : (double)cn * v;
      }
      int dsum = (int)deaths;
      unsigned fl = (unsigned)flag;
      run_block_sums<STATS>(csum, dsum, fl, s0, st);
      const int par = t & 1;
      if (threadIdx.x == 0) {
        RunPart q;
        q.c = csum;
        q.df = (unsigned)dsum | (fl << 24);
        q.s0 = s0;
        R.part[par * G + c] = q;
        if (STATS) R.stat[par * G + c] = st;
        run_arrive(R.sync);
      }
      // while the others arrive: the exclusive scan of the block's counts and the
      // gather index of its copies (copy r of walker i is the block's next walker
      // cnt[i] + r, read from slot i of this step's buffer), used if the step keeps
      // its copies in the block
      const int tot = run_scan(cnt, (int)nc);
      if (R.dbuf) {
        for (int i = threadIdx.x; i < nc; i += kRunTPB) {
          const int c0 = (i + 1 < nc ? cnt[i + 1] : tot) - cnt[i];
          const int j0 = cnt[i];
          for (int r = 0; r < c0; ++r) src[GBDMC_BC(j0 + r, 0, capc, kBcRunShared)] = i;
        }
      }
      // 2. every CTA's partial
      if (!run_wait(R.sync, (unsigned)G * ++nbar)) {
        if (threadIdx.x == 0) {
          atomicOr(&ctrl->status, GBDMC_ST_TIMEOUT);
          ctrl->err_step = (int)step;
        }
        break;
      }
      // 3. the same reduction in every CTA, in warp 0: lane l takes CTAs l, l + 32, ...
      if (threadIdx.x < 32) {
        const unsigned full = 0xffffffffu;
        unsigned nn = 0, below = 0;
        int nd = 0, cmax = 0;
        unsigned f = 0;
        double q0 = 0.0;
        RunStats qs = {0.0, INFINITY, -INFINITY, 0.0};
        // all of the lane's partials are loaded before any is used: one L2 round
        // trip (predicated: every block reads every partial once, so that no L2
        // line is hit by more requests than there are blocks)
        int4 rp[kRunMaxCTA / 32];
        const int4* pp = reinterpret_cast<const int4*>(R.part + par * G);
#pragma unroll
        for (int k = 0; k < kRunMaxCTA / 32; ++k) {
          const int g = lane + 32 * k;
          rp[k] = g < G ? __ldcg(pp + g) : make_int4(0, 0, 0, 0);
        }
#pragma unroll
        for (int k = 0; k < kRunMaxCTA / 32; ++k) {
          const int g = lane + 32 * k;
          const int4 r = rp[k];  // zeros past G: they add nothing
          const int rc = r.x;
          nn += rc;
          nd += (int)((unsigned)r.y & 0xFFFFFFu);
          f |= (unsigned)r.y >> 24;
          if (g < G) q0 += __hiloint2double(r.w, r.z);  // the same additions in every CTA
          if (g < c) below += rc;
          cmax = rc > cmax ? rc : cmax;
          if (STATS && g < G) {
            const double2 a = __ldcg(reinterpret_cast<const double2*>(R.stat + par * G + g));
            const double2 b = __ldcg(reinterpret_cast<const double2*>(R.stat + par * G + g) + 1);
            qs.s1 += a.x;
            qs.vmin = fmin(qs.vmin, a.y);
            qs.vmax = fmax(qs.vmax, b.x);
          }
        }
        if (STATS) {
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) qs.s1 += __shfl_xor_sync(full, qs.s1, o);
          qs.vmin = dkey_inv(warp_min_key(dkey(qs.vmin)));
          qs.vmax = dkey_inv(warp_max_key(dkey(qs.vmax)));
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
        const double num = lane == 0 ? q0 : (lane == 1 ? (double)(Nn - N0) : qs.s1);
        const double den = lane == 0 ? (double)Nn : (lane == 1 ? n0 : (double)N);
        const double qq = num / den;
        const double vbar = __shfl_sync(full, qq, 0), corr = __shfl_sync(full, qq, 1);
        const double vmean = __shfl_sync(full, qq, 2);
        if (lane == 0) {
          int st2 = (int)f;
          if (!st2) {
            if ((double)Nn < n0 - n0 * 0.5) st2 |= GBDMC_ST_POP_LOW;
            if ((double)Nn > n0 + n0 * 0.5) st2 |= GBDMC_ST_POP_HIGH;
            if (Nn > ld) st2 |= GBDMC_ST_OVERFLOW;
          }
          const double vr = vbar - S.alpha * corr;
          if (c == 0 && step < S.hist.len) {
            const int64_t h = step;
            if (STATS) {
              if (S.hist.vmin) S.hist.vmin[h] = qs.vmin;
              if (S.hist.vmax) S.hist.vmax[h] = qs.vmax;
              if (S.hist.vmean) S.hist.vmean[h] = vmean;
            }
            if (!st2) {
              if (S.hist.vref) S.hist.vref[h] = vr;
              if (S.hist.pop) S.hist.pop[h] = (double)Nn;
              if (S.hist.births) S.hist.births[h] = (int)(Nn - (N - nd));  // sum of max(c - 1, 0)
              if (S.hist.deaths) S.hist.deaths[h] = nd;
            }
          }
          const long long even = huge ? (long long)INT32_MAX : (long long)((nn + (unsigned)G - 1u) / (unsigned)G);
          const int stop = st2 ? 2 : ((step + 1 >= R.step_end || (int)t + 1 >= R.kmax || even > capc) ? 1 : 0);
          s_stop = stop;
          // the largest CTA's copies against the warps of an even split plus one: a
          // warp more costs the largest block ~4% of its move (the FP64 work is per
          // walker), an even split through the output ~15% of a step
          const long long lim = ((even + 31) / 32) * 32 + 32;
          s_even = !R.dbuf || (long long)cmax > (lim < capc ? lim : (long long)capc);
          if (c == 0) {
            if (st2) {  // as a failed per-step call leaves it: moved walkers, N, vref and step of the step
              ctrl->n = N;
              ctrl->vref = vref;
              ctrl->step = step;
              ctrl->status = st2;
              ctrl->err_step = (int)step;
            } else if (stop == 1) {
              ctrl->n_prev = N;
              ctrl->n = Nn;
              ctrl->vref = vr;
              ctrl->step = step + 1;
            }
          }
          s_nnew = below;  // the new logical base of this CTA's copies: the earlier CTAs' copies
          s_vref = vr;
          s_N = Nn;
        }
      }
      __syncthreads();
      const int stop = s_stop;
      if (stop == 2) {  // the moved, unbranched walkers, compact in logical order
        for (int i = threadIdx.x; i < nc; i += kRunTPB) {
          const int64_t g = base + i;
#pragma unroll
          for (int k = 0; k < 3 * A; ++k) out.x[k * ld + g] = xs[k * capc + i];
          out.v[g] = vs[i];
          if (track) out.who[g] = whos[i];
        }
        break;
      }
      // 4. branch: the CTA's copies in np.repeat order
      const long long nb = s_nnew;
      if (stop || s_even) {
        // into the output at their logical positions: the whole population compact in logical order
        for (int i = threadIdx.x; i < nc; i += kRunTPB) {
          const int c0 = (i + 1 < nc ? cnt[i + 1] : tot) - cnt[i];
          const int64_t g0 = nb + cnt[i];
          for (int r = 0; r < c0; ++r) {
            const int64_t go = GBDMC_BC(g0 + r, 0, ld, kBcRunOut);
#pragma unroll
            for (int k = 0; k < 3 * A; ++k) out.x[k * ld + go] = xs[k * capc + i];
            out.v[go] = vs[i];
            if (track) out.who[go] = whos[i];
          }
        }
        if (stop) break;
        // every CTA's copies written; each CTA takes its even share of the new
        // population back into shared memory (read past L1: other SMs wrote it)
        if (!run_barrier(R.sync, (unsigned)G * ++nbar)) {
          if (threadIdx.x == 0) {
            atomicOr(&ctrl->status, GBDMC_ST_TIMEOUT);
            ctrl->err_step = (int)step;
          }
          break;
        }
        const long long Nn = s_N, nbase = Nn * c / G, nnc = Nn * (c + 1) / G - nbase;
        const int ld_buf = R.dbuf ? wr ^ 1 : wr;  // the moved walkers are in the output now
        double* xl = xsb + (size_t)ld_buf * 3 * A * capc;
        int* wl = whob + (size_t)ld_buf * capc;
        for (int i = threadIdx.x; i < nnc; i += kRunTPB) {
          const int64_t g = nbase + i;
          const int j = (int)GBDMC_BC(i, 0, capc, kBcRunShared);
#pragma unroll
          for (int k = 0; k < 3 * A; ++k) xl[k * capc + j] = __ldcg(out.x + k * ld + g);
          wl[j] = track ? __ldcg(out.who + g) : 0;
        }
        rd = ld_buf;
        gather = false;
        if (threadIdx.x == 0) {
          s_base = nbase;
          s_nc = nnc;
        }
      } else {
        // the CTA's next run is its copies (their gather index is written), at logical base nb
        rd = wr;
        gather = true;
        if (threadIdx.x == 0) {
          s_base = nb;
          s_nc = tot;
        }
      }
      __syncthreads();
    }
  }
  // the last CTA out resets the barrier words for the next launch
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(&R.sync[1], 1u) == (unsigned)G - 1) {
      R.sync[0] = 0;
      R.sync[1] = 0;
    }
  }
}

// ------------------------------------------------------------ host side
static size_t run_smem_bytes(int A, int capc, int nbuf) {
  return (size_t)capc * (nbuf * (3 * A * sizeof(double) + sizeof(int)) + sizeof(double) + 2 * sizeof(int));
}

struct RunShape {
  int grid, capc, dbuf;
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
// CTA per SM (and kRunMaxCTA); each CTA's buffer holds its even share of the
// largest population the guard allows (1.5 n0) with a margin.  Two buffers
// per CTA (the copies of a step stay in shared memory) when they fit, else one
// (every step splits the population evenly through the output).
static int run_shape(const gbdmc_sim_t& S, RunShape& sh) {
  const int A = S.natoms;
  int g = (int)((S.n0 + 95) / 96);
  const int lim = num_sms() < kRunMaxCTA ? num_sms() : kRunMaxCTA;
  g = g < 1 ? 1 : (g > lim ? lim : g);
  const int64_t capc = ((S.n0 * 3 / 2 + 1 + g - 1) / g + 64 + 31) / 32 * 32;
  const size_t smax = 200 * 1024;
  if (capc > (1 << 20) || run_smem_bytes(A, (int)capc, 1) > smax) {
    set_error("gbdmc_sim_run: %lld walkers per block buffer do not fit shared memory (%zu bytes); use "
              "gbdmc_sim_step", (long long)capc, run_smem_bytes(A, (int)(capc > (1 << 20) ? 1 << 20 : capc), 1));
    return GBDMC_ERR_CAPACITY;
  }
  sh.grid = g;
  sh.capc = (int)capc;
  sh.dbuf = run_smem_bytes(A, (int)capc, 2) <= smax ? 1 : 0;
  sh.smem = run_smem_bytes(A, (int)capc, sh.dbuf ? 2 : 1);
  return GBDMC_OK;
}

GBDMC_BOUNDS_READER(bounds_read_run)

}  // namespace gbdmc

using namespace gbdmc;

extern "C" size_t gbdmc_sim_run_scratch_bytes(void) {
  return align256(sizeof(RunPart) * 2 * kRunMaxCTA) + align256(sizeof(RunStats) * 2 * kRunMaxCTA) +
         align256(2 * sizeof(unsigned));
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
  R.dbuf = sh.dbuf;
  R.part = (RunPart*)b;
  R.stat = (RunStats*)(b + align256(sizeof(RunPart) * 2 * kRunMaxCTA));
  R.sync = (unsigned*)(b + align256(sizeof(RunPart) * 2 * kRunMaxCTA) + align256(sizeof(RunStats) * 2 * kRunMaxCTA));
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
