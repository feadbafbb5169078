// Many plain-DMC steps (discrete weighting, Philox deviates) in one launch:
// the loop of DMC_Sim.propagate (pyvibdmc.py:710-876) between two events.
//
// The walkers of a step live in shared memory.  CTA c of a cooperative grid
// of G CTAs holds the run [c*N/G, (c+1)*N/G) of the population in its logical
// (np.repeat) order.  One step:
//   1. every walker of the CTA moves (x + fl(sigma z) from Philox, keyed by
//      its logical index base_c + i as in k_move), its potential, weight and
//      count (pyvibdmc.py:540-547, :392-403); the CTA's partial (sum c,
//      sum cV, births, deaths, guards; sum V / min / max when logging) goes
//      to global memory;
//   2. a grid barrier (bounded wait, GBDMC_ST_TIMEOUT on expiry);
//   3. every CTA reduces the G partials in the same fixed order, so all
//      of them hold the same N', vref' (calc_vref, :651-661) and guards, and
//      its new base is the sum of the earlier CTAs' counts;
//   4. every CTA writes its walkers' copies (np.repeat order) to the output
//      at their logical positions, so the output holds the branched
//      population compact in logical order;
//   5. a second grid barrier, and every CTA loads its even share of the new
//      population back into shared memory (the shares differ by at most one
//      walker, so no CTA's phase 1 runs longer than another's: without this
//      rebalancing the runs of the CTAs that branch more grow step by step
//      and the barrier waits for the largest).
// After the last step of the launch the output is the result.  A step whose
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
constexpr int kRunMaxCTA = 2 * kRunTPB;  // the partial reduction takes two CTAs per thread
constexpr unsigned kRunSpinLimit = 1u << 22;

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Grid barrier over a monotonic arrival counter: returns false if the wait ran
// out (the caller stops; the other CTAs' next waits run out as well).
__device__ __forceinline__ bool run_barrier(unsigned* arrive, unsigned target) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(arrive, 1u);
    int ok = 1;
    unsigned it = 0;
    while (ld_acquire(arrive) < target) {
      if (++it > kRunSpinLimit) {
        ok = 0;
        break;
      }
      __nanosleep(64);
    }
    __threadfence();
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
  Partial* part;     // [2][G]
  unsigned* sync;    // [0] arrivals, [1] exits
};

template <int PK, int A, int NM, bool STATS>
__global__ void __launch_bounds__(kRunTPB) k_run(const __grid_constant__ gbdmc_sim_t S, const gbdmc_walkers_t in,
                                                 gbdmc_walkers_t out, gbdmc_ctrl_t* ctrl, const RunArgs R) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int capc = R.capc, G = gridDim.x, c = blockIdx.x;
  double* xs = reinterpret_cast<double*>(smem);  // [3A][capc]
  double* vs = xs + 3 * A * capc;                // [capc]
  int* whos = reinterpret_cast<int*>(vs + capc);  // [capc]
  int* cnt = whos + capc;                         // [capc]
  __shared__ long long s_base, s_nc, s_nnew, s_N;
  __shared__ double s_vref;
  __shared__ int s_stop;  // 0 go on, 1 branch to the output and end, 2 guards tripped
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
    // the CTA's even share of the compact input
    for (int i = threadIdx.x; i < s_nc; i += kRunTPB) {
      const int64_t g = s_base + i;
#pragma unroll
      for (int k = 0; k < 3 * A; ++k) xs[k * capc + i] = in.x[k * ld + g];
      whos[i] = track ? in.who[g] : 0;
    }
    for (unsigned t = 0;; ++t, ++step) {
      const long long base = s_base, nc = s_nc, N = s_N;
      const double vref = s_vref;
      // 1. move, potential, weight, count
      Partial p = partial_zero();
      int flag = 0;
      for (int i = threadIdx.x; i < nc; i += kRunTPB) {
        double x[3 * A], z[3 * A], g[3 * A];
        Rng rng(S.seed, (uint64_t)step, (uint64_t)(base + i), S.replica_id);
        gen_normals<NM, 3 * A>(rng, z);
#pragma unroll
        for (int k = 0; k < 3 * A; ++k) {
          x[k] = __dadd_rn(xs[k * capc + i], __dmul_rn(S.sigma[k / 3], z[k]));
          xs[k * capc + i] = x[k];
        }
        const double v = pes<PK, A, false>(x, S.pes, g);
        vs[i] = v;
        if (STATS) {
          p.s1 += v;
          p.vmin = fmin(p.vmin, v);
          p.vmax = fmax(p.vmax, v);
        }
        const int cn = branch_count(v, vref, S.dt, rng.uniform53(), w_hi, flag, p.births, p.deaths);
        cnt[i] = cn;
        p.c += cn;
        p.s0 += cn == 1 ? v : (double)cn * v;
      }
      p.aux = __syncthreads_or(flag & GBDMC_ST_NONFINITE_WEIGHT) ? GBDMC_ST_NONFINITE_WEIGHT : 0;
      p.aux |= __syncthreads_or(flag & GBDMC_ST_HUGE_WEIGHT) ? GBDMC_ST_HUGE_WEIGHT : 0;
      const long long aux = p.aux;
      p = block_reduce_partial<STATS>(p);
      const int par = t & 1;
      if (threadIdx.x == 0) {
        p.aux = aux;
        R.part[par * G + c] = p;
      }
      // 2. every CTA's partial
      if (!run_barrier(R.sync, (unsigned)G * (2 * t + 1))) {
        if (threadIdx.x == 0) {
          atomicOr(&ctrl->status, GBDMC_ST_TIMEOUT);
          ctrl->err_step = (int)step;
        }
        break;
      }
      // 3. the same reduction in every CTA: thread k takes CTAs k and k + kRunTPB
      Partial q = partial_zero();
      long long below = 0, fl = 0;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int g = threadIdx.x + h * kRunTPB;
        if (g < G) {
          const Partial r = load_partial(R.part + par * G + g);
          accumulate(q, r);
          q.aux = 0;
          if (g < c) below += r.c;
          fl |= r.aux;
        }
      }
      q.aux = below;
      q = block_reduce_partial<STATS>(q);  // sums `below` too (aux)
      __shared__ int s_fl[kRunTPB / 32];
      fl = __reduce_or_sync(0xffffffffu, (unsigned)fl);
      if ((threadIdx.x & 31) == 0) s_fl[threadIdx.x >> 5] = (int)fl;
      __syncthreads();
      if (threadIdx.x == 0) {
        int f = 0;
        for (int w = 0; w < kRunTPB / 32; ++w) f |= s_fl[w];
        const long long Nn = q.c;
        int st = f;
        if (!st) {
          if ((double)Nn < n0 - n0 * 0.5) st |= GBDMC_ST_POP_LOW;
          if ((double)Nn > n0 + n0 * 0.5) st |= GBDMC_ST_POP_HIGH;
          if (Nn > ld) st |= GBDMC_ST_OVERFLOW;
        }
        const double vr = q.s0 / (double)Nn - S.alpha * ((double)(Nn - N0) / n0);
        if (c == 0 && step < S.hist.len) {
          const int64_t h = step;
          if (STATS) {
            if (S.hist.vmin) S.hist.vmin[h] = q.vmin;
            if (S.hist.vmax) S.hist.vmax[h] = q.vmax;
            if (S.hist.vmean) S.hist.vmean[h] = q.s1 / (double)N;
          }
          if (!st) {
            if (S.hist.vref) S.hist.vref[h] = vr;
            if (S.hist.pop) S.hist.pop[h] = (double)Nn;
            if (S.hist.births) S.hist.births[h] = (int)q.births;
            if (S.hist.deaths) S.hist.deaths[h] = (int)q.deaths;
          }
        }
        s_stop = st ? 2 : ((step + 1 >= R.step_end || (int)t + 1 >= R.kmax || (Nn + G - 1) / G > capc) ? 1 : 0);
        if (c == 0) {
          if (st) {  // as a failed per-step call leaves it: moved walkers, N, vref and step of the step
            ctrl->n = N;
            ctrl->vref = vref;
            ctrl->step = step;
            ctrl->status = st;
            ctrl->err_step = (int)step;
          } else if (s_stop == 1) {
            ctrl->n_prev = N;
            ctrl->n = Nn;
            ctrl->vref = vr;
            ctrl->step = step + 1;
          }
        }
        s_nnew = q.aux;  // the new logical base of this CTA's copies: the earlier CTAs' copies
        s_vref = vr;
        s_N = Nn;
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
      // 4. branch: the CTA's copies into the output at their logical positions
      // (np.repeat order), the whole population compact in logical order
      const int tot = run_scan(cnt, (int)nc);
      const long long nb = s_nnew;
      for (int i = threadIdx.x; i < nc; i += kRunTPB) {
        const int c0 = (i + 1 < nc ? cnt[i + 1] : tot) - cnt[i];
        const int64_t g0 = nb + cnt[i];
        for (int r = 0; r < c0; ++r) {
#pragma unroll
          for (int k = 0; k < 3 * A; ++k) out.x[k * ld + g0 + r] = xs[k * capc + i];
          out.v[g0 + r] = vs[i];
          if (track) out.who[g0 + r] = whos[i];
        }
      }
      if (stop) break;
      // 5. every CTA's copies written; each CTA takes its even share of the new
      // population back into shared memory (read past L1: other SMs wrote it)
      if (!run_barrier(R.sync, (unsigned)G * (2 * t + 2))) {
        if (threadIdx.x == 0) {
          atomicOr(&ctrl->status, GBDMC_ST_TIMEOUT);
          ctrl->err_step = (int)step;
        }
        break;
      }
      const long long Nn = s_N, nbase = Nn * c / G, nnc = Nn * (c + 1) / G - nbase;
      for (int i = threadIdx.x; i < nnc; i += kRunTPB) {
        const int64_t g = nbase + i;
#pragma unroll
        for (int k = 0; k < 3 * A; ++k) xs[k * capc + i] = __ldcg(out.x + k * ld + g);
        whos[i] = track ? __ldcg(out.who + g) : 0;
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        s_base = nbase;
        s_nc = nnc;
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
static size_t run_smem_bytes(int A, int capc) {
  return (size_t)capc * (3 * A * sizeof(double) + sizeof(double) + 2 * sizeof(int));
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

// Grid and per-CTA buffer of a launch: about 96 walkers per CTA, at most one
// CTA per SM (and kRunMaxCTA); each CTA's buffer holds its even share of the
// largest population the guard allows (1.5 n0) with a margin.
static int run_shape(const gbdmc_sim_t& S, RunShape& sh) {
  const int A = S.natoms;
  int g = (int)((S.n0 + 95) / 96);
  const int lim = num_sms() < kRunMaxCTA ? num_sms() : kRunMaxCTA;
  g = g < 1 ? 1 : (g > lim ? lim : g);
  const int64_t capc = ((S.n0 * 3 / 2 + 1 + g - 1) / g + 64 + 31) / 32 * 32;
  const size_t smem = run_smem_bytes(A, (int)capc);
  if (capc > INT32_MAX || smem > 200 * 1024) {
    set_error("gbdmc_sim_run: %lld walkers per block buffer do not fit shared memory (%zu bytes); use "
              "gbdmc_sim_step", (long long)capc, smem);
    return GBDMC_ERR_CAPACITY;
  }
  sh.grid = g;
  sh.capc = (int)capc;
  sh.smem = smem;
  return GBDMC_OK;
}

}  // namespace gbdmc

using namespace gbdmc;

extern "C" size_t gbdmc_sim_run_scratch_bytes(void) {
  return align256(sizeof(Partial) * 2 * kRunMaxCTA) + align256(2 * sizeof(unsigned));
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
  R.kmax = max_steps;
  R.capc = sh.capc;
  R.part = (Partial*)b;
  R.sync = (unsigned*)(b + align256(sizeof(Partial) * 2 * kRunMaxCTA));
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
