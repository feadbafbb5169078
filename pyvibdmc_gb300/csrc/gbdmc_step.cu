// The DMC walker step on the GPU.
//
// Discrete weighting, plain DMC (2 launches per step):
//   k_move_count  : x += sigma*z (bit-exact x + fl(sigma*z)), V = PES(x),
//                   w = exp(-(V-vref) dt), c = floor(w) + [u < w - floor(w)],
//                   per-block partials; the last block to finish scans the
//                   block counts into prefix[], computes N', vref' and the
//                   population guards (pyvibdmc.py:380-431, :651-661).
//   k_scatter     : each walker writes its c copies at prefix + local scan
//                   into the other buffer (np.repeat(arange(N), c) order).
// Importance sampling inserts k_is_move (drift-diffusion proposal, trial psi
// adjoint at the proposal, Metropolis, accept, V + local KE; pyvibdmc.py:549-612,
// :807-809) before a k_count pass that uses dt_eff = dt * accepted/N.
// Continuous weighting replaces count/scatter by the single-CTA
// k_cont_branch (sequential argmax cloning, pyvibdmc.py:340-356, :432-454).
#include "gbdmc_device.cuh"
#include "gbdmc_internal.cuh"

namespace gbdmc {

__device__ __forceinline__ Partial partial_zero() {
  Partial p;
  p.c = p.births = p.deaths = p.aux = 0;
  p.s0 = p.s1 = 0.0;
  p.vmin = CUDART_INF;
  p.vmax = -CUDART_INF;
  return p;
}

// Deterministic block reduction of a Partial (fixed shuffle/shared tree).
__device__ Partial block_reduce_partial(Partial p) {
  __shared__ Partial sh[kTPB / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  p.c = warp_sum(p.c);
  p.births = warp_sum(p.births);
  p.deaths = warp_sum(p.deaths);
  p.aux = warp_sum(p.aux);
  p.s0 = warp_sum(p.s0);
  p.s1 = warp_sum(p.s1);
  p.vmin = warp_min(p.vmin);
  p.vmax = warp_max(p.vmax);
  if (lane == 0) sh[wid] = p;
  __syncthreads();
  if (wid == 0) {
    p = lane < kTPB / 32 ? sh[lane] : partial_zero();
    p.c = warp_sum(p.c);
    p.births = warp_sum(p.births);
    p.deaths = warp_sum(p.deaths);
    p.aux = warp_sum(p.aux);
    p.s0 = warp_sum(p.s0);
    p.s1 = warp_sum(p.s1);
    p.vmin = warp_min(p.vmin);
    p.vmax = warp_max(p.vmax);
  }
  __syncthreads();
  return p;  // valid in thread 0
}

__device__ __forceinline__ Partial load_partial(const Partial* p) {
  Partial r;
  const long long* q = (const long long*)p;
  long long* o = (long long*)&r;
#pragma unroll
  for (int k = 0; k < 8; ++k) o[k] = __ldcg(q + k);
  return r;
}

__device__ __forceinline__ void accumulate(Partial& a, const Partial& b) {
  a.c += b.c;
  a.births += b.births;
  a.deaths += b.deaths;
  a.aux += b.aux;
  a.s0 += b.s0;
  a.s1 += b.s1;
  a.vmin = fmin(a.vmin, b.vmin);
  a.vmax = fmax(a.vmax, b.vmax);
}

// Elects the last block of the grid to finish (threadFenceReduction pattern).
// All blocks call it after writing their partial; returns true in every thread
// of the last block.
__device__ __forceinline__ bool last_block(gbdmc_ctrl_t* ctrl) {
  __shared__ bool am_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned t = atomicAdd(&ctrl->ticket, 1u);
    am_last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (am_last) __threadfence();
  return am_last;
}

// Last block: fixed-order reduction of all partials (and, when prefix != NULL,
// an exclusive scan of the block counts into prefix[]).  Result in thread 0.
__device__ Partial reduce_partials(const Partial* part, int G, long long* prefix) {
  const int per = (G + kTPB - 1) / kTPB;
  const int beg = min(G, threadIdx.x * per), end = min(G, beg + per);
  Partial acc = partial_zero();
  for (int j = beg; j < end; ++j) accumulate(acc, load_partial(part + j));
  if (prefix) {
    // exclusive scan of per-thread count sums across the block
    __shared__ long long wsum[kTPB / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    long long v = acc.c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const long long t = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= o) v += t;
    }
    if (lane == 31) wsum[wid] = v;
    __syncthreads();
    long long base = 0;
    for (int w = 0; w < wid; ++w) base += wsum[w];
    long long run = base + v - acc.c;  // exclusive prefix of this thread
    for (int j = beg; j < end; ++j) {
      prefix[j] = run;
      run += __ldcg(&part[j].c);
    }
    __syncthreads();
  }
  return block_reduce_partial(acc);
}

// Discrete weight and branch count of one walker (pyvibdmc.py:392-403).
__device__ __forceinline__ int branch_count(double v, double vref, double dt, double u, double w_hi, int& flag,
                                            long long& births, long long& deaths) {
  const double w = exp(__dmul_rn(-__dsub_rn(v, vref), dt));
  if (!isfinite(w)) {
    flag |= GBDMC_ST_NONFINITE_WEIGHT;
    return 0;
  }
  if (w > w_hi) {
    flag |= GBDMC_ST_HUGE_WEIGHT;
    return 0;
  }
  const double fl = floor(w);
  const int c = (int)fl + (u < __dsub_rn(w, fl) ? 1 : 0);
  births += c > 1 ? c - 1 : 0;
  deaths += c == 0 ? 1 : 0;
  return c;
}

// Finalisation of a discrete branching pass (thread 0 of the last block).
__device__ void finalize_discrete(const gbdmc_sim_t& S, gbdmc_ctrl_t* ctrl, const Partial& tot) {
  const long long n = ctrl->n;
  const long long step = ctrl->step;
  const long long nn = tot.c;
  int st = ctrl->status | *(volatile int*)&ctrl->flags;
  ctrl->flags = 0;
  if (!st) {
    const double n0 = (double)S.n0;
    if ((double)nn < n0 - n0 * 0.5) st |= GBDMC_ST_POP_LOW;
    if ((double)nn > n0 + n0 * 0.5) st |= GBDMC_ST_POP_HIGH;
    if (nn > S.ld) st |= GBDMC_ST_OVERFLOW;
  }
  if (st) {
    ctrl->status = st;
    ctrl->err_step = (int)step;
  } else {
    const double vbar = tot.s0 / (double)nn;
    const double corr = (double)(nn - S.n0) / (double)S.n0;
    const double vref = vbar - S.alpha * corr;
    if (step < S.hist.len) {
      if (S.hist.vref) S.hist.vref[step] = vref;
      if (S.hist.pop) S.hist.pop[step] = (double)nn;
      if (S.hist.births) S.hist.births[step] = (int)tot.births;
      if (S.hist.deaths) S.hist.deaths[step] = (int)tot.deaths;
    }
    ctrl->n_prev = n;
    ctrl->n = nn;
    ctrl->vref = vref;
    ctrl->step = step + 1;
  }
  ctrl->ticket = 0;
}

__device__ __forceinline__ void record_vstats(const gbdmc_sim_t& S, long long step, long long n, const Partial& t) {
  if (step < S.hist.len) {
    if (S.hist.vmin) S.hist.vmin[step] = t.vmin;
    if (S.hist.vmax) S.hist.vmax[step] = t.vmax;
    if (S.hist.vmean) S.hist.vmean[step] = t.s1 / (double)n;
  }
}

// ------------------------------------------------------------------ init
// Step 0: V (+ local KE with a trial psi) and the first vref (pyvibdmc.py:760-769).
template <int PK, int A, int TK>
__global__ void __launch_bounds__(kTPB) k_init(const gbdmc_sim_t S, gbdmc_walkers_t W, gbdmc_ctrl_t* ctrl,
                                                Partial* part) {
  const long long n = ctrl->n;
  const int64_t ld = S.ld;
  const int64_t i = (int64_t)blockIdx.x * kTPB + threadIdx.x;
  Partial p = partial_zero();
  if (i < n) {
    double x[3 * A], g[3 * A];
#pragma unroll
    for (int k = 0; k < 3 * A; ++k) x[k] = W.x[k * ld + i];
    double v = pes<PK, A, false>(x, S.pes, g);
    if constexpr (TK != GBDMC_TRIAL_NONE) {
      double d1[3 * A], d2[3 * A];
      const double psi = trial<TK, A>(x, S.trial, d1, d2);
      double ke = 0.0;
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        double s = 0.0;
#pragma unroll
        for (int a = 0; a < A; ++a) s = s + S.inv_mass[a] * d2[3 * a + d];
        ke = ke + s;
      }
      ke = -0.5 * ke;
#pragma unroll
      for (int k = 0; k < 3 * A; ++k) W.f[k * ld + i] = d1[k];
      W.psi[i] = psi;
      W.ke[i] = ke;
      v = v + ke;
    }
    W.v[i] = v;
    if (S.weighting == GBDMC_CONTINUOUS) {
      const double w = W.w[i];
      p.s0 = v * w;
      p.s1 = w;
    } else {
      p.s0 = v;
      p.s1 = 1.0;
    }
    p.c = 1;
  }
  p = block_reduce_partial(p);
  if (threadIdx.x == 0) part[blockIdx.x] = p;
  if (last_block(ctrl)) {
    const Partial t = reduce_partials(part, gridDim.x, nullptr);
    if (threadIdx.x == 0) {
      double vref;
      if (S.weighting == GBDMC_CONTINUOUS)
        vref = t.s0 / t.s1 - S.alpha * ((t.s1 - (double)S.n0) / (double)S.n0);
      else
        vref = t.s0 / (double)n - S.alpha * ((double)(n - S.n0) / (double)S.n0);
      ctrl->vref = vref;
      ctrl->ticket = 0;
    }
  }
}

// --------------------------------------------------------- plain move
// COUNT: fused discrete weights/counts (+ last-block scan); otherwise the
// move and potential only (continuous weighting).
template <int PK, int A, int NM, bool COUNT>
__global__ void __launch_bounds__(kTPB) k_move(const gbdmc_sim_t S, gbdmc_walkers_t W, gbdmc_ctrl_t* ctrl,
                                                Partial* part, long long* prefix, int* counts,
                                                const gbdmc_noise_t nz) {
  if (*(volatile int*)&ctrl->status) return;
  const long long n = ctrl->n;
  const long long step = ctrl->step;
  const double vref = ctrl->vref;
  const int64_t ld = S.ld;
  const int64_t i = (int64_t)blockIdx.x * kTPB + threadIdx.x;
  Partial p = partial_zero();
  int flag = 0;
  if (i < n) {
    double x[3 * A], z[3 * A], g[3 * A];
#pragma unroll
    for (int k = 0; k < 3 * A; ++k) x[k] = W.x[k * ld + i];
    Rng rng(S.seed, (uint64_t)step, (uint64_t)i);
    if constexpr (NM == GBDMC_NOISE_INJECTED) {
#pragma unroll
      for (int k = 0; k < 3 * A; ++k) z[k] = nz.normal[k * nz.ld_noise + i];
    } else {
      gen_normals<NM, 3 * A>(rng, z);
    }
    // x + (0 + sigma*z): the reference adds the drawn displacement (pyvibdmc.py:544-547)
#pragma unroll
    for (int k = 0; k < 3 * A; ++k) {
      x[k] = __dadd_rn(x[k], __dmul_rn(S.sigma[k / 3], z[k]));
      W.x[k * ld + i] = x[k];
    }
    const double v = pes<PK, A, false>(x, S.pes, g);
    W.v[i] = v;
    p.s1 = v;
    p.vmin = v;
    p.vmax = v;
    if constexpr (COUNT) {
      double u;
      if constexpr (NM == GBDMC_NOISE_INJECTED)
        u = nz.u_branch[i];
      else
        u = rng.uniform53();
      const double w_hi = ((double)S.n0 + (double)S.n0 * 0.5) + 1.0;
      const int c = branch_count(v, vref, S.dt, u, w_hi, flag, p.births, p.deaths);
      counts[i] = c;
      p.c = c;
      p.s0 = (double)c * v;
    }
  }
  if (COUNT && __syncthreads_or(flag)) {
    if (threadIdx.x == 0) atomicOr(&ctrl->flags, flag);
  }
  p = block_reduce_partial(p);
  if (threadIdx.x == 0) part[blockIdx.x] = p;
  if (last_block(ctrl)) {
    const Partial t = reduce_partials(part, gridDim.x, COUNT ? prefix : nullptr);
    if (threadIdx.x == 0) {
      record_vstats(S, step, n, t);
      if constexpr (COUNT)
        finalize_discrete(S, ctrl, t);
      else
        ctrl->ticket = 0;
    }
  }
}

// ----------------------------------------------- importance-sampled move
// pyvibdmc.py:549-612 with ImpSamp.metropolis (imp_samp.py:28-47) and
// local_kin (imp_samp.py:49-53).  The Green's-function ratio prod_k
// exp(-a_k^2/2s^2)/exp(-b_k^2/2s^2) is evaluated as one exp of the summed
// exponents.
template <int PK, int A, int TK, int NM>
__global__ void __launch_bounds__(kTPB) k_is_move(const gbdmc_sim_t S, gbdmc_walkers_t W, gbdmc_ctrl_t* ctrl,
                                                   Partial* part, const gbdmc_noise_t nz) {
  if (*(volatile int*)&ctrl->status) return;
  const long long n = ctrl->n;
  const long long step = ctrl->step;
  const int64_t ld = S.ld;
  const double dt = S.dt;
  const int64_t i = (int64_t)blockIdx.x * kTPB + threadIdx.x;
  Partial p = partial_zero();
  if (i < n) {
    double x[3 * A], y[3 * A], fx[3 * A], fy[3 * A], sdy[3 * A], g[3 * A];
#pragma unroll
    for (int k = 0; k < 3 * A; ++k) {
      x[k] = W.x[k * ld + i];
      fx[k] = W.f[k * ld + i];
    }
    const double psi_x = W.psi[i];
    Rng rng(S.seed, (uint64_t)step, (uint64_t)i);
    double z[3 * A];
    if constexpr (NM == GBDMC_NOISE_INJECTED) {
#pragma unroll
      for (int k = 0; k < 3 * A; ++k) z[k] = nz.normal[k * nz.ld_noise + i];
    } else {
      gen_normals<NM, 3 * A>(rng, z);
    }
    // y = (x + disp) + (f_x/m) dt   (pyvibdmc.py:556-576)
#pragma unroll
    for (int k = 0; k < 3 * A; ++k) {
      const double dx = __dmul_rn(S.inv_mass[k / 3], fx[k]);
      y[k] = __dadd_rn(__dadd_rn(x[k], __dmul_rn(S.sigma[k / 3], z[k])), __dmul_rn(dx, dt));
    }
    const double psi_y = trial<TK, A>(y, S.trial, fy, sdy);
    // Metropolis ratio
    double expo = 0.0;
#pragma unroll
    for (int k = 0; k < 3 * A; ++k) {
      const double im = S.inv_mass[k / 3];
      const double s2 = S.sigma[k / 3] * S.sigma[k / 3];
      const double a = x[k] - y[k] - im * fy[k] * dt;
      const double b = y[k] - x[k] - im * fx[k] * dt;
      expo += (b * b - a * a) / (2.0 * s2);
    }
    const double r = psi_y / psi_x;
    double met = exp(expo) * (r * r);
    if (psi_x * psi_y <= 0.0) met = 0.0;
    double u;
    if constexpr (NM == GBDMC_NOISE_INJECTED)
      u = nz.u_accept[i];
    else
      u = rng.uniform53();
    const bool acc = met > u;
    double ke;
    if (acc) {
      double s = 0.0;
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        double t = 0.0;
#pragma unroll
        for (int a = 0; a < A; ++a) t = t + S.inv_mass[a] * sdy[3 * a + d];
        s = s + t;
      }
      ke = -0.5 * s;
#pragma unroll
      for (int k = 0; k < 3 * A; ++k) {
        x[k] = y[k];
        W.x[k * ld + i] = y[k];
        W.f[k * ld + i] = fy[k];
      }
      W.psi[i] = psi_y;
      W.ke[i] = ke;
    } else {
      ke = W.ke[i];
    }
    const double v = pes<PK, A, false>(x, S.pes, g);
    W.v[i] = v + ke;
    p.aux = acc ? 1 : 0;
    p.s1 = v;
    p.vmin = v;
    p.vmax = v;
  }
  p = block_reduce_partial(p);
  if (threadIdx.x == 0) part[blockIdx.x] = p;
  if (last_block(ctrl)) {
    const Partial t = reduce_partials(part, gridDim.x, nullptr);
    if (threadIdx.x == 0) {
      record_vstats(S, step, n, t);
      // dt_factor = accepted / N (pyvibdmc.py:603); effective time (:372-378)
      const double dte = S.dt * ((double)t.aux / (double)n);
      ctrl->dt_eff = dte;
      ctrl->n_acc = t.aux;
      ctrl->eff_ts = (step == 0) ? dte : ctrl->eff_ts + dte;
      if (step < S.hist.len) {
        if (S.hist.rejected) S.hist.rejected[step] = (int)(n - t.aux);
        if (S.hist.eff_ts) S.hist.eff_ts[step] = ctrl->eff_ts;
      }
      ctrl->ticket = 0;
    }
  }
}

// Discrete weights and counts from stored energies with dt_eff (importance sampling).
template <int NM>
__global__ void __launch_bounds__(kTPB) k_count(const gbdmc_sim_t S, gbdmc_walkers_t W, gbdmc_ctrl_t* ctrl,
                                                 Partial* part, long long* prefix, int* counts,
                                                 const gbdmc_noise_t nz) {
  if (*(volatile int*)&ctrl->status) return;
  const long long n = ctrl->n;
  const long long step = ctrl->step;
  const double vref = ctrl->vref;
  const double dt = ctrl->dt_eff;
  const int64_t i = (int64_t)blockIdx.x * kTPB + threadIdx.x;
  Partial p = partial_zero();
  int flag = 0;
  if (i < n) {
    const double v = W.v[i];
    double u;
    if constexpr (NM == GBDMC_NOISE_INJECTED) {
      u = nz.u_branch[i];
    } else {
      Rng rng(S.seed, (uint64_t)step, (uint64_t)i);
      rng.slot = 64;  // stream disjoint from the move's draws
      u = rng.uniform53();
    }
    const double w_hi = ((double)S.n0 + (double)S.n0 * 0.5) + 1.0;
    const int c = branch_count(v, vref, dt, u, w_hi, flag, p.births, p.deaths);
    counts[i] = c;
    p.c = c;
    p.s0 = (double)c * v;
  }
  if (__syncthreads_or(flag)) {
    if (threadIdx.x == 0) atomicOr(&ctrl->flags, flag);
  }
  p = block_reduce_partial(p);
  if (threadIdx.x == 0) part[blockIdx.x] = p;
  if (last_block(ctrl)) {
    const Partial t = reduce_partials(part, gridDim.x, prefix);
    if (threadIdx.x == 0) finalize_discrete(S, ctrl, t);
  }
}

// ---------------------------------------------------------------- scatter
// Walker i writes its counts[i] copies to dst at prefix[block] + (exclusive
// scan of counts inside the block): the order of np.repeat(arange(N), counts).
template <int A, bool IS, bool WHO>
__global__ void __launch_bounds__(kTPB) k_scatter(const gbdmc_sim_t S, const gbdmc_walkers_t src,
                                                   gbdmc_walkers_t dst, const gbdmc_ctrl_t* ctrl,
                                                   const long long* prefix, const int* counts) {
  if (*(volatile const int*)&ctrl->status) return;
  const long long n = ctrl->n_prev;
  const int64_t ld = S.ld;
  const int64_t i = (int64_t)blockIdx.x * kTPB + threadIdx.x;
  const int c = i < n ? counts[i] : 0;
  // block exclusive scan of c
  __shared__ int wsum[kTPB / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int inc = warp_incl_scan(c);
  if (lane == 31) wsum[wid] = inc;
  __syncthreads();
  int base = 0;
#pragma unroll
  for (int w = 0; w < kTPB / 32; ++w) base += (w < wid) ? wsum[w] : 0;
  const long long dest = prefix[blockIdx.x] + base + inc - c;
  if (c == 0) return;
  const long long lim = dest + c <= ld ? c : (ld - dest > 0 ? ld - dest : 0);
#pragma unroll
  for (int k = 0; k < 3 * A; ++k) {
    const double xv = src.x[k * ld + i];
    for (long long r = 0; r < lim; ++r) dst.x[k * ld + dest + r] = xv;
  }
  const double v = src.v[i];
  for (long long r = 0; r < lim; ++r) dst.v[dest + r] = v;
  if constexpr (WHO) {
    const int wh = src.who[i];
    for (long long r = 0; r < lim; ++r) dst.who[dest + r] = wh;
  }
  if constexpr (IS) {
#pragma unroll
    for (int k = 0; k < 3 * A; ++k) {
      const double fv = src.f[k * ld + i];
      for (long long r = 0; r < lim; ++r) dst.f[k * ld + dest + r] = fv;
    }
    const double ps = src.psi[i], ke = src.ke[i];
    for (long long r = 0; r < lim; ++r) {
      dst.psi[dest + r] = ps;
      dst.ke[dest + r] = ke;
    }
  }
}

// ---------------------------------------------------- continuous weights
// One CTA of 1024 threads: w *= exp(-(V-vref) dt); clone the current argmax
// into every walker below the lower threshold, in index order, halving the
// argmax each time (pyvibdmc.py:340-356, :432-438); the optional upper
// threshold branches the k smallest weights (k = #w > upper) in ascending
// index order; then vref from the weighted mean (:659-661).
constexpr int kCTA = 1024;

struct ArgBest {
  double v;
  long long i;
};

// first index of the maximum (MAX) or minimum (!MAX) over w[0..n), skipping flagged entries
template <bool MAX>
__device__ long long block_arg(const double* w, long long n, const unsigned char* skip) {
  __shared__ ArgBest sh[kCTA / 32];
  ArgBest b{MAX ? -CUDART_INF : CUDART_INF, -1};
  for (long long i = threadIdx.x; i < n; i += kCTA) {
    if (skip && skip[i]) continue;
    const double v = w[i];
    if (b.i < 0 || (MAX ? v > b.v : v < b.v)) {
      b.v = v;
      b.i = i;
    }
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double ov = __shfl_down_sync(0xffffffffu, b.v, o);
    const long long oi = __shfl_down_sync(0xffffffffu, b.i, o);
    const bool better = oi >= 0 && (b.i < 0 || (MAX ? ov > b.v : ov < b.v) || (ov == b.v && oi < b.i));
    if (better) {
      b.v = ov;
      b.i = oi;
    }
  }
  if (lane == 0) sh[wid] = b;
  __syncthreads();
  if (wid == 0) {
    b = sh[lane];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double ov = __shfl_down_sync(0xffffffffu, b.v, o);
      const long long oi = __shfl_down_sync(0xffffffffu, b.i, o);
      const bool better = oi >= 0 && (b.i < 0 || (MAX ? ov > b.v : ov < b.v) || (ov == b.v && oi < b.i));
      if (better) {
        b.v = ov;
        b.i = oi;
      }
    }
    if (lane == 0) sh[0] = b;
  }
  __syncthreads();
  const long long r = sh[0].i;
  __syncthreads();
  return r;
}

template <int A, bool IS, bool WHO>
__device__ void clone_walker(const gbdmc_sim_t& S, gbdmc_walkers_t& W, long long from, long long to) {
  const int64_t ld = S.ld;
  const int t = threadIdx.x;
  if (t < 3 * A) {
    W.x[t * ld + to] = W.x[t * ld + from];
    if constexpr (IS) W.f[t * ld + to] = W.f[t * ld + from];
  } else if (t == 3 * A) {
    W.v[to] = W.v[from];
  } else if (t == 3 * A + 1) {
    if constexpr (WHO) W.who[to] = W.who[from];
  } else if (t == 3 * A + 2) {
    if constexpr (IS) {
      W.psi[to] = W.psi[from];
      W.ke[to] = W.ke[from];
    }
  }
}

// ordered list of indices with flag set: list[0..k), returns k
__device__ long long block_compact(const unsigned char* flag, long long n, int* list) {
  __shared__ int wsum[kCTA / 32];
  __shared__ long long total;
  if (threadIdx.x == 0) total = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (long long base = 0; base < n; base += kCTA) {
    const long long i = base + threadIdx.x;
    const int f = (i < n && flag[i]) ? 1 : 0;
    const int inc = warp_incl_scan(f);
    if (lane == 31) wsum[wid] = inc;
    __syncthreads();
    int off = 0;
    for (int w = 0; w < wid; ++w) off += wsum[w];
    if (f) list[total + off + inc - 1] = (int)i;
    __syncthreads();
    if (threadIdx.x == kCTA - 1) total += off + inc;
    __syncthreads();
  }
  return total;
}

template <int A, bool IS, bool WHO>
__global__ void __launch_bounds__(kCTA) k_cont_branch(const gbdmc_sim_t S, gbdmc_walkers_t W, gbdmc_ctrl_t* ctrl,
                                                       int* list, unsigned char* flags) {
  if (*(volatile int*)&ctrl->status) return;
  const long long n = ctrl->n;
  const long long step = ctrl->step;
  const double vref = ctrl->vref;
  const double dt = IS ? ctrl->dt_eff : S.dt;
  __shared__ long long s_nb;
  int bad = 0;
  for (long long i = threadIdx.x; i < n; i += kCTA) {
    const double w = W.w[i] * exp(__dmul_rn(-__dsub_rn(W.v[i], vref), dt));
    W.w[i] = w;
    if (!isfinite(w)) bad = 1;
    flags[i] = (w < S.thresh_lower) ? 1 : 0;
  }
  if (__syncthreads_or(bad)) {
    if (threadIdx.x == 0) {
      ctrl->status |= GBDMC_ST_NONFINITE_WEIGHT;
      ctrl->err_step = (int)step;
    }
    return;
  }
  long long nk = block_compact(flags, n, list);
  long long nb = nk;
  for (long long j = 0; j < nk; ++j) {
    const long long to = list[j];
    const long long m = block_arg<true>(W.w, n, nullptr);
    clone_walker<A, IS, WHO>(S, W, m, to);
    __syncthreads();
    if (threadIdx.x == 0) {
      const double h = W.w[m] / 2.0;
      W.w[m] = h;
      W.w[to] = h;
    }
    __syncthreads();
  }
  if (S.thresh_upper > 0.0) {
    if (threadIdx.x == 0) s_nb = 0;
    __syncthreads();
    long long cnt = 0;
    for (long long i = threadIdx.x; i < n; i += kCTA) {
      cnt += W.w[i] > S.thresh_upper ? 1 : 0;
      flags[i] = 0;
    }
    cnt = warp_sum(cnt);
    if ((threadIdx.x & 31) == 0) atomicAdd((unsigned long long*)&s_nb, (unsigned long long)cnt);
    __syncthreads();
    const long long nup = s_nb;
    // mark the nup smallest weights (ties: lowest index first)
    for (long long j = 0; j < nup; ++j) {
      const long long m = block_arg<false>(W.w, n, flags);
      if (threadIdx.x == 0) flags[m] = 1;
      __syncthreads();
    }
    const long long nk2 = block_compact(flags, n, list);
    for (long long j = 0; j < nk2; ++j) {
      const long long to = list[j];
      const long long m = block_arg<true>(W.w, n, nullptr);
      clone_walker<A, IS, WHO>(S, W, m, to);
      __syncthreads();
      if (threadIdx.x == 0) {
        const double h = W.w[m] / 2.0;
        W.w[m] = h;
        W.w[to] = h;
      }
      __syncthreads();
    }
    nb += nk2;
  }
  // weighted vref and statistics (fixed-order reduction)
  double swv = 0.0, sw = 0.0, wmx = -CUDART_INF, wmn = CUDART_INF;
  for (long long i = threadIdx.x; i < n; i += kCTA) {
    const double w = W.w[i];
    swv += W.v[i] * w;
    sw += w;
    wmx = fmax(wmx, w);
    wmn = fmin(wmn, w);
  }
  __shared__ double r4[4][kCTA / 32];
  swv = warp_sum(swv);
  sw = warp_sum(sw);
  wmx = warp_max(wmx);
  wmn = warp_min(wmn);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) {
    r4[0][wid] = swv;
    r4[1][wid] = sw;
    r4[2][wid] = wmx;
    r4[3][wid] = wmn;
  }
  __syncthreads();
  if (wid == 0) {
    swv = warp_sum(r4[0][lane]);
    sw = warp_sum(r4[1][lane]);
    wmx = warp_max(r4[2][lane]);
    wmn = warp_min(r4[3][lane]);
    if (lane == 0) {
      const double vr = swv / sw - S.alpha * ((sw - (double)S.n0) / (double)S.n0);
      if (step < S.hist.len) {
        if (S.hist.vref) S.hist.vref[step] = vr;
        if (S.hist.pop) S.hist.pop[step] = sw;
        if (S.hist.births) S.hist.births[step] = (int)nb;
      }
      ctrl->vref = vr;
      ctrl->n_prev = n;
      ctrl->step = step + 1;
      // logging extras: max / min weight after branching
      ctrl->reserved[0] = __double_as_longlong(wmx);
      ctrl->reserved[1] = __double_as_longlong(wmn);
    }
  }
}

// -------------------------------------------------------- descendants
__global__ void k_desc(const int32_t* who, const double* w, const int64_t* n_dev, int64_t n_parent, double* desc) {
  const long long n = *n_dev;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int q = who[i];
    if (q >= 0 && q < n_parent) atomicAdd(desc + q, w ? w[i] : 1.0);
  }
}

__global__ void k_iota(int32_t* who, const int64_t* n_dev) {
  const long long n = *n_dev;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    who[i] = (int32_t)i;
}

// ------------------------------------------------------------ dispatch
template <int PK, int A, int TK>
static int run_init(const gbdmc_sim_t& S, const gbdmc_walkers_t& W, gbdmc_ctrl_t* ctrl, const ScratchLayout& L,
                    cudaStream_t s) {
  k_init<PK, A, TK><<<grid_for(S.ld), kTPB, 0, s>>>(S, W, ctrl, L.part);
  return check_launch("gbdmc_sim_init");
}

template <int A, bool IS>
static void launch_scatter(const gbdmc_sim_t& S, const gbdmc_walkers_t& src, const gbdmc_walkers_t& dst,
                           gbdmc_ctrl_t* ctrl, const ScratchLayout& L, cudaStream_t s) {
  const int G = grid_for(S.ld);
  if (S.track_who)
    k_scatter<A, IS, true><<<G, kTPB, 0, s>>>(S, src, dst, ctrl, L.prefix, L.counts);
  else
    k_scatter<A, IS, false><<<G, kTPB, 0, s>>>(S, src, dst, ctrl, L.prefix, L.counts);
}

template <int A, bool IS>
static void launch_cont(const gbdmc_sim_t& S, const gbdmc_walkers_t& W, gbdmc_ctrl_t* ctrl, const ScratchLayout& L,
                        cudaStream_t s) {
  if (S.track_who)
    k_cont_branch<A, IS, true><<<1, kCTA, 0, s>>>(S, W, ctrl, L.list, L.flags);
  else
    k_cont_branch<A, IS, false><<<1, kCTA, 0, s>>>(S, W, ctrl, L.list, L.flags);
}

template <int PK, int A, int TK, int NM>
static int run_step(const gbdmc_sim_t& S, const gbdmc_walkers_t& src, const gbdmc_walkers_t& dst, gbdmc_ctrl_t* ctrl,
                    const ScratchLayout& L, const gbdmc_noise_t& nz, cudaStream_t s) {
  const int G = grid_for(S.ld);
  constexpr bool IS = TK != GBDMC_TRIAL_NONE;
  if constexpr (!IS) {
    if (S.weighting == GBDMC_DISCRETE) {
      const bool prof = g_prof.on && g_prof.count < ProfState::kSlots;
      cudaEvent_t* ev = prof ? g_prof.ev[g_prof.count] : nullptr;
      if (prof) cudaEventRecord(ev[0], s);
      k_move<PK, A, NM, true><<<G, kTPB, 0, s>>>(S, src, ctrl, L.part, L.prefix, L.counts, nz);
      if (prof) cudaEventRecord(ev[1], s);
      launch_scatter<A, false>(S, src, dst, ctrl, L, s);
      if (prof) {
        cudaEventRecord(ev[2], s);
        ++g_prof.count;
      }
    } else {
      k_move<PK, A, NM, false><<<G, kTPB, 0, s>>>(S, src, ctrl, L.part, L.prefix, L.counts, nz);
      launch_cont<A, false>(S, src, ctrl, L, s);
    }
  } else {
    k_is_move<PK, A, TK, NM><<<G, kTPB, 0, s>>>(S, src, ctrl, L.part, nz);
    if (S.weighting == GBDMC_DISCRETE) {
      k_count<NM><<<G, kTPB, 0, s>>>(S, src, ctrl, L.part, L.prefix, L.counts, nz);
      launch_scatter<A, true>(S, src, dst, ctrl, L, s);
    } else {
      launch_cont<A, true>(S, src, ctrl, L, s);
    }
  }
  return check_launch("gbdmc_sim_step");
}

template <int PK, int A, int TK>
static int step_noise(const gbdmc_sim_t& S, const gbdmc_walkers_t& src, const gbdmc_walkers_t& dst,
                      gbdmc_ctrl_t* ctrl, const ScratchLayout& L, const gbdmc_noise_t& nz, cudaStream_t s) {
  switch (S.noise_mode) {
    case GBDMC_NOISE_PHILOX32: return run_step<PK, A, TK, GBDMC_NOISE_PHILOX32>(S, src, dst, ctrl, L, nz, s);
    case GBDMC_NOISE_PHILOX64: return run_step<PK, A, TK, GBDMC_NOISE_PHILOX64>(S, src, dst, ctrl, L, nz, s);
    case GBDMC_NOISE_INJECTED: return run_step<PK, A, TK, GBDMC_NOISE_INJECTED>(S, src, dst, ctrl, L, nz, s);
  }
  set_error("gbdmc_sim_step: unknown noise mode %d", S.noise_mode);
  return GBDMC_ERR_ARG;
}

// Supported (PES, atoms, trial) systems.
template <typename F>
static int dispatch_system(const gbdmc_sim_t& S, const char* what, F&& f) {
  const int PK = S.pes.kind, A = S.natoms, TK = S.trial.kind;
  if (S.pes.natoms != A || (TK != GBDMC_TRIAL_NONE && S.trial.natoms != A)) {
    set_error("%s: natoms mismatch between sim, pes and trial", what);
    return GBDMC_ERR_ARG;
  }
#define GBDMC_SYS(pk, a, tk) \
  if (PK == pk && A == a && TK == tk) return f.template operator()<pk, a, tk>();
  GBDMC_SYS(GBDMC_PES_HO, 1, GBDMC_TRIAL_NONE)
  GBDMC_SYS(GBDMC_PES_HO, 3, GBDMC_TRIAL_NONE)
  GBDMC_SYS(GBDMC_PES_H2O_LM, 3, GBDMC_TRIAL_NONE)
  GBDMC_SYS(GBDMC_PES_DIMER, 6, GBDMC_TRIAL_NONE)
  GBDMC_SYS(GBDMC_PES_HO, 1, GBDMC_TRIAL_HO_GAUSS)
  GBDMC_SYS(GBDMC_PES_HO, 3, GBDMC_TRIAL_HO_GAUSS)
  GBDMC_SYS(GBDMC_PES_H2O_LM, 3, GBDMC_TRIAL_H2O_GAUSS)
#undef GBDMC_SYS
  set_error("%s: unsupported system (pes %d, atoms %d, trial %d)", what, PK, A, TK);
  return GBDMC_ERR_ARG;
}

static int validate(const gbdmc_sim_t* S, const gbdmc_walkers_t* W, const void* ctrl, const void* scratch,
                    const char* what) {
  if (!S || !W || !ctrl || !scratch) {
    set_error("%s: null argument", what);
    return GBDMC_ERR_ARG;
  }
  if (S->natoms < 1 || S->natoms > GBDMC_MAX_ATOMS || S->ld < 1 || S->n0 < 1) {
    set_error("%s: bad sizes (natoms=%d ld=%lld n0=%lld)", what, S->natoms, (long long)S->ld, (long long)S->n0);
    return GBDMC_ERR_ARG;
  }
  if (S->ld > (int64_t)INT32_MAX) {
    set_error("%s: ld %lld exceeds the 2^31-1 walker limit", what, (long long)S->ld);
    return GBDMC_ERR_CAPACITY;
  }
  if (!W->x || !W->v) {
    set_error("%s: walker x and v are required", what);
    return GBDMC_ERR_ARG;
  }
  if (S->trial.kind != GBDMC_TRIAL_NONE && (!W->f || !W->psi || !W->ke)) {
    set_error("%s: importance sampling needs f, psi and ke buffers", what);
    return GBDMC_ERR_ARG;
  }
  if (S->weighting == GBDMC_CONTINUOUS && !W->w) {
    set_error("%s: continuous weighting needs the w buffer", what);
    return GBDMC_ERR_ARG;
  }
  if (S->track_who && !W->who) {
    set_error("%s: track_who needs the who buffer", what);
    return GBDMC_ERR_ARG;
  }
  return GBDMC_OK;
}


struct InitF {
  const gbdmc_sim_t& S;
  const gbdmc_walkers_t& W;
  gbdmc_ctrl_t* ctrl;
  const ScratchLayout& L;
  cudaStream_t s;
  template <int PK, int A, int TK>
  int operator()() {
    return run_init<PK, A, TK>(S, W, ctrl, L, s);
  }
};

struct StepF {
  const gbdmc_sim_t& S;
  const gbdmc_walkers_t& src;
  const gbdmc_walkers_t& dst;
  gbdmc_ctrl_t* ctrl;
  const ScratchLayout& L;
  const gbdmc_noise_t& nz;
  cudaStream_t s;
  template <int PK, int A, int TK>
  int operator()() {
    return step_noise<PK, A, TK>(S, src, dst, ctrl, L, nz, s);
  }
};

}  // namespace gbdmc

using namespace gbdmc;

extern "C" int gbdmc_sim_init(const gbdmc_sim_t* S, const gbdmc_walkers_t* W, gbdmc_ctrl_t* ctrl, void* scratch,
                              void* stream) {
  int rc = validate(S, W, ctrl, scratch, "gbdmc_sim_init");
  if (rc) return rc;
  const ScratchLayout L = scratch_layout(scratch, S->ld);
  cudaStream_t s = (cudaStream_t)stream;
  InitF f{*S, *W, ctrl, L, s};
  return dispatch_system(*S, "gbdmc_sim_init", f);
}

extern "C" int gbdmc_sim_step(const gbdmc_sim_t* S, const gbdmc_walkers_t* src, const gbdmc_walkers_t* dst,
                              gbdmc_ctrl_t* ctrl, void* scratch, const gbdmc_noise_t* noise, void* stream) {
  int rc = validate(S, src, ctrl, scratch, "gbdmc_sim_step");
  if (rc) return rc;
  if (S->weighting == GBDMC_DISCRETE) {
    if (!dst || !dst->x || !dst->v || dst->x == src->x) {
      set_error("gbdmc_sim_step: discrete weighting needs a distinct dst buffer");
      return GBDMC_ERR_ARG;
    }
  }
  gbdmc_noise_t nz{};
  if (S->noise_mode == GBDMC_NOISE_INJECTED) {
    if (!noise || !noise->normal || !noise->u_branch ||
        (S->trial.kind != GBDMC_TRIAL_NONE && !noise->u_accept) || noise->ld_noise < 1) {
      set_error("gbdmc_sim_step: injected noise buffers missing");
      return GBDMC_ERR_ARG;
    }
    nz = *noise;
  }
  const ScratchLayout L = scratch_layout(scratch, S->ld);
  cudaStream_t s = (cudaStream_t)stream;
  const gbdmc_walkers_t d = dst ? *dst : *src;
  StepF f{*S, *src, d, ctrl, L, nz, s};
  return dispatch_system(*S, "gbdmc_sim_step", f);
}

extern "C" int gbdmc_desc_weights(const int32_t* who, const double* w, const int64_t* n_dev, int64_t n_parent,
                                  double* desc, void* stream) {
  if (!who || !n_dev || !desc || n_parent < 0) {
    set_error("gbdmc_desc_weights: invalid arguments");
    return GBDMC_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  if (n_parent > 0) {
    const cudaError_t e = cudaMemsetAsync(desc, 0, sizeof(double) * (size_t)n_parent, s);
    if (e != cudaSuccess) {
      set_error("gbdmc_desc_weights: %s", cudaGetErrorString(e));
      return GBDMC_ERR_CUDA;
    }
  }
  k_desc<<<304, 256, 0, s>>>(who, w, n_dev, n_parent, desc);
  return check_launch("gbdmc_desc_weights");
}

extern "C" int gbdmc_desc_begin(int32_t* who, const int64_t* n_dev, void* stream) {
  if (!who || !n_dev) {
    set_error("gbdmc_desc_begin: invalid arguments");
    return GBDMC_ERR_ARG;
  }
  k_iota<<<304, 256, 0, (cudaStream_t)stream>>>(who, n_dev);
  return check_launch("gbdmc_desc_begin");
}
