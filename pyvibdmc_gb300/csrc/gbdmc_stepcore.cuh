// Building blocks shared by the step kernels: per-tile partials, the
// last-tile election, the fixed-order partial reduction and prefix scan, the
// discrete branch count and the finalisation of a branching pass.
#pragma once
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

// Warp reduction of a Partial (result in lane 0): counts on the integer
// pipes, min/max of V as order-preserving integer keys, the two fp64 sums
// with the paired reduction -- five fp64 adds per lane in all.
template <bool STATS>
__device__ __forceinline__ void warp_reduce_partial(Partial& p) {
  p.c = warp_sum(p.c);
  p.births = warp_sum(p.births);
  p.deaths = warp_sum(p.deaths);
  p.aux = warp_sum(p.aux);
  if (STATS) {
    warp_sum2(p.s0, p.s1);
    p.vmin = dkey_inv(warp_min_key(dkey(p.vmin)));
    p.vmax = dkey_inv(warp_max_key(dkey(p.vmax)));
  } else {
    p.s0 = warp_sum(p.s0);
  }
}

// Deterministic block reduction of a Partial (fixed shuffle/shared tree).
// STATS: also the fp64 sum/min/max of V.  Result valid in thread 0.
template <bool STATS>
__device__ Partial block_reduce_partial(Partial p) {
  __shared__ Partial sh[kMaxTPB / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  warp_reduce_partial<STATS>(p);
  if (lane == 0) sh[wid] = p;
  __syncthreads();
  if (wid == 0) {
    p = lane < nw ? sh[lane] : partial_zero();
    warp_reduce_partial<STATS>(p);
  }
  __syncthreads();
  return p;
}

__device__ __forceinline__ Partial load_partial(const Partial* p) {
  Partial r;
  const longlong2* q = reinterpret_cast<const longlong2*>(p);  // partials are 64-byte aligned
  longlong2* o = reinterpret_cast<longlong2*>(&r);
#pragma unroll
  for (int k = 0; k < 4; ++k) o[k] = __ldcg(q + k);
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

__device__ __forceinline__ int replica_of(const RepTable& T, int tile) {
  int lo = 0, hi = T.nrep - 1;
  while (lo < hi) {  // last r with tile_off[r] <= tile
    const int mid = (lo + hi + 1) >> 1;
    if (T.tile_off[mid] <= tile) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// The weight-guard bits (GBDMC_ST_NONFINITE_WEIGHT, GBDMC_ST_HUGE_WEIGHT)
// raised by any thread of the block, ORed into ctrl->flags by thread 0.
// Called by every thread; one barrier when no walker of the block tripped a
// guard (the common case), three when one did.
__device__ __forceinline__ void flag_weights(gbdmc_ctrl_t* ctrl, int flag) {
  if (__syncthreads_or(flag)) {
    const int f = (__syncthreads_or(flag & GBDMC_ST_NONFINITE_WEIGHT) ? GBDMC_ST_NONFINITE_WEIGHT : 0) |
                  (__syncthreads_or(flag & GBDMC_ST_HUGE_WEIGHT) ? GBDMC_ST_HUGE_WEIGHT : 0);
    if (threadIdx.x == 0) atomicOr(&ctrl->flags, f);
  }
}

// Elects the last tile of replica `ctrl` to finish (threadFenceReduction
// pattern, no waiting).  Every thread of the block calls it after the tile's
// partial is written; returns true in all threads of the electing block.
__device__ __forceinline__ bool last_tile(gbdmc_ctrl_t* ctrl, int ntiles) {
  __shared__ bool am_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned t = atomicAdd(&ctrl->ticket, 1u);
    am_last = (t == (unsigned)ntiles - 1u);
  }
  __syncthreads();
  const bool r = am_last;
  if (r) __threadfence();
  __syncthreads();
  return r;
}

// Fixed-order reduction of the partials of tiles [t0, t0+nt) (and, when
// prefix != NULL, an exclusive scan of their counts into prefix[]).  The
// tiles are taken in chunks of blockDim (thread t accumulates tiles t,
// t+B, t+2B, ...); the next chunk's partial is loaded while the current
// chunk is scanned, and every count is read once.
template <bool STATS>
__device__ Partial reduce_partials(const Partial* part, int t0, int nt, long long* prefix) {
  __shared__ long long wsum[kMaxTPB / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  Partial acc = partial_zero();
  long long carry = 0;
  Partial cur = (int)threadIdx.x < nt ? load_partial(part + t0 + threadIdx.x) : partial_zero();
  for (int c0 = 0; c0 < nt; c0 += blockDim.x) {
    const int j = c0 + threadIdx.x;
    const int jn = j + blockDim.x;
    const Partial nxt = jn < nt ? load_partial(part + t0 + jn) : partial_zero();
    accumulate(acc, cur);
    if (prefix) {
      long long v = cur.c;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const long long t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
      }
      if (lane == 31) wsum[wid] = v;
      __syncthreads();
      long long before = carry, total = 0;
      for (int w = 0; w < nw; ++w) {
        const long long ws = wsum[w];
        if (w < wid) before += ws;
        total += ws;
      }
      if (j < nt) prefix[t0 + j] = before + v - cur.c;
      carry += total;
      __syncthreads();
    }
    cur = nxt;
  }
  return block_reduce_partial<STATS>(acc);
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

__device__ __forceinline__ int64_t hidx(const gbdmc_sim_t& S, int r, long long step) {
  return (int64_t)r * S.hist.len + step;
}

// Finalisation of a discrete branching pass of replica r, run by the 32
// lanes of warp 0 (tot valid in lane 0; n, step = the pass's population and
// step counter).  The pass's three divisions -- <V> of the branched
// population s0/N', the population term (N'-N0)/N0 and the pre-branch mean
// s1/N -- are one SIMT division in lanes 0, 1, 2; lane 0 then applies the
// population guards and writes vref, N', the history and the control block
// (pyvibdmc.py:380-431, :651-661).
template <bool STATS>
__device__ __forceinline__ void finalize_discrete(const gbdmc_sim_t& S, const RepTable& T, int r,
                                                  gbdmc_ctrl_t* ctrl, const Partial& tot, long long n,
                                                  long long step) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  int st = 0;
  if (lane == 0) st = *(volatile int*)&ctrl->status | *(volatile int*)&ctrl->flags;
  const long long nn = __shfl_sync(full, tot.c, 0);
  const long long n0 = T.n0[r];
  const double s0 = __shfl_sync(full, tot.s0, 0);
  const double s1 = STATS ? __shfl_sync(full, tot.s1, 0) : 0.0;
  const double num = lane == 0 ? s0 : (lane == 1 ? (double)(nn - n0) : s1);
  const double den = lane == 0 ? (double)nn : (lane == 1 ? (double)n0 : (double)n);
  const double q = num / den;
  const double vbar = __shfl_sync(full, q, 0);
  const double corr = __shfl_sync(full, q, 1);
  const double vmean = __shfl_sync(full, q, 2);
  if (lane != 0) return;
  if (STATS && step < S.hist.len) {
    const int64_t h = hidx(S, r, step);
    if (S.hist.vmin) S.hist.vmin[h] = tot.vmin;
    if (S.hist.vmax) S.hist.vmax[h] = tot.vmax;
    if (S.hist.vmean) S.hist.vmean[h] = vmean;
  }
  ctrl->flags = 0;
  if (!st) {
    const double d0 = (double)n0;
    if ((double)nn < d0 - d0 * 0.5) st |= GBDMC_ST_POP_LOW;
    if ((double)nn > d0 + d0 * 0.5) st |= GBDMC_ST_POP_HIGH;
    if (nn > T.cap[r]) st |= GBDMC_ST_OVERFLOW;
  }
  if (st) {
    ctrl->status = st;
    ctrl->err_step = (int)step;
  } else {
    const double vref = vbar - S.alpha * corr;
    if (step < S.hist.len) {
      const int64_t h = hidx(S, r, step);
      if (S.hist.vref) S.hist.vref[h] = vref;
      if (S.hist.pop) S.hist.pop[h] = (double)nn;
      if (S.hist.births) S.hist.births[h] = (int)tot.births;
      if (S.hist.deaths) S.hist.deaths[h] = (int)tot.deaths;
    }
    ctrl->n_prev = n;
    ctrl->n = nn;
    ctrl->vref = vref;
    ctrl->step = step + 1;
  }
  ctrl->reserved[2] = 0;  // surrogate path: analytic-energy list of the step
  ctrl->ticket = 0;
}

template <bool STATS>
__device__ __forceinline__ void record_vstats(const gbdmc_sim_t& S, int r, long long step, long long n,
                                              const Partial& t) {
  if (STATS && step < S.hist.len) {
    const int64_t h = hidx(S, r, step);
    if (S.hist.vmin) S.hist.vmin[h] = t.vmin;
    if (S.hist.vmax) S.hist.vmax[h] = t.vmax;
    if (S.hist.vmean) S.hist.vmean[h] = t.s1 / (double)n;
  }
}

template <int A>
__device__ __forceinline__ double local_ke(const gbdmc_sim_t& S, const double (&d2)[3 * A]) {
  // -1/2 sum_d sum_a (1/m_a) d2psi/psi (imp_samp.py:49-53: atoms first, then dims)
  double s = 0.0;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    double t = 0.0;
#pragma unroll
    for (int a = 0; a < A; ++a) t = t + S.inv_mass[a] * d2[3 * a + d];
    s = s + t;
  }
  return -0.5 * s;
}

// Discrete weights and counts from stored fp64 energies with dt =
// ctrl->dt_eff (the importance-sampled fp64 path).
template <int NM>
__global__ void __launch_bounds__(kMaxTPB) k_count(const __grid_constant__ gbdmc_sim_t S,
                                                    const __grid_constant__ RepTable T, const double* __restrict__ V,
                                                    gbdmc_ctrl_t* ctrls, Partial* part, int* counts,
                                                    const gbdmc_noise_t nz) {
  const int ntile = T.tile_off[T.nrep];
  for (int tile = blockIdx.x; tile < ntile; tile += gridDim.x) {
    const int r = replica_of(T, tile);
    gbdmc_ctrl_t* ctrl = ctrls + r;
    const int64_t i = (int64_t)(tile - T.tile_off[r]) * blockDim.x + threadIdx.x;
    const int64_t dst = T.off[r] + i;
    // the energy load is issued with the control-block loads (slot i < cap is inside the replica)
    const double v = i < T.cap[r] ? V[dst] : 0.0;
    if (*(volatile int*)&ctrl->status) continue;
    const long long n = ctrl->n;
    const long long step = ctrl->step;
    const double vref = ctrl->vref;
    const double dt = ctrl->dt_eff;
    const double n0 = (double)T.n0[r];
    const double w_hi = (n0 + n0 * 0.5) + 1.0;
    int flag = 0;
    Partial p = partial_zero();
    if (i < n) {
      double u;
      if constexpr (NM == GBDMC_NOISE_INJECTED) {
        u = nz.u_branch[dst];
      } else {
        Rng rng(S.seed, (uint64_t)step, (uint64_t)i, T.stream[r]);
        rng.slot = 64;  // stream disjoint from the move's draws
        u = rng.uniform53();
      }
      const int c = branch_count(v, vref, dt, u, w_hi, flag, p.births, p.deaths);
      counts[dst] = c;
      p.c = c;
      p.s0 = c == 1 ? v : (double)c * v;
    }
    flag_weights(ctrl, flag);
    p = block_reduce_partial<false>(p);
    if (threadIdx.x == 0) part[tile] = p;
  }
}

// Counting for the surrogate path (fp32 walkers, energies with ~1e-4
// relative error), with no fp64 instruction per walker -- the fp64 pipe
// bounded the fp64 version of this pass:
//   dv = fp32(V) - fp32(vref), V converted on the integer pipes, fp32(vref)
//   and fp32(dt_eff) from ctrl->reserved[3] (written by the step's first
//   kernel, and by the audit for dt_eff);
//   w = exp(-dv dt) in fp32 (ex2.approx, ~2 ulp); the weight cap as the fp32
//   w_hi_f of the table;
//   the branching uniform compared with the fractional weight as its 53-bit
//   integer (u53_below);
//   the tile's sum of c V as fp32(vref) sum c + sum c dv, the second sum in
//   fp32 (the rounding of vref cancels); births = sum c - live + deaths.
// A block takes TPI consecutive tiles per iteration (their loads in flight
// together, one pair of barriers for all TPI reductions; TPI = 1 when the
// tiles fit the resident blocks).  Tiles at or beyond N write nothing:
// k_count_finalize reduces the first ceil(N / tile) partials only.
template <int NM, int TPI>
__global__ void __launch_bounds__(kMaxTPB) k_count_f32(const __grid_constant__ gbdmc_sim_t S,
                                                        const __grid_constant__ RepTable T,
                                                        const double* __restrict__ V, gbdmc_ctrl_t* ctrls,
                                                        Partial* part, int* counts, const gbdmc_noise_t nz) {
  static_assert(TPI >= 1 && TPI <= 4, "warp u of the block reduces tile u: launched with >= 4 warps per block");
  __shared__ int4 sh[TPI][kMaxTPB / 32];  // per warp: sum c, deaths, guard bits, sum c dv
  pdl_wait();
  const int ntile = T.tile_off[T.nrep];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int tb = blockIdx.x * TPI; tb < ntile; tb += gridDim.x * TPI) {
    int r[TPI];
    int64_t i[TPI];
    double v[TPI];
    int rr = replica_of(T, tb);
#pragma unroll
    for (int u = 0; u < TPI; ++u) {
      const int tile = min(tb + u, ntile - 1);  // a clamped duplicate is masked below
      while (rr + 1 < T.nrep && tile >= T.tile_off[rr + 1]) ++rr;
      r[u] = rr;
      i[u] = (int64_t)(tile - T.tile_off[rr]) * blockDim.x + threadIdx.x;
      v[u] = i[u] < T.cap[rr] ? V[T.off[rr] + i[u]] : 0.0;
    }
    int c[TPI], nd[TPI], fl[TPI];
    long long nn[TPI];
    float sf[TPI], vr[TPI];
#pragma unroll
    for (int u = 0; u < TPI; ++u) {
      c[u] = nd[u] = fl[u] = 0;
      sf[u] = 0.f;
      const gbdmc_ctrl_t* ctrl = ctrls + r[u];
      const int st = *(volatile const int*)&ctrl->status;
      nn[u] = st == 0 && tb + u < ntile ? ctrl->n : 0;  // 0: nothing of this tile is counted
      const float2 vd = *reinterpret_cast<const float2*>(&ctrl->reserved[3]);  // fp32 vref, dt_eff
      vr[u] = vd.x;
      if (i[u] < nn[u]) {
        const int64_t dst = T.off[r[u]] + i[u];
        const float dv = d2f_rn_int(v[u]) - vd.x;
        const float wf = __expf(-dv * vd.y);
        if (!isfinite(wf)) {
          fl[u] = GBDMC_ST_NONFINITE_WEIGHT;
        } else if (wf > T.w_hi_f[r[u]]) {
          fl[u] = GBDMC_ST_HUGE_WEIGHT;
        } else {
          const float w0 = floorf(wf), fr = wf - w0;
          bool up;
          if constexpr (NM == GBDMC_NOISE_INJECTED) {
            up = nz.u_branch[dst] < (double)fr;
          } else {
            Rng rng(S.seed, (uint64_t)ctrl->step, (uint64_t)i[u], T.stream[r[u]]);
            rng.slot = 64;  // stream disjoint from the move's draws
            up = u53_below(rng.bits53(), fr);
          }
          c[u] = (int)w0 + (up ? 1 : 0);
          nd[u] = c[u] == 0 ? 1 : 0;
          sf[u] = (float)c[u] * dv;
        }
        counts[dst] = c[u];
      }
    }
#pragma unroll
    for (int u = 0; u < TPI; ++u) {
      c[u] = __reduce_add_sync(0xffffffffu, c[u]);
      nd[u] = __reduce_add_sync(0xffffffffu, nd[u]);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) sf[u] += __shfl_down_sync(0xffffffffu, sf[u], o);
      fl[u] = __reduce_or_sync(0xffffffffu, fl[u]);
      if (lane == 0) sh[u][wid] = make_int4(c[u], nd[u], fl[u], __float_as_int(sf[u]));
    }
    __syncthreads();
    if (wid < TPI) {  // warp u: the fixed-order sums of tile tb + u
      int ru = r[0];
      long long nu = nn[0];
      int64_t i0 = i[0] - threadIdx.x;
      float vu = vr[0];
#pragma unroll
      for (int u = 1; u < TPI; ++u)
        if (wid == u) {
          ru = r[u];
          nu = nn[u];
          i0 = i[u] - threadIdx.x;
          vu = vr[u];
        }
      if (i0 < nu) {  // a live tile of a running replica (warp-uniform)
        int4 q = lane < nw ? sh[wid][lane] : make_int4(0, 0, 0, 0);
        float t = __int_as_float(q.w);
        q.x = __reduce_add_sync(0xffffffffu, q.x);
        q.y = __reduce_add_sync(0xffffffffu, q.y);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
        const int f = __reduce_or_sync(0xffffffffu, q.z);
        if (lane == 0) {
          if (f) atomicOr(&ctrls[ru].flags, f);
          const long long live = nu - i0 < (long long)blockDim.x ? nu - i0 : (long long)blockDim.x;
          Partial p = partial_zero();
          p.c = q.x;
          p.births = (long long)q.x - live + q.y;
          p.deaths = q.y;
          p.s0 = fma((double)vu, (double)q.x, (double)t);
          part[tb + wid] = p;
        }
      }
    }
    __syncthreads();  // sh is reused by the next iteration
  }
}

// Finalisation of a counting pass, one CTA per replica: the partial
// reduction, the tile-count scan into prefix[] and finalize_discrete.  The
// kernel boundary after k_count makes every tile's partial visible, so the
// counting tiles need no fence and no last-tile election.
static __global__ void __launch_bounds__(kMaxTPB) k_count_finalize(const __grid_constant__ gbdmc_sim_t S,
                                                                    const __grid_constant__ RepTable T,
                                                                    gbdmc_ctrl_t* ctrls, const Partial* part,
                                                                    long long* prefix) {
  pdl_wait();  // (a no-op when launched without programmatic serialisation)
  for (int r = blockIdx.x; r < T.nrep; r += gridDim.x) {
    gbdmc_ctrl_t* ctrl = ctrls + r;
    if (*(volatile int*)&ctrl->status) continue;  // block-uniform: only this block writes this replica's status
    const long long n = ctrl->n, step = ctrl->step;
    const int nt = (int)((n + T.tpb - 1) / T.tpb);  // the tiles below N (the counting passes' live tiles)
    const Partial t = reduce_partials<false>(part, T.tile_off[r], nt, prefix);
    if (threadIdx.x < 32) finalize_discrete<false>(S, T, r, ctrl, t, n, step);
    __syncthreads();  // the next replica reuses reduce_partials' shared memory
  }
}

}  // namespace gbdmc
