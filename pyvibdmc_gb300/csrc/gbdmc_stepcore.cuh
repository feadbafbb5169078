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

// Coordinates per walker and dimensions per atom of a simulation: the
// caller's layout for GBDMC_PES_EXTERNAL (pes.p[0], pes.p[1]), else 3 per atom.
__host__ __device__ __forceinline__ int ext_coords(const gbdmc_sim_t& S) {
  return (S.pes.kind == GBDMC_PES_EXTERNAL && S.pes.p[0] > 0.0) ? (int)S.pes.p[0] : 3 * S.natoms;
}
__host__ __device__ __forceinline__ int ext_dims(const gbdmc_sim_t& S) {
  return (S.pes.kind == GBDMC_PES_EXTERNAL && S.pes.p[1] > 0.0) ? (int)S.pes.p[1] : 3;
}

// Discrete weights and counts from stored fp64 energies with dt =
// ctrl->dt_eff (EFF: the importance-sampled fp64 path) or sim->dt (the
// caller-evaluated potential).
template <int NM, bool EFF>
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
    const double dt = EFF ? ctrl->dt_eff : S.dt;
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
        if (EFF) {
          rng.slot = 64;  // stream disjoint from the importance-sampled move's draws
        } else {
          // the draw after the move's normals (ext_coords of them, in pairs),
          // the branching uniform k_move takes for the same walker and step
          rng.skip32((uint32_t)((ext_coords(S) + 1) / 2) * (NM == GBDMC_NOISE_PHILOX32 ? 2u : 4u));
        }
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

// The surrogate step's counting, finalisation and branching in one pass
// (decoupled look-back): the discrete counts, then the gather index that
// k_branch writes for the fp64 path, with the tile prefixes found on the fly
// instead of by a separate finalisation kernel.  Tiles are kCBW walkers,
// kCBW / blockDim consecutive walkers per thread (the table T is cut at that
// width).  No fp64 instruction per walker (the fp64 pipe bounded the fp64
// counting of this path):
//   dv = fp32(V) - fp32(vref), V converted on the integer pipes, fp32(vref)
//   and fp32(dt_eff) from ctrl->reserved[3] (written by the step's first
//   kernel, and by the audit for dt_eff);
//   w = exp(-dv dt) in fp32 (ex2.approx, ~2 ulp); the weight cap as the fp32
//   w_hi_f of the table;
//   the branching uniform compared with the fractional weight as its 53-bit
//   integer (u53_below);
//   the tile's sum of c V as fp32(vref) sum c + sum c dv, the second sum in
//   fp32 (the rounding of vref cancels); births = sum c - live + deaths.
// - Blocks take tiles in ticket order (sync[0]); a tile's predecessors in its
//   replica hold earlier tickets, so they are running or done.
// - A tile publishes its count total as an aggregate (state A) in its status
//   word, then warp 0 looks back over its predecessors 32 at a time (bounded
//   waits) until it meets an inclusive prefix (state P), and the tile
//   publishes its own inclusive prefix.  The words carry the replica's step,
//   so a word left from an earlier step never counts; the audit kernel
//   zeroes them and the tickets every step.
// - Each walker then writes its ancestor index c times from the tile's
//   prefix plus its place in the tile's scan (np.repeat(arange(N), counts),
//   pyvibdmc.py:417-430).
// - Live tiles write their partial (c, births, deaths, sum c V) before they
//   publish; the replica's last tile, once its look-back has seen every
//   earlier tile, reduces the live partials in the fixed order of
//   reduce_partials and finalises N', vref and the guards.
// A wait that runs out sets GBDMC_ST_TIMEOUT on the replica (its later tiles
// then skip, and their own waits run out too) and the kernel returns.
constexpr int kCBW = 2048;  // walkers per tile of the single-pass counting kernel (measured: 1024, 2048, 4096)
template <int NM>
__global__ void __launch_bounds__(kMaxTPB) k_count_branch_f32(const __grid_constant__ gbdmc_sim_t S,
                                                               const __grid_constant__ RepTable T,
                                                               const double* __restrict__ V, gbdmc_ctrl_t* ctrls,
                                                               Partial* part, unsigned long long* tstat,
                                                               unsigned int* sync, int32_t* __restrict__ idx,
                                                               const gbdmc_noise_t nz) {
  constexpr unsigned long long kA = 1ull << 30, kP = 2ull << 30, kVal = (1ull << 30) - 1;
  constexpr int kSpin = 1 << 22;
  constexpr int WPT = kCBW / kMaxTPB;  // launched with kMaxTPB threads
  __shared__ int s_tile, s_st;
  __shared__ long long s_n, s_step, s_prefix;
  __shared__ float2 s_vd;
  __shared__ int wsum[kMaxTPB / 32];
  __shared__ int4 sh[kMaxTPB / 32];  // per warp: deaths, guard bits, sum c dv (bits)
  pdl_wait();
  const int ntile = T.tile_off[T.nrep];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (;;) {
    if (threadIdx.x == 0) {
      const int t = (int)atomicAdd(&sync[0], 1u);
      s_tile = t;
      if (t < ntile) {
        const gbdmc_ctrl_t* ctrl = ctrls + replica_of(T, t);
        s_st = *(volatile const int*)&ctrl->status;
        s_n = ctrl->n;
        s_step = ctrl->step;
        s_vd = *reinterpret_cast<const float2*>(&ctrl->reserved[3]);  // fp32 vref, dt_eff
      }
    }
    __syncthreads();
    const int tile = s_tile;
    if (tile >= ntile) break;  // block-uniform
    const int r = replica_of(T, tile);
    gbdmc_ctrl_t* ctrl = ctrls + r;
    const int t0 = T.tile_off[r], t1 = T.tile_off[r + 1];
    const long long n = s_n, step = s_step;
    if (s_st == 0) {  // block-uniform (read once by thread 0)
      const int64_t i0 = (int64_t)(tile - t0) * kCBW;
      const int64_t ib = i0 + (int64_t)threadIdx.x * WPT;  // this thread's first walker
      const int64_t base = T.off[r];
      double v[WPT];
#pragma unroll
      for (int k = 0; k < WPT; ++k) v[k] = ib + k < n ? V[base + ib + k] : 0.0;
      int c[WPT], csum = 0, nd = 0, fl = 0;
      float sf = 0.f;
#pragma unroll
      for (int k = 0; k < WPT; ++k) {
        c[k] = 0;
        const int64_t i = ib + k;
        if (i < n) {
          const float dv = d2f_rn_int(v[k]) - s_vd.x;
          const float wf = __expf(-dv * s_vd.y);
          if (!isfinite(wf)) {
            fl |= GBDMC_ST_NONFINITE_WEIGHT;
          } else if (wf > T.w_hi_f[r]) {
            fl |= GBDMC_ST_HUGE_WEIGHT;
          } else {
            const float w0 = floorf(wf), fr = wf - w0;
            bool up;
            if constexpr (NM == GBDMC_NOISE_INJECTED) {
              up = nz.u_branch[base + i] < (double)fr;
            } else {
              Rng rng(S.seed, (uint64_t)step, (uint64_t)i, T.stream[r]);
              rng.slot = 64;  // stream disjoint from the move's draws
              up = u53_below(rng.bits53(), fr);
            }
            c[k] = (int)w0 + (up ? 1 : 0);
            nd += c[k] == 0 ? 1 : 0;
            sf += (float)c[k] * dv;
          }
        }
        csum += c[k];
      }
      // the tile's scan of the thread totals and its sums (fixed order)
      const int inc = warp_incl_scan(csum);
      nd = __reduce_add_sync(0xffffffffu, nd);
      fl = __reduce_or_sync(0xffffffffu, fl);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) sf += __shfl_down_sync(0xffffffffu, sf, o);
      if (lane == 31) wsum[wid] = inc;
      if (lane == 0) sh[wid] = make_int4(nd, fl, __float_as_int(sf), 0);
      __syncthreads();
      int off = 0;
      for (int w = 0; w < wid; ++w) off += wsum[w];
      if (wid == 0) {  // warp 0: totals, partial, publication and look-back
        long long ctot = 0, dtot = 0;
        int ftot = 0;
        float stot = 0.f;
        for (int w = 0; w < nw; ++w) {
          ctot += wsum[w];
          dtot += sh[w].x;
          ftot |= sh[w].y;
          stot += __int_as_float(sh[w].z);
        }
        const unsigned long long ep = (unsigned long long)(uint32_t)step << 32;
        const unsigned long long agg = (unsigned long long)(ctot < (long long)kVal ? ctot : (long long)kVal);
        if (lane == 0) {
          if (i0 < n) {  // a live tile: its partial for the finalisation
            const long long live = n - i0 < (long long)kCBW ? n - i0 : (long long)kCBW;
            Partial p = partial_zero();
            p.c = ctot;
            p.births = ctot - live + dtot;
            p.deaths = dtot;
            p.s0 = fma((double)s_vd.x, (double)ctot, (double)stot);
            part[tile] = p;
          }
          if (ftot) atomicOr(&ctrl->flags, ftot);
          __threadfence();  // partial and guard bits before the status word
          atomicExch(&tstat[tile], ep | (tile == t0 ? kP : kA) | agg);
        }
        long long prefix = 0;
        bool timeout = false;
        for (int jt = tile - 1; jt >= t0; jt -= 32) {  // 32 predecessors per round (warp-uniform)
          const int j = jt - lane;
          unsigned long long w = 0;
          bool ready = j < t0;  // lanes before the replica's first tile add nothing
          for (int it = 0;; ++it) {
            if (!ready) {
              w = *(volatile unsigned long long*)&tstat[j];
              ready = (w >> 32) == (uint32_t)step && (w & (kA | kP)) != 0;
            }
            if (__all_sync(0xffffffffu, ready)) break;
            if (it >= kSpin) {
              timeout = true;
              break;
            }
            if (it > 64) __nanosleep(64);
          }
          if (timeout) break;
          const unsigned pm = __ballot_sync(0xffffffffu, j >= t0 && (w & kP) != 0);
          const int stop = pm ? __ffs(pm) - 1 : 32;  // the nearest inclusive prefix
          long long val = (j >= t0 && lane <= stop) ? (long long)(w & kVal) : 0;
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) val += __shfl_xor_sync(0xffffffffu, val, o);
          prefix += val;
          if (pm) break;
        }
        if (lane == 0) {
          if (timeout) atomicOr(&ctrl->status, GBDMC_ST_TIMEOUT);
          __threadfence();  // what the predecessors published, before this tile's word and the finalisation
          if (tile != t0) {
            const long long inclusive = prefix + ctot;
            atomicExch(&tstat[tile],
                       ep | kP | (unsigned long long)(inclusive < (long long)kVal ? inclusive : (long long)kVal));
          }
          s_prefix = prefix;
        }
      }
      __syncthreads();
      // the ancestor index of each copy
      long long dest = s_prefix + off + inc - csum;
      const long long cap = T.cap[r];
#pragma unroll
      for (int k = 0; k < WPT; ++k) {
        for (int q = 0; q < c[k]; ++q)
          if (GBDMC_BC(dest + q, 0, cap + 1, kBcSurrogateWrite) < cap) idx[base + dest + q] = (int32_t)(ib + k);
        dest += c[k];
      }
      // the replica's last tile finalises it (block-uniform)
      if (tile == t1 - 1) {
        const int nt = (int)((n + kCBW - 1) / kCBW);
        const Partial tot = reduce_partials<false>(part, t0, nt, nullptr);
        if (threadIdx.x < 32) finalize_discrete<false>(S, T, r, ctrl, tot, n, step);
      }
    }
    __syncthreads();  // the shared words are rewritten by the next ticket
  }
  if (threadIdx.x == 0 && atomicAdd(&sync[1], 1u) == gridDim.x - 1) {  // the last block out resets the tickets
    sync[0] = 0;
    sync[1] = 0;
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
