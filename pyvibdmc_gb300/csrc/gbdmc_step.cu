// The DMC walker step on the GPU, for one simulation or a batch of
// independent replicas (up to GBDMC_MAX_REPLICAS per launch).
//
// Walkers are SoA; replica r owns slots [off_r, off_r + cap_r).  Each
// replica's capacity is cut into tiles of `tpb` walkers; a launch runs a
// grid-stride (persistent) loop over all tiles of all replicas.  Per step,
// discrete weighting, plain DMC (2 launches):
//   k_move   : gather walker j of the replica through src->idx, x += sigma*z
//              (bit-exact x + fl(sigma*z)), V = PES(x), w = exp(-(V-vref) dt),
//              c = floor(w) + [u < w - floor(w)]; writes the moved walker to
//              slot j of dst (pre-branch order), c to counts[], a partial per
//              tile.  The last tile of each replica to finish scans the tile
//              counts into prefix[], computes N', vref' and the population
//              guards (pyvibdmc.py:380-431, :651-661).
//   k_branch : walker j writes its index j into dst->idx[prefix + scan, +c),
//              i.e. np.repeat(arange(N), counts); the next step gathers
//              through it, so branching moves 4 bytes per walker copy instead
//              of the whole walker state.
// Importance sampling: k_is_move (drift-diffusion proposal, trial psi and its
// adjoint at the proposal, Metropolis, accept, V + local KE;
// pyvibdmc.py:549-612, :807-809), then k_count (weights with
// dt_eff = dt * accepted/N) and k_branch.  Continuous weighting replaces
// count/branch by k_cont_branch, one CTA per replica (sequential argmax
// cloning, pyvibdmc.py:340-356, :432-454).
#include <cmath>
#include <mutex>
#include "gbdmc_device.cuh"
#include "gbdmc_internal.cuh"
#include "gbdmc_stepcore.cuh"
#include "gbdmc_select.cuh"

namespace gbdmc {

// ------------------------------------------------------------------ init
// Step 0 on compact walkers: V (+ local KE with a trial psi) and the first
// vref (pyvibdmc.py:760-769).
template <int PK, int A, int TK>
__global__ void __launch_bounds__(kMaxTPB) k_init(const __grid_constant__ gbdmc_sim_t S,
                                                   const __grid_constant__ RepTable T, gbdmc_walkers_t W,
                                                   gbdmc_ctrl_t* ctrls, Partial* part) {
  const int64_t ld = S.ld;
  const int ntile = T.tile_off[T.nrep];
  for (int tile = blockIdx.x; tile < ntile; tile += gridDim.x) {
    const int r = replica_of(T, tile);
    gbdmc_ctrl_t* ctrl = ctrls + r;
    const long long n = ctrl->n;
    const int64_t i = (int64_t)(tile - T.tile_off[r]) * blockDim.x + threadIdx.x;
    const int64_t slot = T.off[r] + i;
    Partial p = partial_zero();
    if (i < n) {
      double v;
      if constexpr (PK == GBDMC_PES_EXTERNAL) {
        v = W.v[slot];  // the caller's potential
      } else {
        double x[3 * A], g[3 * A];
#pragma unroll
        for (int k = 0; k < 3 * A; ++k) x[k] = W.x[k * ld + slot];
        v = pes<PK, A, false>(x, S.pes, g);
      }
      if constexpr (TK != GBDMC_TRIAL_NONE && PK != GBDMC_PES_EXTERNAL) {
        double x[3 * A];
#pragma unroll
        for (int k = 0; k < 3 * A; ++k) x[k] = W.x[k * ld + slot];
        double d1[3 * A], d2[3 * A];
        const double psi = trial<TK, A>(x, S.trial, d1, d2);
        const double ke = local_ke<A>(S, d2);
#pragma unroll
        for (int k = 0; k < 3 * A; ++k) W.f[k * ld + slot] = d1[k];
        W.psi[slot] = psi;
        W.ke[slot] = ke;
        v = v + ke;
      }
      W.v[slot] = v;
      if (S.weighting == GBDMC_CONTINUOUS) {
        const double w = W.w[slot];
        p.s0 = v * w;
        p.s1 = w;
      } else {
        p.s0 = v;
        p.s1 = 1.0;
      }
      p.c = 1;
    }
    p = block_reduce_partial<true>(p);
    if (threadIdx.x == 0) part[tile] = p;
    const int nt = T.tile_off[r + 1] - T.tile_off[r];
    if (last_tile(ctrl, nt)) {
      const Partial t = reduce_partials<true>(part, T.tile_off[r], nt, nullptr);
      if (threadIdx.x == 0) {
        const double n0 = (double)T.n0[r];
        double vref;
        if (S.weighting == GBDMC_CONTINUOUS)
          vref = t.s0 / t.s1 - S.alpha * ((t.s1 - n0) / n0);
        else
          vref = t.s0 / (double)n - S.alpha * ((double)(n - T.n0[r]) / n0);
        ctrl->vref = vref;
        ctrl->ticket = 0;
      }
    }
  }
}

// --------------------------------------------------------- plain move
// COUNT: fused discrete weights/counts (+ last-tile scan); otherwise the
// move and potential only (continuous weighting).
template <int PK, int A, int NM, bool COUNT, bool STATS>
__global__ void __launch_bounds__(kMaxTPB) k_move(const __grid_constant__ gbdmc_sim_t S,
                                                   const __grid_constant__ RepTable T, const gbdmc_walkers_t in,
                                                   gbdmc_walkers_t out, gbdmc_ctrl_t* ctrls, Partial* part,
                                                   long long* prefix, int* counts, const gbdmc_noise_t nz) {
  pdl_wait();
  pdl_trigger();
  const int64_t ld = S.ld;
  const int ntile = T.tile_off[T.nrep];
  for (int tile = blockIdx.x; tile < ntile; tile += gridDim.x) {
    const int r = replica_of(T, tile);
    gbdmc_ctrl_t* ctrl = ctrls + r;
    const int64_t base = T.off[r];
    const int64_t i = (int64_t)(tile - T.tile_off[r]) * blockDim.x + threadIdx.x;
    // A gather through the index is issued before the control block arrives
    // (their loads overlap): slot i < cap lies inside the replica and the index
    // is clamped into it, so the walkers of slots i >= N are read harmlessly
    // and then ignored.  Compact sources (possibly host memory) are read after
    // N is known, walkers i < N only.
    double x[3 * A];
    int64_t src = base + i;
    if (in.idx && i < T.cap[r]) {
      src = base + min(max((int64_t)__ldg(in.idx + base + i), (int64_t)0), T.cap[r] - 1);
#pragma unroll
      for (int k = 0; k < 3 * A; ++k) x[k] = in.x[k * ld + src];
    }
    if (*(volatile int*)&ctrl->status) continue;  // replica stopped by a previous kernel
    const long long n = ctrl->n;
#ifdef GBDMC_BOUNDS_CHECK
    if (in.idx && i < n) (void)GBDMC_BC(in.idx[base + i], 0, ctrl->n_prev, kBcMoveGather);
#endif
    if (!in.idx && i < n) {
#pragma unroll
      for (int k = 0; k < 3 * A; ++k) x[k] = in.x[k * ld + src];
    }
    const long long step = ctrl->step;
    const double vref = ctrl->vref;
    Partial p = partial_zero();
    int flag = 0;
    if (i < n) {
      const int64_t dst = base + i;
      double z[3 * A], g[3 * A];
      Rng rng(S.seed, (uint64_t)step, (uint64_t)i, T.stream[r]);
      if constexpr (NM == GBDMC_NOISE_INJECTED) {
#pragma unroll
        for (int k = 0; k < 3 * A; ++k) z[k] = nz.normal[k * nz.ld_noise + dst];
      } else {
        gen_normals<NM, 3 * A>(rng, z);
      }
      // x + (0 + sigma*z): the reference adds the drawn displacement (pyvibdmc.py:544-547)
#pragma unroll
      for (int k = 0; k < 3 * A; ++k) {
        x[k] = __dadd_rn(x[k], __dmul_rn(S.sigma[k / 3], z[k]));
        out.x[k * ld + dst] = x[k];
      }
      if (out.who && in.who) out.who[dst] = in.who[src];
      const double v = pes<PK, A, false>(x, S.pes, g);
      out.v[dst] = v;
      if (STATS) {
        p.s1 = v;
        p.vmin = v;
        p.vmax = v;
      }
      if constexpr (COUNT) {
        double u;
        if constexpr (NM == GBDMC_NOISE_INJECTED)
          u = nz.u_branch[dst];
        else
          u = rng.uniform53();
        const double n0 = (double)T.n0[r];
        const double w_hi = (n0 + n0 * 0.5) + 1.0;
        const int c = branch_count(v, vref, S.dt, u, w_hi, flag, p.births, p.deaths);
        counts[dst] = c;
        p.c = c;
        p.s0 = c == 1 ? v : (double)c * v;
      } else if (S.weighting == GBDMC_CONTINUOUS) {
        // this step's weight update (pyvibdmc.py:433, :837) on every SM, with the
        // vref that k_cont_branch reads (it writes the next one): the exp of
        // each walker is FP64 work that the one-CTA branching kernel would
        // otherwise do on a single SM
        out.w[dst] = in.w[src] * exp(__dmul_rn(-__dsub_rn(v, vref), S.dt));
      }
    }
    if (COUNT) flag_weights(ctrl, flag);
    p = block_reduce_partial<STATS>(p);
    if (threadIdx.x == 0) part[tile] = p;
    const int nt = T.tile_off[r + 1] - T.tile_off[r];
    if (last_tile(ctrl, nt)) {
      const Partial t = reduce_partials<STATS>(part, T.tile_off[r], nt, COUNT ? prefix : nullptr);
      if constexpr (COUNT) {
        if (threadIdx.x < 32) finalize_discrete<STATS>(S, T, r, ctrl, t, n, step);
      } else if (threadIdx.x == 0) {
        record_vstats<STATS>(S, r, step, n, t);
        ctrl->ticket = 0;
      }
    }
  }
}

// ------------------------------------- move for a caller-evaluated potential
// move_randomly (pyvibdmc.py:540-547) alone: the logical walkers of `in`
// (through in.idx) moved and written in order to `out`; nc coordinates per
// walker, d per atom (the reference's (N, A, d) walkers, drawn as (N, d, A)
// and transposed: coordinate k = d*atom + dim takes sigma[k / d]).  The
// caller evaluates V on the moved walkers and gbdmc_sim_branch weighs them.
template <int NM>
__global__ void __launch_bounds__(kMaxTPB) k_move_ext(const __grid_constant__ gbdmc_sim_t S,
                                                       const __grid_constant__ RepTable T, const gbdmc_walkers_t in,
                                                       gbdmc_walkers_t out, const gbdmc_ctrl_t* ctrls, int nc, int d,
                                                       const gbdmc_noise_t nz) {
  const int64_t ld = S.ld;
  const int ntile = T.tile_off[T.nrep];
  for (int tile = blockIdx.x; tile < ntile; tile += gridDim.x) {
    const int r = replica_of(T, tile);
    const gbdmc_ctrl_t* ctrl = ctrls + r;
    if (*(volatile const int*)&ctrl->status) continue;
    const long long n = ctrl->n;
    const int64_t i = (int64_t)(tile - T.tile_off[r]) * blockDim.x + threadIdx.x;
    if (i >= n) continue;
    const int64_t base = T.off[r];
    const int64_t src = base + (in.idx ? (int64_t)GBDMC_BC(in.idx[base + i], 0, ctrl->n_prev, kBcExtGather) : i);
    const int64_t dst = base + i;
    Rng rng(S.seed, (uint64_t)ctrl->step, (uint64_t)i, T.stream[r]);
    double z1 = 0.0;
    for (int k = 0; k < nc; ++k) {
      double z;
      if constexpr (NM == GBDMC_NOISE_INJECTED) {
        z = nz.normal[k * nz.ld_noise + dst];
      } else if ((k & 1) == 0) {  // normals in pairs, in coordinate order
        if constexpr (NM == GBDMC_NOISE_PHILOX32) {
          float a, b;
          rng.normal2_f32(a, b);
          z = widen_f32(a);
          z1 = widen_f32(b);
        } else {
          rng.normal2_f64(z, z1);
        }
      } else {
        z = z1;
      }
      out.x[k * ld + dst] = __dadd_rn(in.x[k * ld + src], __dmul_rn(S.sigma[k / d], z));
    }
    if (out.who && in.who) out.who[dst] = in.who[src];
    if (S.weighting == GBDMC_CONTINUOUS) out.w[dst] = in.w[src];
  }
}

// ----------------------------------------------- importance-sampled move
// pyvibdmc.py:549-612 with ImpSamp.metropolis (imp_samp.py:28-47) and
// local_kin (imp_samp.py:49-53).  The Green's-function ratio prod_k
// exp(-a_k^2/2s^2)/exp(-b_k^2/2s^2) is evaluated as one exp of the summed
// exponents.
template <int PK, int A, int TK, int NM, bool STATS>
__global__ void __launch_bounds__(kMaxTPB) k_is_move(const __grid_constant__ gbdmc_sim_t S,
                                                      const __grid_constant__ RepTable T, const gbdmc_walkers_t in,
                                                      gbdmc_walkers_t out, gbdmc_ctrl_t* ctrls, Partial* part,
                                                      const gbdmc_noise_t nz) {
  const int64_t ld = S.ld;
  const double dt = S.dt;
  const int ntile = T.tile_off[T.nrep];
  for (int tile = blockIdx.x; tile < ntile; tile += gridDim.x) {
    const int r = replica_of(T, tile);
    gbdmc_ctrl_t* ctrl = ctrls + r;
    if (*(volatile int*)&ctrl->status) continue;
    const long long n = ctrl->n;
    const long long step = ctrl->step;
    const int64_t base = T.off[r];
    const int64_t i = (int64_t)(tile - T.tile_off[r]) * blockDim.x + threadIdx.x;
    Partial p = partial_zero();
    if (i < n) {
      const int64_t src = base + (in.idx ? (int64_t)GBDMC_BC(in.idx[base + i], 0, ctrl->n_prev, kBcIsGather) : i);
      const int64_t dst = base + i;
      double x[3 * A], y[3 * A], fx[3 * A], fy[3 * A], sdy[3 * A], g[3 * A];
#pragma unroll
      for (int k = 0; k < 3 * A; ++k) {
        x[k] = in.x[k * ld + src];
        fx[k] = in.f[k * ld + src];
      }
      const double psi_x = in.psi[src];
      Rng rng(S.seed, (uint64_t)step, (uint64_t)i, T.stream[r]);
      double z[3 * A];
      if constexpr (NM == GBDMC_NOISE_INJECTED) {
#pragma unroll
        for (int k = 0; k < 3 * A; ++k) z[k] = nz.normal[k * nz.ld_noise + dst];
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
      double h[A];  // 1 / (2 sigma_a^2), one division per atom
#pragma unroll
      for (int a = 0; a < A; ++a) h[a] = 0.5 / (S.sigma[a] * S.sigma[a]);
      double expo = 0.0;
#pragma unroll
      for (int k = 0; k < 3 * A; ++k) {
        const double im = S.inv_mass[k / 3];
        const double a = x[k] - y[k] - im * fy[k] * dt;
        const double b = y[k] - x[k] - im * fx[k] * dt;
        expo += (b * b - a * a) * h[k / 3];
      }
      const double rr = psi_y / psi_x;
      double met = exp(expo) * (rr * rr);
      if (psi_x * psi_y <= 0.0) met = 0.0;
      double u;
      if constexpr (NM == GBDMC_NOISE_INJECTED)
        u = nz.u_accept[dst];
      else
        u = rng.uniform53();
      const bool acc = met > u;
      double ke, psi;
      if (acc) {
        ke = local_ke<A>(S, sdy);
        psi = psi_y;
#pragma unroll
        for (int k = 0; k < 3 * A; ++k) {
          x[k] = y[k];
          fx[k] = fy[k];
        }
      } else {
        ke = in.ke[src];
        psi = psi_x;
      }
#pragma unroll
      for (int k = 0; k < 3 * A; ++k) {
        out.x[k * ld + dst] = x[k];
        out.f[k * ld + dst] = fx[k];
      }
      out.psi[dst] = psi;
      out.ke[dst] = ke;
      if (out.who && in.who) out.who[dst] = in.who[src];
      if (S.weighting == GBDMC_CONTINUOUS) out.w[dst] = in.w[src];
      const double v = pes<PK, A, false>(x, S.pes, g);
      out.v[dst] = v + ke;
      p.aux = acc ? 1 : 0;
      if (STATS) {
        p.s1 = v;
        p.vmin = v;
        p.vmax = v;
      }
    }
    p = block_reduce_partial<STATS>(p);
    if (threadIdx.x == 0) part[tile] = p;
    const int nt = T.tile_off[r + 1] - T.tile_off[r];
    if (last_tile(ctrl, nt)) {
      const Partial t = reduce_partials<STATS>(part, T.tile_off[r], nt, nullptr);
      if (threadIdx.x == 0) {
        record_vstats<STATS>(S, r, step, n, t);
        // dt_factor = accepted / N (pyvibdmc.py:603); effective time (:372-378)
        const double dte = S.dt * ((double)t.aux / (double)n);
        ctrl->dt_eff = dte;
        ctrl->n_acc = t.aux;
        ctrl->eff_ts = (step == 0) ? dte : ctrl->eff_ts + dte;
        if (step < S.hist.len) {
          const int64_t h = hidx(S, r, step);
          if (S.hist.rejected) S.hist.rejected[h] = (int)(n - t.aux);
          if (S.hist.eff_ts) S.hist.eff_ts[h] = ctrl->eff_ts;
        }
        ctrl->ticket = 0;
      }
    }
  }
}

// ----------------------------------------------------------- branching
// Walker j (pre-branch order) writes j into idx[prefix[tile] + scan .. + c):
// the np.repeat(arange(N), counts) order of pyvibdmc.py:417-430.  A block
// takes TPI consecutive tiles per iteration (their loads in flight together,
// one pair of barriers for all TPI scans); TPI = 1 when the tiles fit the
// resident blocks.  Tiles at or beyond the pre-branch N are skipped.
template <int TPI>
__global__ void __launch_bounds__(kMaxTPB) k_branch(const __grid_constant__ RepTable T, int32_t* __restrict__ idx,
                                                     const gbdmc_ctrl_t* ctrls, const long long* prefix,
                                                     const int* counts) {
  pdl_wait();
  const int ntile = T.tile_off[T.nrep];
  __shared__ int wsum[TPI][kMaxTPB / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int tb = blockIdx.x * TPI; tb < ntile; tb += gridDim.x * TPI) {
    int r[TPI], c[TPI], inc[TPI];
    int64_t i[TPI];
    long long pre[TPI], np[TPI];
    // the control blocks first: tiles at or beyond N (whose prefix was not
    // written) and stopped replicas load nothing else
    int rr = replica_of(T, tb);
    bool any = false;
#pragma unroll
    for (int u = 0; u < TPI; ++u) {
      const int tile = min(tb + u, ntile - 1);  // a clamped duplicate is masked below
      while (rr + 1 < T.nrep && tile >= T.tile_off[rr + 1]) ++rr;
      r[u] = rr;
      i[u] = (int64_t)(tile - T.tile_off[rr]) * blockDim.x + threadIdx.x;
      const gbdmc_ctrl_t* ctrl = ctrls + rr;
      np[u] = tb + u < ntile && *(volatile const int*)&ctrl->status == 0 ? ctrl->n_prev : 0;
      any |= i[u] - threadIdx.x < np[u];
    }
    if (!any) continue;  // block-uniform
#pragma unroll
    for (int u = 0; u < TPI; ++u) {
      const bool tile_live = i[u] - threadIdx.x < np[u];
      c[u] = i[u] < np[u] ? counts[T.off[r[u]] + i[u]] : 0;
      pre[u] = tile_live ? prefix[tb + u] : 0;
    }
#pragma unroll
    for (int u = 0; u < TPI; ++u) {
      inc[u] = warp_incl_scan(c[u]);
      if (lane == 31) wsum[u][wid] = inc[u];
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < TPI; ++u) {
      int off = 0;
      for (int w = 0; w < wid; ++w) off += wsum[u][w];
      const long long dest = pre[u] + off + inc[u] - c[u];
      const int64_t base = T.off[r[u]];
      const long long cap = T.cap[r[u]];
      for (int q = 0; q < c[u]; ++q)
        if (GBDMC_BC(dest + q, 0, cap + 1, kBcBranchWrite) < cap) idx[base + dest + q] = (int32_t)i[u];
    }
    __syncthreads();
  }
}

// TPI = 4 once there are more than two tiles per resident block.
TileBatch tile_batch(const RepTable& T) {
  const int tiles = T.tile_off[T.nrep];
  const int resident = num_sms() * (2048 / T.tpb);
  if (tiles > 2 * resident && T.tpb >= 128) {
    const int g = (tiles + 3) / 4;
    return {4, g < resident ? g : resident};
  }
  return {1, tiles < resident ? tiles : resident};
}

// Branching straight into compact walkers, for the host-resident step:
// walker i (pre-branch, in `in`) is copied c_i times to slots prefix + scan
// .. + c_i of `out` -- the np.repeat(arange(N), counts) order of
// pyvibdmc.py:417-430 -- so no gather index and no compaction pass are needed;
// block 0 then copies the control block to ctrl_out.  A replica whose step
// failed (status set) is not written: `out` keeps the walkers it had.
template <int A, bool IS>
__global__ void __launch_bounds__(kMaxTPB) k_branch_scatter(const __grid_constant__ RepTable T, int64_t ld,
                                                             const gbdmc_walkers_t in, gbdmc_walkers_t out,
                                                             const gbdmc_ctrl_t* ctrls, const long long* prefix,
                                                             const int* counts, gbdmc_ctrl_t* ctrl_out) {
  pdl_wait();
  const int ntile = T.tile_off[T.nrep];
  __shared__ int wsum[kMaxTPB / 32];
  for (int tile = blockIdx.x; tile < ntile; tile += gridDim.x) {
    const int r = replica_of(T, tile);
    const gbdmc_ctrl_t* ctrl = ctrls + r;
    const int64_t i = (int64_t)(tile - T.tile_off[r]) * blockDim.x + threadIdx.x;
    const int64_t base = T.off[r];
    const long long cap = T.cap[r];
    const int c_raw = i < cap ? counts[base + i] : 0;
    const long long pre = prefix[tile];
    if (*(volatile const int*)&ctrl->status) continue;  // block-uniform: not written by this kernel
    const long long n = ctrl->n_prev;
    const int c = i < n ? c_raw : 0;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int inc = warp_incl_scan(c);
    if (lane == 31) wsum[wid] = inc;
    __syncthreads();
    int off = 0;
    for (int w = 0; w < wid; ++w) off += wsum[w];
    __syncthreads();
    if (c > 0) {
      const int64_t src = base + i;
      const long long dest = pre + off + inc - c;
      double x[3 * A], f[3 * A];
#pragma unroll
      for (int k = 0; k < 3 * A; ++k) x[k] = in.x[k * ld + src];
      if constexpr (IS) {
#pragma unroll
        for (int k = 0; k < 3 * A; ++k) f[k] = in.f[k * ld + src];
      }
      const double v = in.v[src];
      const int32_t who = in.who ? in.who[src] : 0;
      const double psi = IS ? in.psi[src] : 0.0, ke = IS ? in.ke[src] : 0.0;
      for (int q = 0; q < c; ++q) {
        if (dest + q >= cap) break;
        const int64_t d = base + dest + q;
#pragma unroll
        for (int k = 0; k < 3 * A; ++k) out.x[k * ld + d] = x[k];
        out.v[d] = v;
        if (out.who) out.who[d] = who;
        if constexpr (IS) {
#pragma unroll
          for (int k = 0; k < 3 * A; ++k) out.f[k * ld + d] = f[k];
          out.psi[d] = psi;
          out.ke[d] = ke;
        }
      }
    }
  }
  if (ctrl_out && blockIdx.x == 0 && threadIdx.x < (int)(sizeof(gbdmc_ctrl_t) / 8))
    reinterpret_cast<long long*>(ctrl_out)[threadIdx.x] = reinterpret_cast<const long long*>(ctrls)[threadIdx.x];
}

// ---------------------------------------------------------- compaction
template <int A, bool IS>
__global__ void __launch_bounds__(kMaxTPB) k_compact(const __grid_constant__ gbdmc_sim_t S,
                                                      const __grid_constant__ RepTable T, const gbdmc_walkers_t in,
                                                      gbdmc_walkers_t out, const gbdmc_ctrl_t* ctrls) {
  const int64_t ld = S.ld;
  const int ntile = T.tile_off[T.nrep];
  for (int tile = blockIdx.x; tile < ntile; tile += gridDim.x) {
    const int r = replica_of(T, tile);
    const long long n = ctrls[r].n;
    const int64_t i = (int64_t)(tile - T.tile_off[r]) * blockDim.x + threadIdx.x;
    if (i >= n) continue;
    const int64_t base = T.off[r];
    const int64_t src =
        base + (in.idx ? (int64_t)GBDMC_BC(in.idx[base + i], 0, ctrls[r].n_prev, kBcCompactGather) : i);
    const int64_t dst = base + i;
#pragma unroll
    for (int k = 0; k < 3 * A; ++k) out.x[k * ld + dst] = in.x[k * ld + src];
    out.v[dst] = in.v[src];
    if (in.who && out.who) out.who[dst] = in.who[src];
    if (in.w && out.w) out.w[dst] = in.w[src];
    if constexpr (IS) {
#pragma unroll
      for (int k = 0; k < 3 * A; ++k) out.f[k * ld + dst] = in.f[k * ld + src];
      out.psi[dst] = in.psi[src];
      out.ke[dst] = in.ke[src];
    }
  }
}

// ---------------------------------------------------- continuous weights
// One CTA of 1024 threads per replica: w *= exp(-(V-vref) dt); clone the
// current argmax into every walker below the lower threshold, in index order,
// halving the argmax each time (pyvibdmc.py:340-356, :432-438); the optional
// upper threshold branches the k smallest weights (k = #w > upper) in the
// order of np.argpartition(w, k)[:k] (:439-445, block_argpartition); then
// vref from the weighted mean (:659-661).  Works in place on compact walkers.
constexpr int kCTA = 1024;
static_assert(kCTA == kSelCTA, "k_cont_branch runs the block-wide select");

struct ArgBest {
  double v;
  long long i;
};

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
  const long long res = sh[0].i;
  __syncthreads();
  return res;
}

// A = 0: the atom count is sim->natoms (walkers of a caller-evaluated potential)
template <int A, bool IS>
__device__ void clone_walker(const gbdmc_sim_t& S, gbdmc_walkers_t& W, int64_t base, long long from, long long to) {
  const int64_t ld = S.ld;
  const int t = threadIdx.x;
  const int nat = A > 0 ? A : S.natoms;
  const int64_t f = base + from, d = base + to;
  if (t < 3 * nat) {
    W.x[t * ld + d] = W.x[t * ld + f];
    if constexpr (IS) W.f[t * ld + d] = W.f[t * ld + f];
  } else if (t == 3 * nat) {
    W.v[d] = W.v[f];
  } else if (t == 3 * nat + 1) {
    if (W.who) W.who[d] = W.who[f];
  } else if (t == 3 * nat + 2) {
    if constexpr (IS) {
      W.psi[d] = W.psi[f];
      W.ke[d] = W.ke[f];
    }
  }
}

__device__ long long block_compact_flags(const unsigned char* flag, long long n, int* list) {
  __shared__ int wsum[kCTA / 32];
  __shared__ long long total;
  if (threadIdx.x == 0) total = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (long long b = 0; b < n; b += kCTA) {
    const long long i = b + threadIdx.x;
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

// The kills below the lower threshold (pyvibdmc.py:340-356, :432-439): for
// each kill-list slot to_j in order, the walker m_j of the largest weight
// (the first on ties, np.argmax) is cloned into to_j and both keep half its
// weight.  The argmax runs in one warp over per-chunk maxima kept in shared
// memory; after a kill only the chunks of m_j and to_j are scanned again, so
// a kill costs a few hundred cycles instead of a block-wide pass over all n
// weights.  The copies are deferred: aux[to_j] = m_j records where each
// killed slot takes its walker from, and afterwards every copy follows the
// chain aux[.] through slots killed earlier (flags 2) to an original walker,
// all kills in parallel.  The argmax can be a slot that is still waiting to
// be killed only when every other weight has fallen below the threshold; if
// that happens the copies run one kill at a time in kill order instead, the
// reference's order.  w: the weights (global); flags: 1 for kill slots
// (set to 2 as they are killed); the CTA's 1024 threads call it.
constexpr int kChunkLogMin = 6;  // chunks of at least 64 weights
constexpr int kMaxChunks = 2048;

template <int A, bool IS>
__device__ void fast_kills(const gbdmc_sim_t& S, gbdmc_walkers_t& W, int64_t base, double* wg, long long n,
                           const int* list, long long nk, int* aux, unsigned char* flags, double* ws, int ws_cap) {
  // The weights are non-negative and finite here, so their bit patterns as
  // signed 64-bit integers order like their values: the comparisons run on
  // the integer pipes (a warp-wide FP64 instruction costs tens of cycles on
  // this part's narrow FP64 pipe).
  __shared__ long long s_cv[kMaxChunks];  // chunk maxima: the weight's bits
  __shared__ int s_ci[kMaxChunks];
  __shared__ int s_patho;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const unsigned full = 0xffffffffu;
  // the weights in shared memory while the kills run, when they fit
  const bool in_smem = n <= ws_cap;
  double* w = in_smem ? ws : wg;
  if (in_smem) {
    for (long long i = threadIdx.x; i < n; i += kCTA) ws[i] = wg[i];
    __syncthreads();
  }
  // chunks of 2^lk weights (lk >= kChunkLogMin, at most kMaxChunks chunks): the
  // chunk of a slot is a shift, and the indices are 32-bit (n < 2^31).  A kill
  // reads about 2 ceil(chunks / 32) chunk maxima and ceil(2^lk / 32) weights
  // per lane; lk minimises their sum (the result does not depend on lk).
  int lk = kChunkLogMin;
  while ((n + (1LL << lk) - 1) >> lk > kMaxChunks) ++lk;
  {
    auto cost = [&](int l) {
      const long long ch = (n + (1LL << l) - 1) >> l;
      return 2 * ((ch + 31) >> 5) + (((1LL << l) + 31) >> 5);
    };
    for (int l = lk + 1; l < 20 && cost(l) < cost(lk); ++l) lk = l;
  }
  const int ni = (int)n;
  const int nch = (ni + (1 << lk) - 1) >> lk;
  // (key, index) of the largest weight, the first index on ties, over a warp:
  // the keys are non-negative, so the high words, then the low words of the
  // lanes that hold the largest high word, order them as unsigned integers
  constexpr int kNone = 0x7fffffff;  // a lane without a weight: key 0, last index
  auto warp_best = [&](long long& bk, int& bi) {
    const unsigned hi = (unsigned)((unsigned long long)bk >> 32), lo = (unsigned)bk;
    const unsigned mh = __reduce_max_sync(full, hi);
    const unsigned ml = __reduce_max_sync(full, hi == mh ? lo : 0u);
    bi = (int)__reduce_min_sync(full, (hi == mh && lo == ml) ? (unsigned)bi : (unsigned)kNone);
    bk = (long long)(((unsigned long long)mh << 32) | ml);
  };
  // per-chunk maxima of the current weights
  auto chunk_max = [&](int c, long long& bk, int& bi) {
    bk = 0;
    bi = kNone;
    const int e = ((c + 1) << lk) < ni ? ((c + 1) << lk) : ni;
    for (int i = (c << lk) + lane; i < e; i += 32) {
      const long long x = __double_as_longlong(w[i]);
      if (bi == kNone || x > bk) {
        bk = x;
        bi = i;
      }
    }
    warp_best(bk, bi);
  };
  if (threadIdx.x == 0) s_patho = 0;
  for (int c = wid; c < nch; c += kCTA / 32) {
    long long bk;
    int bi;
    chunk_max(c, bk, bi);
    if (lane == 0) {
      s_cv[c] = bk;
      s_ci[c] = bi;
    }
  }
  __syncthreads();
  if (wid == 0) {
    const long long thr_key = __double_as_longlong(S.thresh_lower);  // > 0: ordered like the weights
    int patho = 0;
    for (long long j0 = 0; j0 < nk; j0 += 32) {
      // lane q holds kill j0 + q: its slot, then the slot it is cloned from
      const int myto = j0 + lane < nk ? list[j0 + lane] : -1;
      const int cnt = nk - j0 < 32 ? (int)(nk - j0) : 32;
      int mym = 0;
      for (int q = 0; q < cnt; ++q) {
        const long long to = GBDMC_BC(__shfl_sync(full, myto, q), 0, n, kBcContSlot);
        long long bk = 0;
        int bi = kNone;
#pragma unroll 4
        for (int c = lane; c < nch; c += 32) {
          const long long x = s_cv[c];
          const int xi = s_ci[c];
          if (x > bk || (x == bk && xi < bi)) {
            bk = x;
            bi = xi;
          }
        }
        warp_best(bk, bi);
        const long long m = GBDMC_BC(bi, 0, n, kBcContSlot);
        // a slot still waiting to be killed can be the largest only when every
        // weight is below the threshold: then the copies keep the kill order
        if (bk < thr_key) patho = 1;
        const double h = __longlong_as_double(bk) * 0.5;  // w[m] halved (exact)
        const long long hk = __double_as_longlong(h);
        if (lane == q) mym = (int)m;
        if (lane == 0) {
          w[m] = h;
          w[to] = h;
        }
        __syncwarp();
        const int cm = (int)m >> lk, ct = (int)to >> lk;
        long long k1;
        int i1;
        chunk_max(cm, k1, i1);  // m's chunk lost its largest weight: scanned again
        if (lane == 0) {
          s_cv[cm] = k1;
          s_ci[cm] = i1;
        }
        if (ct != cm) {
          // to's chunk: only w[to] changed, so its largest is the old one or h
          // at to -- unless the old largest was to itself, whose weight may
          // have fallen (h can be below it when every weight is small): then
          // the chunk is scanned again
          const long long ck = s_cv[ct];
          const int ci = s_ci[ct];
          if (ci == (int)to) {
            chunk_max(ct, k1, i1);
            if (lane == 0) {
              s_cv[ct] = k1;
              s_ci[ct] = i1;
            }
          } else if (lane == 0 && (hk > ck || (hk == ck && (int)to < ci))) {
            s_cv[ct] = hk;
            s_ci[ct] = (int)to;
          }
        }
        __syncwarp();
      }
      if (lane < cnt) {  // the batch's sources and killed marks, once per 32 kills
        aux[myto] = mym;
        flags[myto] = 2;
      }
    }
    if (lane == 0) s_patho = patho;
  }
  __syncthreads();
  if (in_smem) {
    for (long long i = threadIdx.x; i < n; i += kCTA) wg[i] = ws[i];
    __syncthreads();
  }
  const int nat = A > 0 ? A : S.natoms;
  const int64_t ld = S.ld;
  if (!s_patho) {
    // every killed slot from the original walker at the end of its chain
    for (long long j = threadIdx.x; j < nk; j += kCTA) {
      const long long to = list[j];
      long long src = aux[to];
      while (flags[src] == 2) src = aux[src];
      const int64_t f = base + src, d = base + to;
      for (int k = 0; k < 3 * nat; ++k) {
        W.x[k * ld + d] = W.x[k * ld + f];
        if constexpr (IS) W.f[k * ld + d] = W.f[k * ld + f];
      }
      W.v[d] = W.v[f];
      if (W.who) W.who[d] = W.who[f];
      if constexpr (IS) {
        W.psi[d] = W.psi[f];
        W.ke[d] = W.ke[f];
      }
    }
  } else {
    // the reference's order, one kill at a time (a source may be killed later)
    for (long long j = 0; j < nk; ++j) {
      const long long to = list[j];
      clone_walker<A, IS>(S, W, base, aux[to], to);
      __syncthreads();
    }
  }
  __syncthreads();
}

template <int A, bool IS>
__global__ void __launch_bounds__(kCTA) k_cont_branch(const __grid_constant__ gbdmc_sim_t S,
                                                       const __grid_constant__ RepTable T, gbdmc_walkers_t W,
                                                       gbdmc_ctrl_t* ctrls, int* list_all, int* aux_all,
                                                       unsigned char* flags_all, int ws_cap, int weighted) {
  extern __shared__ double ws_dyn[];  // ws_cap doubles: the weights during the kills
  const int r = blockIdx.x;
  gbdmc_ctrl_t* ctrl = ctrls + r;
  if (*(volatile int*)&ctrl->status) return;
  const int64_t base = T.off[r];
  const long long n = ctrl->n;
  const long long step = ctrl->step;
  const double vref = ctrl->vref;
  const double dt = IS ? ctrl->dt_eff : S.dt;
  double* w = W.w + base;
  const double* v = W.v + base;
  int* list = list_all + base;
  unsigned char* flags = flags_all + base;
  __shared__ long long s_nb;
  int bad = 0, neg = 0;
  // the tests on the weight's bits (integer pipes): with a positive threshold,
  // wi < thresh_lower holds exactly when the signed 64-bit patterns compare so
  // for every finite wi (a negative wi has a negative pattern)
  const long long thr_key = __double_as_longlong(S.thresh_lower);
  const bool key_cmp = S.thresh_lower > 0.0;
  constexpr long long kExpMask = 0x7FF0000000000000LL;
  for (long long i = threadIdx.x; i < n; i += kCTA) {
    // weighted: the move kernel has applied this step's factor already
    double wi = w[i];
    if (!weighted) {
      wi *= exp(__dmul_rn(-__dsub_rn(v[i], vref), dt));
      w[i] = wi;
    }
    const long long k = __double_as_longlong(wi);
    if ((k & kExpMask) == kExpMask) bad = 1;  // inf or NaN
    if (k < 0) neg = 1;                         // the sign bit
    flags[i] = (key_cmp ? k < thr_key : wi < S.thresh_lower) ? 1 : 0;
  }
  const bool any_neg = __syncthreads_or(neg);
  if (__syncthreads_or(bad)) {
    if (threadIdx.x == 0) {
      ctrl->status |= GBDMC_ST_NONFINITE_WEIGHT;
      ctrl->err_step = (int)step;
    }
    return;
  }
  const long long nk = block_compact_flags(flags, n, list);
  long long nb = nk;
  if (nk > 0 && nk < n && !any_neg && S.thresh_lower > 0.0) {
    fast_kills<A, IS>(S, W, base, w, n, list, nk, aux_all + base, flags, ws_dyn, ws_cap);
  } else {
  for (long long j = 0; j < nk; ++j) {
    const long long to = GBDMC_BC(list[j], 0, n, kBcContSlot);
    const long long m = GBDMC_BC(block_arg<true>(w, n, nullptr), 0, n, kBcContSlot);
    clone_walker<A, IS>(S, W, base, m, to);
    __syncthreads();
    if (threadIdx.x == 0) {
      const double h = w[m] / 2.0;
      w[m] = h;
      w[to] = h;
    }
    __syncthreads();
  }
  }
  if (S.thresh_upper > 0.0) {
    if (threadIdx.x == 0) s_nb = 0;
    __syncthreads();
    long long cnt = 0;
    for (long long i = threadIdx.x; i < n; i += kCTA) cnt += w[i] > S.thresh_upper ? 1 : 0;
    cnt = warp_sum(cnt);
    if ((threadIdx.x & 31) == 0) atomicAdd((unsigned long long*)&s_nb, (unsigned long long)cnt);
    __syncthreads();
    const long long nup = s_nb;
    if (nup >= n && nup > 0) {  // np.argpartition raises: kth out of bounds
      if (threadIdx.x == 0) {
        ctrl->status |= GBDMC_ST_HUGE_WEIGHT;
        ctrl->err_step = (int)step;
      }
      return;
    }
    if (nup > 0 && !block_argpartition(w, list, n, nup, aux_all + base, flags)) {
      if (threadIdx.x == 0) {
        ctrl->status |= GBDMC_ST_OVERFLOW;
        ctrl->err_step = (int)step;
      }
      return;
    }
    const long long nk2 = nup;
    for (long long j = 0; j < nk2; ++j) {
      const long long to = GBDMC_BC(list[j], 0, n, kBcContSlot);
      const long long m = GBDMC_BC(block_arg<true>(w, n, nullptr), 0, n, kBcContSlot);
      clone_walker<A, IS>(S, W, base, m, to);
      __syncthreads();
      if (threadIdx.x == 0) {
        const double h = w[m] / 2.0;
        w[m] = h;
        w[to] = h;
      }
      __syncthreads();
    }
    nb += nk2;
  }
  double swv = 0.0, sw = 0.0, wmx = -CUDART_INF, wmn = CUDART_INF;
  if (!any_neg) {
    // non-negative weights order like their bit patterns: the extremes on the
    // integer pipes (the patterns of -inf and +inf start them)
    long long kmx = __double_as_longlong(-CUDART_INF), kmn = __double_as_longlong(CUDART_INF);
    for (long long i = threadIdx.x; i < n; i += kCTA) {
      const double wi = w[i];
      swv += v[i] * wi;
      sw += wi;
      const long long k = __double_as_longlong(wi);
      kmx = k > kmx ? k : kmx;
      kmn = k < kmn ? k : kmn;
    }
    wmx = __longlong_as_double(kmx);
    wmn = __longlong_as_double(kmn);
  } else {
    for (long long i = threadIdx.x; i < n; i += kCTA) {
      const double wi = w[i];
      swv += v[i] * wi;
      sw += wi;
      wmx = fmax(wmx, wi);
      wmn = fmin(wmn, wi);
    }
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
      const double n0 = (double)T.n0[r];
      const double vr = swv / sw - S.alpha * ((sw - n0) / n0);
      if (step < S.hist.len) {
        const int64_t h = hidx(S, r, step);
        if (S.hist.vref) S.hist.vref[h] = vr;
        if (S.hist.pop) S.hist.pop[h] = sw;
        if (S.hist.births) S.hist.births[h] = (int)nb;
      }
      ctrl->vref = vr;
      ctrl->n_prev = n;
      ctrl->step = step + 1;
      ctrl->reserved[0] = __double_as_longlong(wmx);
      ctrl->reserved[1] = __double_as_longlong(wmn);
    }
  }
}

// One CTA per replica; the weights of replicas of up to kWsMax walkers sit in
// shared memory while their kills run.
constexpr int kWsMax = 24000;
// weighted: the move kernel has multiplied this step's factor into the weights.
template <int A, bool IS>
static void launch_cont_branch(const gbdmc_sim_t& S, const RepTable& T, const gbdmc_walkers_t& dst,
                               gbdmc_ctrl_t* ctrl, int* list, int* aux, unsigned char* flags, bool weighted,
                               cudaStream_t s) {
  long long cap = 0;
  for (int r = 0; r < T.nrep; ++r) cap = T.cap[r] > cap ? T.cap[r] : cap;
  const int ws_cap = (int)(cap < kWsMax ? cap : kWsMax);
  const size_t smem = (size_t)ws_cap * sizeof(double);
  cudaFuncSetAttribute((const void*)k_cont_branch<A, IS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k_cont_branch<A, IS><<<T.nrep, kCTA, smem, s>>>(S, T, dst, ctrl, list, aux, flags, ws_cap, weighted ? 1 : 0);
}

// np.argpartition of one weight array by one CTA (gbdmc_argpartition).
__global__ void __launch_bounds__(kSelCTA) k_argpartition(const double* w, long long n, long long kth, int* perm,
                                                          int* lpos, unsigned char* fl) {
  if (!block_argpartition(w, perm, n, kth, lpos, fl) && threadIdx.x == 0) perm[0] = -1;
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

// ============================================================ host side
int num_sms() {
  static int cached[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 152;
  if (dev < 64 && cached[dev]) return cached[dev];
  int n = 0;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 152;
  if (dev < 64) cached[dev] = n;
  return n;
}

// Tile width: spread sum(n0) over all SMs in one wave (multiple of 32, 64..256).
static int pick_tpb(const gbdmc_sim_t& S, const gbdmc_replica_t* reps, int nrep) {
  if (S.block_threads) return S.block_threads;
  int64_t tot = 0;
  for (int r = 0; r < nrep; ++r) tot += reps[r].n0;
  const int64_t per_sm = (tot * 103 / 100 + num_sms() - 1) / num_sms();
  int t = (int)((per_sm + 31) / 32 * 32);
  return t < 64 ? 64 : (t > kMaxTPB ? kMaxTPB : t);
}

int build_table(const gbdmc_sim_t& S, const gbdmc_replica_t* reps, int nrep, RepTable& T, const char* what) {
  memset(&T, 0, sizeof(T));
  if (nrep < 1 || nrep > GBDMC_MAX_REPLICAS) {
    set_error("%s: nrep must be 1..%d (got %d)", what, GBDMC_MAX_REPLICAS, nrep);
    return GBDMC_ERR_CAPACITY;
  }
  const int tpb = pick_tpb(S, reps, nrep);
  if (tpb < kMinTPB || tpb > kMaxTPB || tpb % 32) {
    set_error("%s: block_threads must be a multiple of 32 in [32, 256] (got %d)", what, tpb);
    return GBDMC_ERR_ARG;
  }
  T.nrep = nrep;
  T.tpb = tpb;
  int64_t tiles = 0;
  for (int r = 0; r < nrep; ++r) {
    const gbdmc_replica_t& R = reps[r];
    if (R.off < 0 || R.cap < 1 || R.off + R.cap > S.ld || R.n0 < 1) {
      set_error("%s: replica %d has bad off/cap/n0 (%lld/%lld/%lld, ld %lld)", what, r, (long long)R.off,
                (long long)R.cap, (long long)R.n0, (long long)S.ld);
      return GBDMC_ERR_ARG;
    }
    for (int q = 0; q < r; ++q) {  // replicas own disjoint slot ranges (their kernels write them concurrently)
      if (R.off < reps[q].off + reps[q].cap && reps[q].off < R.off + R.cap) {
        set_error("%s: replicas %d and %d overlap", what, q, r);
        return GBDMC_ERR_ARG;
      }
    }
    T.tile_off[r] = (int32_t)tiles;
    T.off[r] = R.off;
    T.cap[r] = R.cap;
    T.n0[r] = R.n0;
    T.stream[r] = R.stream;
    const double d0 = (double)R.n0, w_hi = (d0 + d0 * 0.5) + 1.0;
    float wf = (float)w_hi;
    if ((double)wf > w_hi) wf = std::nextafter(wf, -INFINITY);
    T.w_hi_f[r] = wf;
    tiles += (R.cap + tpb - 1) / tpb;
    if (tiles > INT32_MAX / 2) {
      set_error("%s: too many tiles", what);
      return GBDMC_ERR_CAPACITY;
    }
  }
  T.tile_off[nrep] = (int32_t)tiles;
  return GBDMC_OK;
}

int grid_for(const RepTable& T) {
  const int tiles = T.tile_off[T.nrep];
  const int resident = num_sms() * (2048 / T.tpb);
  return tiles < resident ? tiles : resident;
}

void launch_branch(const RepTable& T, int32_t* idx, const gbdmc_ctrl_t* ctrl, const long long* prefix,
                   const int* counts, cudaStream_t s) {
  const TileBatch tb = tile_batch(T);
  if (tb.tpi == 4)
    launch_pdl(k_branch<4>, tb.grid, T.tpb, s, T, idx, ctrl, prefix, counts);
  else
    launch_pdl(k_branch<1>, tb.grid, T.tpb, s, T, idx, ctrl, prefix, counts);
}

template <int PK, int A, int TK>
static int run_init(const gbdmc_sim_t& S, const RepTable& T, const gbdmc_walkers_t& W, gbdmc_ctrl_t* ctrl,
                    const ScratchLayout& L, cudaStream_t s) {
  k_init<PK, A, TK><<<grid_for(T), T.tpb, 0, s>>>(S, T, W, ctrl, L.part);
  return check_launch("gbdmc init");
}

// Where a discrete branching pass puts its result: the gather index of dst
// (out == nullptr) or compact walkers in `out` plus a copy of the control
// block in `ctrl_out` (the host-resident step).
struct BranchTarget {
  const gbdmc_walkers_t* out;
  gbdmc_ctrl_t* ctrl_out;
};

template <int A, bool IS>
static void launch_branch_to(const RepTable& T, const gbdmc_sim_t& S, const gbdmc_walkers_t& dst, gbdmc_ctrl_t* ctrl,
                             const ScratchLayout& L, const BranchTarget& bt, cudaStream_t s) {
  if (bt.out)
    launch_pdl(k_branch_scatter<A, IS>, grid_for(T), T.tpb, s, T, S.ld, dst, *bt.out, ctrl, L.prefix, L.counts,
               bt.ctrl_out);
  else
    launch_branch(T, dst.idx, ctrl, L.prefix, L.counts, s);
}

template <int PK, int A, int TK, int NM, bool STATS>
static void launch_step(const gbdmc_sim_t& S, const RepTable& T, const gbdmc_walkers_t& src,
                        const gbdmc_walkers_t& dst, gbdmc_ctrl_t* ctrl, const ScratchLayout& L,
                        const gbdmc_noise_t& nz, const BranchTarget& bt, cudaStream_t s) {
  const int G = grid_for(T);
  constexpr bool IS = TK != GBDMC_TRIAL_NONE;
  const bool prof = g_prof.on && g_prof.count < ProfState::kSlots;
  cudaEvent_t* ev = prof ? g_prof.ev[g_prof.count] : nullptr;
  if (prof) cudaEventRecord(ev[0], s);
  if constexpr (!IS) {
    if (S.weighting == GBDMC_DISCRETE) {
      // k_move is launched in stream order (its CTAs then spread one per SM, which
      // its fp64 pipes need); k_branch may be launched while k_move finishes
      k_move<PK, A, NM, true, STATS><<<G, T.tpb, 0, s>>>(S, T, src, dst, ctrl, L.part, L.prefix, L.counts, nz);
      if (prof) cudaEventRecord(ev[1], s);
      launch_branch_to<A, false>(T, S, dst, ctrl, L, bt, s);
    } else {
      k_move<PK, A, NM, false, STATS><<<G, T.tpb, 0, s>>>(S, T, src, dst, ctrl, L.part, L.prefix, L.counts, nz);
      if (prof) cudaEventRecord(ev[1], s);
      launch_cont_branch<A, false>(S, T, dst, ctrl, L.list, L.counts, L.flags, true, s);
    }
  } else {
    k_is_move<PK, A, TK, NM, STATS><<<G, T.tpb, 0, s>>>(S, T, src, dst, ctrl, L.part, nz);
    if (prof) cudaEventRecord(ev[1], s);
    if (S.weighting == GBDMC_DISCRETE) {
      k_count<NM, true><<<G, T.tpb, 0, s>>>(S, T, dst.v, ctrl, L.part, L.counts, nz);
      k_count_finalize<<<T.nrep, kMaxTPB, 0, s>>>(S, T, ctrl, L.part, L.prefix);
      launch_branch_to<A, true>(T, S, dst, ctrl, L, bt, s);
    } else {
      launch_cont_branch<A, true>(S, T, dst, ctrl, L.list, L.counts, L.flags, false, s);
    }
  }
  if (prof) {
    cudaEventRecord(ev[2], s);
    ++g_prof.count;
  }
}

template <int PK, int A, int TK>
static int run_step(const gbdmc_sim_t& S, const RepTable& T, const gbdmc_walkers_t& src, const gbdmc_walkers_t& dst,
                    gbdmc_ctrl_t* ctrl, const ScratchLayout& L, const gbdmc_noise_t& nz, const BranchTarget& bt,
                    cudaStream_t s) {
  const bool stats = S.hist.vmin || S.hist.vmax || S.hist.vmean;
#define GBDMC_NM(nm)                                                         \
  if (S.noise_mode == nm) {                                                  \
    if (stats)                                                               \
      launch_step<PK, A, TK, nm, true>(S, T, src, dst, ctrl, L, nz, bt, s);  \
    else                                                                     \
      launch_step<PK, A, TK, nm, false>(S, T, src, dst, ctrl, L, nz, bt, s); \
    return check_launch("gbdmc step");                                       \
  }
  GBDMC_NM(GBDMC_NOISE_PHILOX32)
  GBDMC_NM(GBDMC_NOISE_PHILOX64)
  GBDMC_NM(GBDMC_NOISE_INJECTED)
#undef GBDMC_NM
  set_error("gbdmc step: unknown noise mode %d", S.noise_mode);
  return GBDMC_ERR_ARG;
}

template <int A>
static int run_compact(const gbdmc_sim_t& S, const RepTable& T, const gbdmc_walkers_t& in,
                       const gbdmc_walkers_t& out, const gbdmc_ctrl_t* ctrl, cudaStream_t s) {
  if (in.f && out.f)
    k_compact<A, true><<<grid_for(T), T.tpb, 0, s>>>(S, T, in, out, ctrl);
  else
    k_compact<A, false><<<grid_for(T), T.tpb, 0, s>>>(S, T, in, out, ctrl);
  return check_launch("gbdmc_walkers_compact");
}

struct InitF {
  const gbdmc_sim_t& S;
  const RepTable& T;
  const gbdmc_walkers_t& W;
  gbdmc_ctrl_t* ctrl;
  const ScratchLayout& L;
  cudaStream_t s;
  template <int PK, int A, int TK>
  int operator()() {
    return run_init<PK, A, TK>(S, T, W, ctrl, L, s);
  }
};

struct StepF {
  const gbdmc_sim_t& S;
  const RepTable& T;
  const gbdmc_walkers_t& src;
  const gbdmc_walkers_t& dst;
  gbdmc_ctrl_t* ctrl;
  const ScratchLayout& L;
  const gbdmc_noise_t& nz;
  const BranchTarget& bt;
  cudaStream_t s;
  template <int PK, int A, int TK>
  int operator()() {
    return run_step<PK, A, TK>(S, T, src, dst, ctrl, L, nz, bt, s);
  }
};

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
  GBDMC_SYS(GBDMC_PES_H2O_PS, 3, GBDMC_TRIAL_NONE)
  GBDMC_SYS(GBDMC_PES_H2O_PS, 3, GBDMC_TRIAL_H2O_GAUSS)
  GBDMC_SYS(GBDMC_PES_HO, 1, GBDMC_TRIAL_HO_GAUSS)
  GBDMC_SYS(GBDMC_PES_HO, 3, GBDMC_TRIAL_HO_GAUSS)
  GBDMC_SYS(GBDMC_PES_H2O_LM, 3, GBDMC_TRIAL_H2O_GAUSS)
  GBDMC_SYS(GBDMC_PES_DIMER, 6, GBDMC_TRIAL_DIMER_GAUSS)
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
  if (S->natoms < 1 || S->natoms > GBDMC_MAX_ATOMS || S->ld < 1) {
    set_error("%s: bad sizes (natoms=%d ld=%lld)", what, S->natoms, (long long)S->ld);
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

static int step_common(const gbdmc_sim_t* S, const gbdmc_replica_t* reps, int nrep, const gbdmc_walkers_t* src,
                       const gbdmc_walkers_t* dst, gbdmc_ctrl_t* ctrl, void* scratch, const gbdmc_noise_t* noise,
                       void* stream, const char* what, const BranchTarget& bt = BranchTarget{nullptr, nullptr}) {
  int rc = validate(S, src, ctrl, scratch, what);
  if (rc) return rc;
  rc = validate(S, dst, ctrl, scratch, what);
  if (rc) return rc;
  if (src->x == dst->x || src->v == dst->v || (src->who && src->who == dst->who)) {
    set_error("%s: src and dst must use different arrays", what);
    return GBDMC_ERR_ARG;
  }
  if (S->weighting == GBDMC_DISCRETE && !dst->idx && !bt.out) {
    set_error("%s: discrete weighting writes the branch index: dst->idx is required", what);
    return GBDMC_ERR_ARG;
  }
  if (S->weighting == GBDMC_CONTINUOUS && (dst->idx || src->idx)) {
    set_error("%s: continuous weighting works on compact walkers (idx must be NULL)", what);
    return GBDMC_ERR_ARG;
  }
  gbdmc_noise_t nz{};
  if (S->noise_mode == GBDMC_NOISE_INJECTED) {
    if (!noise || !noise->normal || (S->weighting == GBDMC_DISCRETE && !noise->u_branch) ||
        (S->trial.kind != GBDMC_TRIAL_NONE && !noise->u_accept) || noise->ld_noise < 1) {
      set_error("%s: injected noise buffers missing", what);
      return GBDMC_ERR_ARG;
    }
    nz = *noise;
  }
  RepTable T;
  rc = build_table(*S, reps, nrep, T, what);
  if (rc) return rc;
  const ScratchLayout L = scratch_layout(scratch, slot_extent(S->ld, reps, nrep), max_tiles_for(reps, nrep));
  StepF f{*S, T, *src, *dst, ctrl, L, nz, bt, (cudaStream_t)stream};
  return dispatch_system(*S, what, f);
}

// Layout of a caller-evaluated potential's walkers (GBDMC_PES_EXTERNAL).
static int ext_layout(const gbdmc_sim_t* S, const char* what, int& nc, int& d) {
  nc = ext_coords(*S);
  d = ext_dims(*S);
  if (S->trial.kind != GBDMC_TRIAL_NONE) {
    set_error("%s: a caller-evaluated potential runs plain DMC (trial kind must be GBDMC_TRIAL_NONE)", what);
    return GBDMC_ERR_ARG;
  }
  if (d < 1 || d > 3 || nc < 1 || nc > 3 * S->natoms || nc % d || nc / d > GBDMC_MAX_ATOMS) {
    set_error("%s: bad walker layout (nc=%d coordinates, d=%d per atom, %d storage atoms)", what, nc, d,
              S->natoms);
    return GBDMC_ERR_ARG;
  }
  return GBDMC_OK;
}

static int init_common(const gbdmc_sim_t* S, const gbdmc_replica_t* reps, int nrep, const gbdmc_walkers_t* W,
                       gbdmc_ctrl_t* ctrl, void* scratch, void* stream, const char* what) {
  int rc = validate(S, W, ctrl, scratch, what);
  if (rc) return rc;
  RepTable T;
  rc = build_table(*S, reps, nrep, T, what);
  if (rc) return rc;
  const ScratchLayout L = scratch_layout(scratch, slot_extent(S->ld, reps, nrep), max_tiles_for(reps, nrep));
  if (S->pes.kind == GBDMC_PES_EXTERNAL) {  // V of the start walkers is the caller's (W->v)
    int nc, d;
    rc = ext_layout(S, what, nc, d);
    if (rc) return rc;
    return run_init<GBDMC_PES_EXTERNAL, 1, GBDMC_TRIAL_NONE>(*S, T, *W, ctrl, L, (cudaStream_t)stream);
  }
  InitF f{*S, T, *W, ctrl, L, (cudaStream_t)stream};
  return dispatch_system(*S, what, f);
}

static gbdmc_replica_t single_replica(const gbdmc_sim_t* S) {
  gbdmc_replica_t r{};
  r.off = 0;
  r.cap = S->ld;
  r.n0 = S->n0;
  r.stream = S->replica_id;
  return r;
}

}  // namespace gbdmc

using namespace gbdmc;

extern "C" size_t gbdmc_scratch_bytes(int64_t ld) {
  if (ld <= 0) return 0;
  return scratch_layout(nullptr, ld, (ld + kMinTPB - 1) / kMinTPB).bytes;
}

extern "C" size_t gbdmc_batch_scratch_bytes(const gbdmc_replica_t* reps, int32_t nrep) {
  if (!reps || nrep < 1) return 0;
  return scratch_layout(nullptr, slot_extent(0, reps, nrep), max_tiles_for(reps, nrep)).bytes;
}

extern "C" int gbdmc_sim_init(const gbdmc_sim_t* S, const gbdmc_walkers_t* W, gbdmc_ctrl_t* ctrl, void* scratch,
                              void* stream) {
  if (!S) {
    set_error("gbdmc_sim_init: null sim");
    return GBDMC_ERR_ARG;
  }
  if (S->n0 < 1) {
    set_error("gbdmc_sim_init: n0 must be >= 1");
    return GBDMC_ERR_ARG;
  }
  const gbdmc_replica_t r = single_replica(S);
  return init_common(S, &r, 1, W, ctrl, scratch, stream, "gbdmc_sim_init");
}

extern "C" int gbdmc_sim_step(const gbdmc_sim_t* S, const gbdmc_walkers_t* src, const gbdmc_walkers_t* dst,
                              gbdmc_ctrl_t* ctrl, void* scratch, const gbdmc_noise_t* noise, void* stream) {
  if (!S || !dst) {
    set_error("gbdmc_sim_step: null argument");
    return GBDMC_ERR_ARG;
  }
  if (S->n0 < 1) {
    set_error("gbdmc_sim_step: n0 must be >= 1");
    return GBDMC_ERR_ARG;
  }
  const gbdmc_replica_t r = single_replica(S);
  return step_common(S, &r, 1, src, dst, ctrl, scratch, noise, stream, "gbdmc_sim_step");
}

extern "C" int gbdmc_sim_move(const gbdmc_sim_t* S, const gbdmc_walkers_t* src, const gbdmc_walkers_t* dst,
                              gbdmc_ctrl_t* ctrl, void* scratch, const gbdmc_noise_t* noise, void* stream) {
  const char* what = "gbdmc_sim_move";
  int rc = validate(S, src, ctrl, scratch, what);
  if (rc) return rc;
  rc = validate(S, dst, ctrl, scratch, what);
  if (rc) return rc;
  if (src->x == dst->x || src->v == dst->v || (src->who && src->who == dst->who)) {
    set_error("%s: src and dst must use different arrays", what);
    return GBDMC_ERR_ARG;
  }
  if (S->weighting == GBDMC_CONTINUOUS && (dst->idx || src->idx)) {
    set_error("%s: continuous weighting works on compact walkers (idx must be NULL)", what);
    return GBDMC_ERR_ARG;
  }
  int nc, d;
  rc = ext_layout(S, what, nc, d);
  if (rc) return rc;
  gbdmc_noise_t nz{};
  if (S->noise_mode == GBDMC_NOISE_INJECTED) {
    if (!noise || !noise->normal || noise->ld_noise < 1) {
      set_error("%s: injected noise buffers missing", what);
      return GBDMC_ERR_ARG;
    }
    nz = *noise;
  }
  const gbdmc_replica_t r = single_replica(S);
  RepTable T;
  rc = build_table(*S, &r, 1, T, what);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  switch (S->noise_mode) {
    case GBDMC_NOISE_PHILOX32:
      k_move_ext<GBDMC_NOISE_PHILOX32><<<grid_for(T), T.tpb, 0, s>>>(*S, T, *src, *dst, ctrl, nc, d, nz);
      break;
    case GBDMC_NOISE_PHILOX64:
      k_move_ext<GBDMC_NOISE_PHILOX64><<<grid_for(T), T.tpb, 0, s>>>(*S, T, *src, *dst, ctrl, nc, d, nz);
      break;
    case GBDMC_NOISE_INJECTED:
      k_move_ext<GBDMC_NOISE_INJECTED><<<grid_for(T), T.tpb, 0, s>>>(*S, T, *src, *dst, ctrl, nc, d, nz);
      break;
    default:
      set_error("%s: unknown noise mode %d", what, S->noise_mode);
      return GBDMC_ERR_ARG;
  }
  return check_launch(what);
}

extern "C" int gbdmc_sim_branch(const gbdmc_sim_t* S, const gbdmc_walkers_t* dst, gbdmc_ctrl_t* ctrl, void* scratch,
                                const gbdmc_noise_t* noise, void* stream) {
  const char* what = "gbdmc_sim_branch";
  int rc = validate(S, dst, ctrl, scratch, what);
  if (rc) return rc;
  if (S->weighting == GBDMC_DISCRETE && !dst->idx) {
    set_error("%s: discrete weighting writes the branch index: dst->idx is required", what);
    return GBDMC_ERR_ARG;
  }
  if (S->weighting == GBDMC_CONTINUOUS && dst->idx) {
    set_error("%s: continuous weighting works on compact walkers (idx must be NULL)", what);
    return GBDMC_ERR_ARG;
  }
  int nc, d;
  rc = ext_layout(S, what, nc, d);
  if (rc) return rc;
  gbdmc_noise_t nz{};
  if (S->noise_mode == GBDMC_NOISE_INJECTED && S->weighting == GBDMC_DISCRETE) {
    if (!noise || !noise->u_branch) {
      set_error("%s: injected branching uniforms missing", what);
      return GBDMC_ERR_ARG;
    }
    nz = *noise;
  }
  const gbdmc_replica_t r = single_replica(S);
  RepTable T;
  rc = build_table(*S, &r, 1, T, what);
  if (rc) return rc;
  const ScratchLayout L = scratch_layout(scratch, S->ld, max_tiles_for(&r, 1));
  cudaStream_t s = (cudaStream_t)stream;
  if (S->weighting == GBDMC_CONTINUOUS) {
    launch_cont_branch<0, false>(*S, T, *dst, ctrl, L.list, L.counts, L.flags, false, s);
    return check_launch(what);
  }
  const int G = grid_for(T);
  switch (S->noise_mode) {
    case GBDMC_NOISE_PHILOX32:
      k_count<GBDMC_NOISE_PHILOX32, false><<<G, T.tpb, 0, s>>>(*S, T, dst->v, ctrl, L.part, L.counts, nz);
      break;
    case GBDMC_NOISE_PHILOX64:
      k_count<GBDMC_NOISE_PHILOX64, false><<<G, T.tpb, 0, s>>>(*S, T, dst->v, ctrl, L.part, L.counts, nz);
      break;
    case GBDMC_NOISE_INJECTED:
      k_count<GBDMC_NOISE_INJECTED, false><<<G, T.tpb, 0, s>>>(*S, T, dst->v, ctrl, L.part, L.counts, nz);
      break;
    default:
      set_error("%s: unknown noise mode %d", what, S->noise_mode);
      return GBDMC_ERR_ARG;
  }
  k_count_finalize<<<1, kMaxTPB, 0, s>>>(*S, T, ctrl, L.part, L.prefix);
  launch_branch(T, dst->idx, ctrl, L.prefix, L.counts, s);
  return check_launch(what);
}

extern "C" int gbdmc_batch_init(const gbdmc_sim_t* S, const gbdmc_replica_t* reps, int32_t nrep,
                                const gbdmc_walkers_t* W, gbdmc_ctrl_t* ctrl, void* scratch, void* stream) {
  if (!reps) {
    set_error("gbdmc_batch_init: null replica table");
    return GBDMC_ERR_ARG;
  }
  return init_common(S, reps, nrep, W, ctrl, scratch, stream, "gbdmc_batch_init");
}

extern "C" int gbdmc_batch_step(const gbdmc_sim_t* S, const gbdmc_replica_t* reps, int32_t nrep,
                                const gbdmc_walkers_t* src, const gbdmc_walkers_t* dst, gbdmc_ctrl_t* ctrl,
                                void* scratch, const gbdmc_noise_t* noise, void* stream) {
  if (!reps || !dst) {
    set_error("gbdmc_batch_step: null argument");
    return GBDMC_ERR_ARG;
  }
  return step_common(S, reps, nrep, src, dst, ctrl, scratch, noise, stream, "gbdmc_batch_step");
}

extern "C" int gbdmc_walkers_compact(const gbdmc_sim_t* S, const gbdmc_replica_t* reps, int32_t nrep,
                                     const gbdmc_walkers_t* in, const gbdmc_walkers_t* out,
                                     const gbdmc_ctrl_t* ctrl, void* stream) {
  if (!S || !in || !out || !ctrl || !in->x || !in->v || !out->x || !out->v || in->x == out->x) {
    set_error("gbdmc_walkers_compact: invalid arguments");
    return GBDMC_ERR_ARG;
  }
  gbdmc_replica_t one;
  if (nrep == 0) {
    one = single_replica(S);
    one.n0 = S->n0 > 0 ? S->n0 : 1;
    reps = &one;
    nrep = 1;
  }
  RepTable T;
  int rc = build_table(*S, reps, nrep, T, "gbdmc_walkers_compact");
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  switch (S->natoms) {
    case 1: return run_compact<1>(*S, T, *in, *out, ctrl, s);
    case 2: return run_compact<2>(*S, T, *in, *out, ctrl, s);
    case 3: return run_compact<3>(*S, T, *in, *out, ctrl, s);
    case 4: return run_compact<4>(*S, T, *in, *out, ctrl, s);
    case 5: return run_compact<5>(*S, T, *in, *out, ctrl, s);
    case 6: return run_compact<6>(*S, T, *in, *out, ctrl, s);
    case 7: return run_compact<7>(*S, T, *in, *out, ctrl, s);
    case 8: return run_compact<8>(*S, T, *in, *out, ctrl, s);
  }
  set_error("gbdmc_walkers_compact: unsupported natoms %d", S->natoms);
  return GBDMC_ERR_ARG;
}

// Device alias of a page-locked host pointer (NULL stays NULL); false when p
// is not host memory the device can address.
static bool host_alias(const void* p, void** d) {
  *d = nullptr;
  if (!p) return true;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    (void)cudaGetLastError();
    return false;
  }
  if (a.type != cudaMemoryTypeHost || !a.devicePointer) return false;
  *d = a.devicePointer;
  return true;
}

extern "C" int gbdmc_sim_step_host(const gbdmc_sim_t* S, const gbdmc_walkers_t* host, const gbdmc_walkers_t* work,
                                   gbdmc_ctrl_t* ctrl, gbdmc_ctrl_t* ctrl_host, void* scratch,
                                   const gbdmc_noise_t* noise, void* stream) {
  if (!S || !host || !work || !ctrl || !ctrl_host || !host->x || !host->v || host->idx || !work->x || !work->v) {
    set_error("gbdmc_sim_step_host: invalid arguments (host walkers need x and v and no idx)");
    return GBDMC_ERR_ARG;
  }
  gbdmc_walkers_t h = {};
  void* d[7];
  const void* hp[7] = {host->x, host->v, host->who, host->f, host->psi, host->ke, host->w};
  for (int k = 0; k < 7; ++k) {
    if (!host_alias(hp[k], &d[k])) {
      set_error("gbdmc_sim_step_host: host walker array %d is not page-locked host memory", k);
      return GBDMC_ERR_ARG;
    }
  }
  h.x = (double*)d[0];
  h.v = (double*)d[1];
  h.who = (int32_t*)d[2];
  h.f = (double*)d[3];
  h.psi = (double*)d[4];
  h.ke = (double*)d[5];
  h.w = (double*)d[6];
  if (S->weighting == GBDMC_DISCRETE) {
    // the branching pass writes the branched walkers and the control block straight into host memory
    void* ch;
    if (!host_alias(ctrl_host, &ch)) {
      set_error("gbdmc_sim_step_host: ctrl_host is not page-locked host memory");
      return GBDMC_ERR_ARG;
    }
    if (S->n0 < 1) {
      set_error("gbdmc_sim_step_host: n0 must be >= 1");
      return GBDMC_ERR_ARG;
    }
    const gbdmc_replica_t r = single_replica(S);
    return step_common(S, &r, 1, &h, work, ctrl, scratch, noise, stream, "gbdmc_sim_step_host",
                       BranchTarget{&h, (gbdmc_ctrl_t*)ch});
  }
  int rc = gbdmc_sim_step(S, &h, work, ctrl, scratch, noise, stream);
  if (rc) return rc;
  rc = gbdmc_walkers_compact(S, nullptr, 0, work, &h, ctrl, stream);
  if (rc) return rc;
  if (cudaMemcpyAsync(ctrl_host, ctrl, sizeof(gbdmc_ctrl_t), cudaMemcpyDeviceToHost, (cudaStream_t)stream) !=
      cudaSuccess)
    return check_launch("gbdmc_sim_step_host: control block copy");
  return GBDMC_OK;
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
  k_desc<<<2 * num_sms(), 256, 0, s>>>(who, w, n_dev, n_parent, desc);
  return check_launch("gbdmc_desc_weights");
}

extern "C" int gbdmc_argpartition(const double* w, int64_t n, int64_t kth, int32_t* perm, int32_t* lpos,
                                  uint8_t* flags, void* stream) {
  if (!w || !perm || !lpos || !flags || n < 1 || n > (int64_t)INT32_MAX || kth < 0 || kth >= n) {
    set_error("gbdmc_argpartition: need 0 <= kth < n <= 2^31-1 and non-null buffers (n=%lld kth=%lld)",
              (long long)n, (long long)kth);
    return GBDMC_ERR_ARG;
  }
  k_argpartition<<<1, kSelCTA, 0, (cudaStream_t)stream>>>(w, n, kth, perm, lpos, flags);
  return check_launch("gbdmc_argpartition");
}

extern "C" int gbdmc_desc_begin(int32_t* who, const int64_t* n_dev, void* stream) {
  if (!who || !n_dev) {
    set_error("gbdmc_desc_begin: invalid arguments");
    return GBDMC_ERR_ARG;
  }
  k_iota<<<2 * num_sms(), 256, 0, (cudaStream_t)stream>>>(who, n_dev);
  return check_launch("gbdmc_desc_begin");
}

// ------------------------------------------------ allocation-free variant
// Step scratch for callers that cannot allocate device memory.  The array
// lives in the library's own device image: every GPU that loads libgbdmc.so
// holds these bytes until the process exits, and every call shares them.
#define GBDMC_STATIC_SCRATCH_BYTES (1u << 20)
static __device__ __align__(256) unsigned char g_static_scratch[GBDMC_STATIC_SCRATCH_BYTES];

namespace gbdmc {
// Device address of g_static_scratch, looked up once per device.
static void* g_static_scratch_ptr[64] = {nullptr};
static std::mutex g_static_scratch_mu;

static int static_scratch_ptr(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= 64) {
    set_error("gbdmc_sim_step_static: cudaGetDevice: %s", e != cudaSuccess ? cudaGetErrorString(e) : "device id >= 64");
    return GBDMC_ERR_CUDA;
  }
  std::lock_guard<std::mutex> lock(g_static_scratch_mu);
  if (!g_static_scratch_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess || !p) {
      set_error("gbdmc_sim_step_static: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
      return GBDMC_ERR_CUDA;
    }
    g_static_scratch_ptr[dev] = p;
  }
  *out = g_static_scratch_ptr[dev];
  return GBDMC_OK;
}
GBDMC_BOUNDS_READER(bounds_read_step)
}  // namespace gbdmc

extern "C" size_t gbdmc_sim_step_static_max_ld(void) {
  // largest capacity whose step scratch fits the static array
  int64_t lo = 1, hi = (int64_t)GBDMC_STATIC_SCRATCH_BYTES;
  while (lo < hi) {
    const int64_t mid = (lo + hi + 1) / 2;
    if (gbdmc_scratch_bytes(mid) <= GBDMC_STATIC_SCRATCH_BYTES) lo = mid; else hi = mid - 1;
  }
  return (size_t)lo;
}

extern "C" int gbdmc_sim_step_static(const gbdmc_sim_t* S, const gbdmc_walkers_t* src, const gbdmc_walkers_t* dst,
                                     gbdmc_ctrl_t* ctrl, const gbdmc_noise_t* noise, void* stream) {
  if (!S || !dst) {
    set_error("gbdmc_sim_step_static: null argument");
    return GBDMC_ERR_ARG;
  }
  if (S->n0 < 1) {
    set_error("gbdmc_sim_step_static: n0 must be >= 1");
    return GBDMC_ERR_ARG;
  }
  if (S->ld < 1 || gbdmc_scratch_bytes(S->ld) > GBDMC_STATIC_SCRATCH_BYTES) {
    set_error("gbdmc_sim_step_static: ld %lld needs %zu scratch bytes; the static scratch holds %u (ld <= %zu)",
              (long long)S->ld, gbdmc_scratch_bytes(S->ld), GBDMC_STATIC_SCRATCH_BYTES,
              gbdmc_sim_step_static_max_ld());
    return GBDMC_ERR_CAPACITY;
  }
  void* scratch = nullptr;
  const int rc = static_scratch_ptr(&scratch);
  if (rc) return rc;
  const gbdmc_replica_t r = single_replica(S);
  return step_common(S, &r, 1, src, dst, ctrl, scratch, noise, stream, "gbdmc_sim_step_static");
}
