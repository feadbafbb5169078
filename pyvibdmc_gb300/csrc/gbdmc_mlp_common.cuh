// Device helpers shared by the surrogate kernels (mma.sync and tcgen05 paths).
#pragma once
#include <cuda_bf16.h>
#include "gbdmc_stepcore.cuh"

namespace gbdmc {

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&v);
}

// SiLU through the single-instruction tanh.approx.f32 (|error| ~ 1e-3
// relative, below the bf16 rounding of the activations):
//   silu(z) = z (1 + tanh(z/2)) / 2 = h + h tanh(h),  h = z/2.
// silu_half takes h; the tcgen05 path pre-scales its hidden-layer weights and
// biases by 1/2 (exact in bf16 / fp32), so its accumulator already holds h.
__device__ __forceinline__ float tanh_approx(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float sigmoidf_(float z) { return fmaf(0.5f, tanh_approx(0.5f * z), 0.5f); }
__device__ __forceinline__ float silu_half(float h) { return fmaf(h, tanh_approx(h), h); }
__device__ __forceinline__ float silu(float z) { return silu_half(0.5f * z); }

// fp32 copies of the step parameters that the surrogate kernels use,
// converted once on the host (round to nearest, the device conversion), so
// that the per-walker code issues no fp64 conversion.
struct StepF32 {
  float sigma[6];     // sqrt(dt / m_a)
  float inv_mass[6];  // 1 / m_a
  float h[6];         // 1 / (2 sigma_a^2), fp32 arithmetic on the fp32 sigma
  float dt;
  float trial[8];     // dimer trial parameters (gbdmc_trial_t.p[0..7])
  float pes[10];      // dimer PES parameters (gbdmc_pes_t.p[0..9])
};

inline StepF32 step_f32(const gbdmc_sim_t& S) {
  StepF32 P{};
  for (int a = 0; a < 6; ++a) {
    P.sigma[a] = (float)S.sigma[a];
    P.inv_mass[a] = (float)S.inv_mass[a];
    const float sg = P.sigma[a];
    P.h[a] = 0.5f / (sg * sg);
  }
  P.dt = (float)S.dt;
  for (int k = 0; k < 8; ++k) P.trial[k] = (float)S.trial.p[k];
  for (int k = 0; k < 10; ++k) P.pes[k] = (float)S.pes.p[k];
  return P;
}

// fp32 copies of the replica's vref and dt_eff for the surrogate counting
// pass (k_count_branch_f32), kept in ctrl->reserved[3]: written by the step's first
// kernel from the replica's first tile (vref as of the step's start; dt_eff
// is rewritten by the audit when a trial changes it).
__device__ __forceinline__ float2* count_params(gbdmc_ctrl_t* ctrl) {
  return reinterpret_cast<float2*>(&ctrl->reserved[3]);
}
__device__ __forceinline__ void store_count_params(gbdmc_ctrl_t* ctrl) {
  *count_params(ctrl) = make_float2((float)ctrl->vref, (float)ctrl->dt_eff);
}

// The dimer trial in fp32 for the surrogate move: ln psi at x (without the
// normalisation), the drift d1 = d ln psi/dx, and the mass-weighted
// Laplacian sum lap = sum_k (1/m_k) (d2 psi/dx_k^2)/psi, so that the local
// kinetic energy is -lap/2 (imp_samp.py:49-53) -- the terms of
// dimer_trial_log, with the second derivatives summed as they are produced
// instead of kept per Cartesian component (18 fewer live registers).
__device__ __forceinline__ void h2o_trial_f32(const float (&x)[18], const float* p, int o, float imo, float imh1,
                                              float imh2, float (&f)[18], float& lnpsi, float& tsum) {
  const float a1 = p[0], a2 = p[1], ath = p[2], r1e = p[3], r2e = p[4], the = p[5];
  const int h1 = o + 1, h2 = o + 2;
  float v1[3], v2[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    v1[d] = x[3 * h1 + d] - x[3 * o + d];
    v2[d] = x[3 * h2 + d] - x[3 * o + d];
  }
  const float r1 = sqrtf(v1[0] * v1[0] + v1[1] * v1[1] + v1[2] * v1[2]);
  const float r2 = sqrtf(v2[0] * v2[0] + v2[1] * v2[1] + v2[2] * v2[2]);
  const float ir1 = 1.f / r1, ir2 = 1.f / r2;
  const float g = ir1 * ir2;
  float c = (v1[0] * v2[0] + v1[1] * v2[1] + v1[2] * v2[2]) * g;
  c = fminf(1.f, fmaxf(-1.f, c));
  const float th = acosf(c);
  const float one_m_c2 = 1.f - c * c;
  const float s = one_m_c2 > 0.f ? -rsqrtf(one_m_c2) : 0.f;  // dtheta/dcos
  const float s2 = c * s * s * s;                            // d2theta/dcos2
  const float L1 = -a1 * (r1 - r1e), L2 = -a2 * (r2 - r2e), Lt = -ath * (th - the);
  const float ir1s = ir1 * ir1, ir2s = ir2 * ir2;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const float e1 = v1[d] * ir1, e2 = v2[d] * ir2;
    const float dch1 = v2[d] * g - c * ir1 * e1;
    const float dch2 = v1[d] * g - c * ir2 * e2;
    const float dco = -(dch1 + dch2);
    const float d2ch1 = c * (3.f * e1 * e1 - 1.f) * ir1s - 2.f * v2[d] * e1 * ir1s * ir2;
    const float d2ch2 = c * (3.f * e2 * e2 - 1.f) * ir2s - 2.f * v1[d] * e2 * ir2s * ir1;
    const float h = e1 * ir1 + e2 * ir2;
    const float d2co = 2.f * g - 2.f * (v1[d] + v2[d]) * g * h +
                       c * (h * h + (2.f * e1 * e1 - 1.f) * ir1s + (2.f * e2 * e2 - 1.f) * ir2s);
    const float dth_o = s * dco, dth_1 = s * dch1, dth_2 = s * dch2;
    const float d2th_o = s2 * dco * dco + s * d2co;
    const float d2th_1 = s2 * dch1 * dch1 + s * d2ch1;
    const float d2th_2 = s2 * dch2 * dch2 + s * d2ch2;
    const float d2r1 = (1.f - e1 * e1) * ir1, d2r2 = (1.f - e2 * e2) * ir2;
    f[3 * o + d] += -L1 * e1 - L2 * e2 + Lt * dth_o;
    f[3 * h1 + d] += L1 * e1 + Lt * dth_1;
    f[3 * h2 + d] += L2 * e2 + Lt * dth_2;
    tsum += imo * (-a1 * e1 * e1 - a2 * e2 * e2 - ath * dth_o * dth_o + L1 * d2r1 + L2 * d2r2 + Lt * d2th_o) +
            imh1 * (-a1 * e1 * e1 - ath * dth_1 * dth_1 + L1 * d2r1 + Lt * d2th_1) +
            imh2 * (-a2 * e2 * e2 - ath * dth_2 * dth_2 + L2 * d2r2 + Lt * d2th_2);
  }
  lnpsi += -0.5f * (a1 * (r1 - r1e) * (r1 - r1e) + a2 * (r2 - r2e) * (r2 - r2e) + ath * (th - the) * (th - the));
}

__device__ __forceinline__ float dimer_trial_f32(const float (&x)[18], const StepF32& P, float (&d1)[18],
                                                 float& lap) {
  const float* p = P.trial;
#pragma unroll
  for (int k = 0; k < 18; ++k) d1[k] = 0.f;
  float lnpsi = 0.f, tsum = 0.f;
  h2o_trial_f32(x, p, 0, P.inv_mass[0], P.inv_mass[1], P.inv_mass[2], d1, lnpsi, tsum);
  h2o_trial_f32(x, p, 3, P.inv_mass[3], P.inv_mass[4], P.inv_mass[5], d1, lnpsi, tsum);
  const float aR = p[6], Re = p[7];
  float v[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) v[d] = x[9 + d] - x[d];
  const float R = sqrtf(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  const float iR = 1.f / R;
  const float LR = -aR * (R - Re);
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const float ed = v[d] * iR;
    const float tt = -aR * ed * ed + LR * (1.f - ed * ed) * iR;
    d1[9 + d] += LR * ed;
    d1[d] -= LR * ed;
    tsum += (P.inv_mass[3] + P.inv_mass[0]) * tt;
  }
  lnpsi += -0.5f * aR * (R - Re) * (R - Re);
  float q = 0.f;
#pragma unroll
  for (int k = 0; k < 18; ++k) q += P.inv_mass[k / 3] * d1[k] * d1[k];
  lap = q + tsum;
  return lnpsi;
}

// Importance-sampled move of one fp32 dimer walker (pyvibdmc.py:549-612 with
// ImpSamp.metropolis, imp_samp.py:28-47): proposal y = x + sigma z + (f_x/m) dt,
// trial at y, acceptance min(1, G(y->x)/G(x->y) (psi_y/psi_x)^2) with the
// psi ratio folded into one exponent through ln psi; accept(met) decides
// met > u (it may draw u, after the deviates z).  On return x, f, lnpsi and ke
// hold the walker's state after the Metropolis test; returns whether the
// proposal was accepted.
template <typename Acc>
__device__ __forceinline__ bool is_move_f32(const StepF32& P, float (&x)[18], float (&f)[18], float& lnpsi,
                                            float& ke, const float (&z)[18], const Acc& accept) {
  const float dt = P.dt;
  float y[18], fy[18], lap;
#pragma unroll
  for (int k = 0; k < 18; ++k) y[k] = x[k] + P.sigma[k / 3] * z[k] + P.inv_mass[k / 3] * f[k] * dt;
  const float lpy = dimer_trial_f32(y, P, fy, lap);
  float expo = 0.f;
#pragma unroll
  for (int k = 0; k < 18; ++k) {
    const float im = P.inv_mass[k / 3];
    const float a = x[k] - y[k] - im * fy[k] * dt;
    const float b = y[k] - x[k] - im * f[k] * dt;
    expo += (b * b - a * a) * P.h[k / 3];
  }
  const float met = __expf(expo + 2.f * (lpy - lnpsi));
  const bool acc = accept(met);
  if (acc) {
#pragma unroll
    for (int k = 0; k < 18; ++k) {
      x[k] = y[k];
      f[k] = fy[k];
    }
    lnpsi = lpy;
    ke = -0.5f * lap;
  }
  return acc;
}

// The analytic dimer energy in fp32: the terms of pes_dimer (two local-mode
// monomers, the O-O Lennard-Jones, nine intermolecular charge pairs) in its
// summation order, p = De, a, re, k_theta, theta_e, k_rr, eps, sigma, q_H,
// q_O.  About 1e-7 relative (~1e-2 cm^-1 per walker), far below the
// surrogate error that the audit measures; used for the audit and the
// out-of-box fallback of the fp32 surrogate walkers.
__device__ __forceinline__ float dimer_energy_f32(const float (&x)[18], const float (&p)[10]) {
  float v = 0.f;
#pragma unroll
  for (int m = 0; m < 2; ++m) {
    const int o = 3 * m, h1 = o + 1, h2 = o + 2;
    float d1[3], d2[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      d1[d] = x[3 * h1 + d] - x[3 * o + d];
      d2[d] = x[3 * h2 + d] - x[3 * o + d];
    }
    const float r1 = sqrtf(d1[0] * d1[0] + d1[1] * d1[1] + d1[2] * d1[2]);
    const float r2 = sqrtf(d2[0] * d2[0] + d2[1] * d2[1] + d2[2] * d2[2]);
    const float dot = d1[0] * d2[0] + d1[1] * d2[1] + d1[2] * d2[2];
    const float c = fminf(1.f, fmaxf(-1.f, dot / (r1 * r2)));
    const float dth = acosf(c) - p[4];
    const float dr1 = r1 - p[2], dr2 = r2 - p[2];
    const float e1 = 1.f - expf(-p[1] * dr1), e2 = 1.f - expf(-p[1] * dr2);
    v += p[0] * e1 * e1 + p[0] * e2 * e2 + 0.5f * p[3] * dth * dth + p[5] * dr1 * dr2;
  }
  {
    float d[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) d[k] = x[9 + k] - x[k];
    const float s2 = p[7] * p[7] / (d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    const float s6 = s2 * s2 * s2;
    v += 4.f * p[6] * (s6 * s6 - s6);
  }
  const float q[3] = {p[9], p[8], p[8]};  // O, H, H
#pragma unroll
  for (int i = 0; i < 3; ++i) {
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      float d[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) d[k] = x[3 * (3 + j) + k] - x[3 * i + k];
      const float r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
      v += q[i] * q[j] * (r2 > 0.f ? rsqrtf(r2) : 0.f);
    }
  }
  return v;
}

// The descriptor normalisation and training box of a network, prepared on
// the host: f_q = r_q scale_q + shift_q (scale = 1/sd, shift = -mu/sd) and
// the box [lo_q - margin, hi_q + margin]; sorted: the atoms are put in the
// canonical order of dimer_sort_pairs before the descriptors are formed.
struct FeatBox {
  float scale[15], shift[15], lo[15], hi[15];
  int sorted;
};

inline FeatBox feat_box(const gbdmc_mlp_t& net) {
  FeatBox B{};
  for (int q = 0; q < 15; ++q) {
    B.scale[q] = net.feat_inv_sd[q];
    B.shift[q] = -net.feat_mu[q] * net.feat_inv_sd[q];
    B.lo[q] = net.feat_lo[q] - net.hull_margin;
    B.hi[q] = net.feat_hi[q] + net.hull_margin;
  }
  B.sorted = net.sort_atoms != 0;
  return B;
}

__device__ __forceinline__ float sqrt_approx(float x) {
  float y;
  asm("sqrt.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// Exchange a[i] and a[j] when c (selects, no divergence).
template <typename A>
__device__ __forceinline__ void cswap(bool c, A&& a, int i, int j) {
  const float u = a[i], w = a[j];
  a[i] = c ? w : u;
  a[j] = c ? u : w;
}

// Pair index of atoms (i, j), i < j, in itertools.combinations order:
// (0,1) 0, (0,2) 1, (0,3) 2, (0,4) 3, (0,5) 4, (1,2) 5, (1,3) 6, (1,4) 7,
// (1,5) 8, (2,3) 9, (2,4) 10, (2,5) 11, (3,4) 12, (3,5) 13, (4,5) 14.
//
// The water dimer (O,H,H,O,H,H) in the canonical atom order of DistIt with
// method 'coulomb', sorted_atoms [[0],[1,2],[3],[4,5]] and sorted_groups
// [[0,1,2],[3,4,5]] (tensorflow_descriptors/distance_descriptors.py:115-152,
// 154-165, 177-213).  On the Coulomb matrix M (M_ij = z_i z_j / r_ij, M_ii = z_i^2.4
// / 2, z = 8, 1, 1, 8, 1, 1):
//   1. in each water the hydrogen with the larger column norm of M first;
//   2. the water whose columns' norms sum higher first.
// Decided on ir (the 15 inverse pair distances, original order); applies the
// atom permutation to the pair values ir and, when t is given, t (the
// directional derivatives of the same descriptors).  A permutation of
// equivalent atoms leaves the descriptor values of a walker unchanged as a
// set, so every copy of a geometry under the dimer's eight-element
// permutation group gets the same descriptors.  Ties keep the given order.
template <bool TANG, typename A, typename Tg>
__device__ __forceinline__ void dimer_sort_pairs(A&& ir, Tg&& t) {
  // Column c of M has norm sqrt(M_cc^2 + z_c^2 s_c), s_c = sum_{i != c} z_i^2 / r_ic^2.
  // Two hydrogens of a water share z and M_cc, so their norms order as their s.
  float s[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  {
    int q = 0;
#pragma unroll
    for (int i = 0; i < 6; ++i) {
#pragma unroll
      for (int j = i + 1; j < 6; ++j) {
        const float w = ir[q] * ir[q];
        s[i] = fmaf((j % 3 == 0) ? 64.f : 1.f, w, s[i]);
        s[j] = fmaf((i % 3 == 0) ? 64.f : 1.f, w, s[j]);
        ++q;
      }
    }
  }
  const bool sA = s[2] > s[1], sB = s[5] > s[4];
  // The waters' sums of column norms, with the single-instruction square root
  // (sqrt.approx, relative error ~2^-23): it moves only decisions within a few
  // ulps of a tie, where the two orders are both in the training data.
  constexpr float dO2 = 5404.7044f;  // (8^2.4 / 2)^2 = 5404.70440...
  constexpr float dH2 = 0.25f;       // (1^2.4 / 2)^2
  const float nA = sqrt_approx(fmaf(64.f, s[0], dO2)) + sqrt_approx(dH2 + s[1]) + sqrt_approx(dH2 + s[2]);
  const float nB = sqrt_approx(fmaf(64.f, s[3], dO2)) + sqrt_approx(dH2 + s[4]) + sqrt_approx(dH2 + s[5]);
  const bool sG = nB > nA;
  // 1. hydrogens 1 <-> 2, then 4 <-> 5
  cswap(sA, ir, 0, 1), cswap(sA, ir, 6, 9), cswap(sA, ir, 7, 10), cswap(sA, ir, 8, 11);
  cswap(sB, ir, 3, 4), cswap(sB, ir, 7, 8), cswap(sB, ir, 10, 11), cswap(sB, ir, 12, 13);
  // 2. waters (0,1,2) <-> (3,4,5)
  cswap(sG, ir, 0, 12), cswap(sG, ir, 1, 13), cswap(sG, ir, 3, 6), cswap(sG, ir, 4, 9), cswap(sG, ir, 5, 14),
      cswap(sG, ir, 8, 10);
  if constexpr (TANG) {
    cswap(sA, t, 0, 1), cswap(sA, t, 6, 9), cswap(sA, t, 7, 10), cswap(sA, t, 8, 11);
    cswap(sB, t, 3, 4), cswap(sB, t, 7, 8), cswap(sB, t, 10, 11), cswap(sB, t, 12, 13);
    cswap(sG, t, 0, 12), cswap(sG, t, 1, 13), cswap(sG, t, 3, 6), cswap(sG, t, 4, 9), cswap(sG, t, 5, 14),
        cswap(sG, t, 8, 10);
  }
}

// Descriptors of one walker into its feature row (15 normalised inverse pair
// distances, in the canonical atom order when B.sorted, then a zero pad):
// a register array float[16] or a row of shared memory (float*); returns
// true when the walker lies outside the training box.  The pair values are
// formed in the row itself and normalised there.
template <typename Row>
__device__ __forceinline__ bool walker_features(const float (&xs)[18], const FeatBox& B, Row&& row) {
  int q = 0;
#pragma unroll
  for (int i = 0; i < 6; ++i) {
#pragma unroll
    for (int j = i + 1; j < 6; ++j) {
      const float dx = xs[3 * i] - xs[3 * j], dy = xs[3 * i + 1] - xs[3 * j + 1], dz = xs[3 * i + 2] - xs[3 * j + 2];
      row[q++] = rsqrtf(dx * dx + dy * dy + dz * dz);
    }
  }
  if (B.sorted) dimer_sort_pairs<false>(row, row);
  bool out = false;
#pragma unroll
  for (int k = 0; k < 15; ++k) {
    const float f = fmaf(row[k], B.scale[k], B.shift[k]);
    out |= (f < B.lo[k]) || (f > B.hi[k]);
    row[k] = f;
  }
  row[15] = 0.f;
  return out;
}

// Audit selection of a walker from its 32-bit hash h of (walker, step,
// replica stream): h * audit_every < 2^32, probability 1/audit_every
// (every walker for 1, none for 0) with one wide multiply.
__device__ __forceinline__ bool audit_pick(uint32_t h, int audit_every) {
  return audit_every > 0 && (uint64_t)h * (uint64_t)(uint32_t)audit_every < (1ull << 32);
}

}  // namespace gbdmc
