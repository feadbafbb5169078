// Device helpers shared by the surrogate kernels (mma.sync and tcgen05 paths).
#pragma once
#include <cuda_bf16.h>
#include "gbdmc_stepcore.cuh"

namespace gbdmc {

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&v);
}

// sigmoid(z) = (1 + tanh(z/2)) / 2 with the single-instruction tanh.approx.f32
// (|error| ~ 1e-3 relative, below the bf16 rounding of the activations).
__device__ __forceinline__ float tanh_approx(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float sigmoidf_(float z) { return fmaf(0.5f, tanh_approx(0.5f * z), 0.5f); }
__device__ __forceinline__ float silu(float z) { return z * sigmoidf_(z); }

// -1/2 sum_d sum_a (1/m_a) (d2 psi/dx2)/psi in fp32, the summation order of
// local_ke (imp_samp.py:49-53).
__device__ __forceinline__ float local_ke_f32(const gbdmc_sim_t& S, const float (&d2)[18]) {
  float s = 0.f;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    float t = 0.f;
#pragma unroll
    for (int a = 0; a < 6; ++a) t += (float)S.inv_mass[a] * d2[3 * a + d];
    s += t;
  }
  return -0.5f * s;
}

// Importance-sampled move of one fp32 dimer walker (pyvibdmc.py:549-612 with
// ImpSamp.metropolis, imp_samp.py:28-47): proposal y = x + sigma z + (f_x/m) dt,
// trial at y, acceptance min(1, G(y->x)/G(x->y) (psi_y/psi_x)^2) with the
// psi ratio folded into one exponent through ln psi.  On return x, f, lnpsi
// and ke hold the walker's state after the Metropolis test; returns whether
// the proposal was accepted.  u is the acceptance uniform.
__device__ __forceinline__ bool is_move_f32(const gbdmc_sim_t& S, float (&x)[18], float (&f)[18], float& lnpsi,
                                            float& ke, const float (&z)[18], double u) {
  const float dt = (float)S.dt;
  float y[18], fy[18], d2y[18];
#pragma unroll
  for (int k = 0; k < 18; ++k) y[k] = x[k] + (float)S.sigma[k / 3] * z[k] + (float)S.inv_mass[k / 3] * f[k] * dt;
  const float lpy = dimer_trial_log(y, S.trial.p, fy, d2y);
  float h[6];  // 1 / (2 sigma_a^2), one division per atom
#pragma unroll
  for (int a = 0; a < 6; ++a) {
    const float sg = (float)S.sigma[a];
    h[a] = 0.5f / (sg * sg);
  }
  float expo = 0.f;
#pragma unroll
  for (int k = 0; k < 18; ++k) {
    const float im = (float)S.inv_mass[k / 3];
    const float a = x[k] - y[k] - im * fy[k] * dt;
    const float b = y[k] - x[k] - im * f[k] * dt;
    expo += (b * b - a * a) * h[k / 3];
  }
  const float met = expf(expo + 2.f * (lpy - lnpsi));
  const bool acc = (double)met > u;
  if (acc) {
#pragma unroll
    for (int k = 0; k < 18; ++k) {
      x[k] = y[k];
      f[k] = fy[k];
    }
    lnpsi = lpy;
    ke = local_ke_f32(S, d2y);
  }
  return acc;
}

// Descriptors of one walker into the warp's feature row; returns true when
// the walker lies outside the training box (normalised range +- margin).
__device__ __forceinline__ bool walker_features(const float (&xs)[18], const gbdmc_mlp_t& net, float* row) {
  int q = 0;
  bool out = false;
#pragma unroll
  for (int i = 0; i < 6; ++i) {
#pragma unroll
    for (int j = i + 1; j < 6; ++j) {
      const float dx = xs[3 * i] - xs[3 * j], dy = xs[3 * i + 1] - xs[3 * j + 1], dz = xs[3 * i + 2] - xs[3 * j + 2];
      const float f = (rsqrtf(dx * dx + dy * dy + dz * dz) - net.feat_mu[q]) * net.feat_inv_sd[q];
      out |= (f < net.feat_lo[q] - net.hull_margin) || (f > net.feat_hi[q] + net.hull_margin);
      row[q] = f;
      ++q;
    }
  }
  row[15] = 0.f;
  return out;
}

}  // namespace gbdmc
