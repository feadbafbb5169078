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
