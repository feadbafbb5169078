// MLP surrogate of the water-dimer PES: the mma.sync (m16n8k16, BF16, FP32
// accumulation) inference path, the training pipeline and the surrogate DMC
// step's audit and counting kernels.
//
// Network: 15 inverse O/H distances (normalised, padded to 16) -> 128 -> 128
// -> 128 (SiLU) -> 1.  The mma.sync inference keeps a warp's 16 walkers'
// activations in registers from layer to layer: the m16n8 accumulator
// fragments of one layer are repacked as the m16k16 A fragments of the next,
// and the weights stay in shared memory for the whole persistent CTA.
//
// Training (force matching): the GEMMs Y = X W (+b) and G += X^T D run on the
// tcgen05 tensor cores (gbdmc_mlp_tc.cu); here are the fused SiLU
// forward/backward with a tangent (directional-derivative) stream, so that
// d(E . u)/dW -- the gradient of the force residual -- is one more pass of
// the same GEMMs, the head, the batch inputs and the fused Adam step.
#include <mutex>

#include "gbdmc_mlp_common.cuh"

namespace gbdmc {

constexpr int kH = 128;    // hidden width
constexpr int kIn = 16;    // padded input width (15 features)
constexpr int kPadH = 136; // smem row stride (bf16) of 128-wide weights
constexpr int kPadI = 24;  // smem row stride (bf16) of 16-wide weights

__device__ __forceinline__ void mma16816(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// Copy a transposed bf16 weight matrix Wt[128][K] from global into smem rows of stride P.
__device__ __forceinline__ void load_wt(uint16_t* dst, const uint16_t* __restrict__ src, int K, int P) {
  for (int e = threadIdx.x; e < kH * K / 2; e += blockDim.x) {
    const int n = (2 * e) / K, k = (2 * e) % K;
    *reinterpret_cast<uint32_t*>(dst + n * P + k) = __ldg(reinterpret_cast<const uint32_t*>(src) + e);
  }
}

// acc[16 n-tiles][4] += A(16 x 16 k-chunk) * W(k-chunk x 128), W from smem Wt rows of stride P.
__device__ __forceinline__ void mma_row16(float (&acc)[16][4], const uint32_t (&a)[4], const uint16_t* Ws, int P,
                                          int kc) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int j = 0; j < 16; ++j) {
    const uint16_t* row = Ws + (8 * j + g) * P + 16 * kc + 2 * t;
    const uint32_t b0 = *reinterpret_cast<const uint32_t*>(row);
    const uint32_t b1 = *reinterpret_cast<const uint32_t*>(row + 8);
    mma16816(acc[j], a[0], a[1], a[2], a[3], b0, b1);
  }
}

// --------------------------------------------------------- training GEMMs
// Y[M x 128] = X[M x K] W[K x 128] (+ bias); X fp32 row-major, Wt bf16 [128][K].
// blockIdx.y selects one of two operand sets that share W (a pair of GEMMs,
// e.g. the primal and tangent streams of a layer, in one launch).
template <int K>
__global__ void __launch_bounds__(256) k_gemm_xw(const float* __restrict__ X0, const float* __restrict__ X1,
                                                  long long M, const uint16_t* __restrict__ Wt,
                                                  const float* __restrict__ bias0, const float* __restrict__ bias1,
                                                  float* __restrict__ Y0, float* __restrict__ Y1) {
  const float* __restrict__ X = blockIdx.y ? X1 : X0;
  const float* __restrict__ bias = blockIdx.y ? bias1 : bias0;
  float* __restrict__ Y = blockIdx.y ? Y1 : Y0;
  constexpr int P = K == kH ? kPadH : kPadI;
  __shared__ __align__(16) uint16_t Ws[kH * P];
  load_wt(Ws, Wt, K, P);
  __syncthreads();
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3, w = threadIdx.x >> 5;
  for (long long r0 = (long long)blockIdx.x * 128 + 16 * w; r0 < M; r0 += (long long)gridDim.x * 128) {
    float acc[16][4];
#pragma unroll
    for (int j = 0; j < 16; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
    const long long ra = r0 + g, rb = r0 + g + 8;
#pragma unroll
    for (int kc = 0; kc < K / 16; ++kc) {
      const int c = 16 * kc + 2 * t;
      float2 xa0 = make_float2(0.f, 0.f), xa1 = xa0, xb0 = xa0, xb1 = xa0;
      if (ra < M) {
        xa0 = *reinterpret_cast<const float2*>(X + ra * K + c);
        xa1 = *reinterpret_cast<const float2*>(X + ra * K + c + 8);
      }
      if (rb < M) {
        xb0 = *reinterpret_cast<const float2*>(X + rb * K + c);
        xb1 = *reinterpret_cast<const float2*>(X + rb * K + c + 8);
      }
      const uint32_t a[4] = {pack_bf16(xa0.x, xa0.y), pack_bf16(xb0.x, xb0.y), pack_bf16(xa1.x, xa1.y),
                             pack_bf16(xb1.x, xb1.y)};
      mma_row16(acc, a, Ws, P, kc);
    }
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      const int col = 8 * j + 2 * t;
      const float b0 = bias ? bias[col] : 0.f, b1 = bias ? bias[col + 1] : 0.f;
      if (ra < M) *reinterpret_cast<float2*>(Y + ra * kH + col) = make_float2(acc[j][0] + b0, acc[j][1] + b1);
      if (rb < M) *reinterpret_cast<float2*>(Y + rb * kH + col) = make_float2(acc[j][2] + b0, acc[j][3] + b1);
    }
  }
}

// G[K x 128] += X[M x K]^T D[M x 128]: chunks of 64 rows staged transposed in
// smem (bf16), reduced over M in registers, then one fp32 atomicAdd per element.
// blockIdx.y selects one of two (X, D) pairs accumulated into the same G.
template <int K>
__global__ void __launch_bounds__(256) k_gemm_tn(const float* __restrict__ X0, const float* __restrict__ D0,
                                                  const float* __restrict__ X1, const float* __restrict__ D1,
                                                  long long M, float* __restrict__ G) {
  const float* __restrict__ X = blockIdx.y ? X1 : X0;
  const float* __restrict__ D = blockIdx.y ? D1 : D0;
  constexpr int CH = 64, PC = CH + 8;
  __shared__ __align__(16) uint16_t Xt[K * PC];
  __shared__ __align__(16) uint16_t Dt[kH * PC];
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3, w = threadIdx.x >> 5;
  constexpr int NTW = K == kH ? 16 : 2;  // n-tiles per warp
  const int mt = K == kH ? w : 0;         // m-tile (rows of K) of this warp
  const int nt0 = K == kH ? 0 : 2 * w;
  float acc[NTW][4];
#pragma unroll
  for (int j = 0; j < NTW; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
  for (long long c0 = (long long)blockIdx.x * CH; c0 < M; c0 += (long long)gridDim.x * CH) {
    __syncthreads();
    for (int e = threadIdx.x; e < CH * K; e += blockDim.x) {
      const int r = e / K, c = e % K;
      const float v = (c0 + r < M) ? X[(c0 + r) * K + c] : 0.f;
      const __nv_bfloat16 b = __float2bfloat16_rn(v);
      Xt[c * PC + r] = *reinterpret_cast<const uint16_t*>(&b);
    }
    for (int e = threadIdx.x; e < CH * kH; e += blockDim.x) {
      const int r = e / kH, c = e % kH;
      const float v = (c0 + r < M) ? D[(c0 + r) * kH + c] : 0.f;
      const __nv_bfloat16 b = __float2bfloat16_rn(v);
      Dt[c * PC + r] = *reinterpret_cast<const uint16_t*>(&b);
    }
    __syncthreads();
#pragma unroll
    for (int ks = 0; ks < CH; ks += 16) {
      const uint16_t* xa = Xt + (16 * mt + g) * PC + ks + 2 * t;
      const uint16_t* xb = Xt + (16 * mt + g + 8) * PC + ks + 2 * t;
      const uint32_t a0 = *reinterpret_cast<const uint32_t*>(xa);
      const uint32_t a1 = *reinterpret_cast<const uint32_t*>(xb);
      const uint32_t a2 = *reinterpret_cast<const uint32_t*>(xa + 8);
      const uint32_t a3 = *reinterpret_cast<const uint32_t*>(xb + 8);
#pragma unroll
      for (int j = 0; j < NTW; ++j) {
        const uint16_t* db = Dt + (8 * (nt0 + j) + g) * PC + ks + 2 * t;
        mma16816(acc[j], a0, a1, a2, a3, *reinterpret_cast<const uint32_t*>(db),
                 *reinterpret_cast<const uint32_t*>(db + 8));
      }
    }
  }
#pragma unroll
  for (int j = 0; j < NTW; ++j) {
    const int col = 8 * (nt0 + j) + 2 * t;
    const int ra = 16 * mt + g, rb = ra + 8;
    atomicAdd(G + ra * kH + col, acc[j][0]);
    atomicAdd(G + ra * kH + col + 1, acc[j][1]);
    atomicAdd(G + rb * kH + col, acc[j][2]);
    atomicAdd(G + rb * kH + col + 1, acc[j][3]);
  }
}

// ------------------------------------------------------------ elementwise
// The training kernels take the logistic function through CUDA's expf and an
// IEEE division (a few fp32 ulps), so that the gradients can be checked
// against an oracle that rounds where these kernels round; inference keeps
// the tanh.approx form (sigmoidf_), whose error is below the bf16 rounding of
// its activations.
__device__ __forceinline__ float sigmoid_acc(float z) { return 1.f / (1.f + expf(-z)); }

// H = silu(Z); Ht = silu'(Z) Zt  (tangent stream, may be NULL)
__global__ void k_silu_fwd(const float* __restrict__ Z, const float* __restrict__ Zt, float* __restrict__ H,
                           float* __restrict__ Ht, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float z = Z[i];
    const float s = sigmoid_acc(z);
    H[i] = z * s;
    if (Ht) Ht[i] = s * (1.f + z * (1.f - s)) * Zt[i];
  }
}

// Zb = silu'(Z) Hb + silu''(Z) Zt Htb ;  Ztb = silu'(Z) Htb, on rows of 128
// columns; with gbias also the bias gradient gbias[c] += sum over rows of
// Zb[., c] (each thread keeps one column, a block adds its two row halves
// and issues one atomic per column).
__global__ void __launch_bounds__(256) k_silu_bwd(const float* __restrict__ Z, const float* __restrict__ Zt,
                                                  const float* __restrict__ Hb, const float* __restrict__ Htb,
                                                  float* __restrict__ Zb, float* __restrict__ Ztb, long long rows,
                                                  float* __restrict__ gbias) {
  const int c = threadIdx.x & (kH - 1);
  float acc = 0.f;
  for (long long r = 2LL * blockIdx.x + (threadIdx.x >> 7); r < rows; r += 2LL * gridDim.x) {
    const long long i = r * kH + c;
    const float z = Z[i];
    const float s = sigmoid_acc(z);
    const float d1 = s * (1.f + z * (1.f - s));
    const float d2 = s * (1.f - s) * (2.f + z * (1.f - 2.f * s));
    const float hb = Hb[i];
    float zb;
    if (Zt) {
      const float htb = Htb[i];
      zb = d1 * hb + d2 * Zt[i] * htb;
      Ztb[i] = d1 * htb;
    } else {
      zb = d1 * hb;
    }
    Zb[i] = zb;
    acc += zb;
  }
  if (gbias) {
    __shared__ float half[kH];
    if (threadIdx.x >= kH) half[c] = acc;
    __syncthreads();
    if (threadIdx.x < kH) atomicAdd(gbias + c, acc + half[c]);
  }
}

// Output layer and loss, one warp per sample:
//   E = H3 w4 + b4, Et = Ht3 w4;  L = wE (E - e)^2 + wF (Et - et)^2 (mean over samples)
//   writes dL/dH3, dL/dHt3, accumulates dL/dw4, dL/db4 and the loss terms
//   (per block in shared memory, then one atomic per quantity and block).
//   b4 is read on the device when b4_dev is given.
__global__ void __launch_bounds__(256) k_head(const float* __restrict__ H3, const float* __restrict__ Ht3,
                                              const float* __restrict__ w4, float b4_val,
                                              const float* __restrict__ b4_dev, const float* __restrict__ e_true,
                                              const float* __restrict__ et_true, long long M, float wE, float wF,
                                              float* __restrict__ H3b, float* __restrict__ Ht3b,
                                              float* __restrict__ gw4, float* __restrict__ gb4,
                                              double* __restrict__ loss) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  const float b4 = b4_dev ? *b4_dev : b4_val;
  float gw[4] = {0.f, 0.f, 0.f, 0.f}, gb = 0.f;
  double lE = 0.0, lF = 0.0;
  for (long long s = warp; s < M; s += nw) {
    float e = 0.f, et = 0.f;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int c = lane + 32 * q;
      e += H3[s * kH + c] * w4[c];
      if (Ht3) et += Ht3[s * kH + c] * w4[c];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      e += __shfl_xor_sync(0xffffffffu, e, o);
      et += __shfl_xor_sync(0xffffffffu, et, o);
    }
    e += b4;
    const float de = 2.f * wE * (e - e_true[s]) / (float)M;
    const float det = Ht3 ? 2.f * wF * (et - et_true[s]) / (float)M : 0.f;
    if (lane == 0) {
      lE += (double)(e - e_true[s]) * (double)(e - e_true[s]);
      if (Ht3) lF += (double)(et - et_true[s]) * (double)(et - et_true[s]);
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int c = lane + 32 * q;
      H3b[s * kH + c] = de * w4[c];
      if (Ht3) {
        Ht3b[s * kH + c] = det * w4[c];
        gw[q] += de * H3[s * kH + c] + det * Ht3[s * kH + c];
      } else {
        gw[q] += de * H3[s * kH + c];
      }
    }
    gb += de;
  }
  __shared__ float sgw[8][kH];
  __shared__ float sgb[8];
  __shared__ double sl[8][2];
#pragma unroll
  for (int q = 0; q < 4; ++q) sgw[wid][lane + 32 * q] = gw[q];
  if (lane == 0) {
    sgb[wid] = gb;
    sl[wid][0] = lE;
    sl[wid][1] = lF;
  }
  __syncthreads();
  const int nwb = blockDim.x >> 5;
  if (threadIdx.x < kH) {
    float t = 0.f;
    for (int w = 0; w < nwb; ++w) t += sgw[w][threadIdx.x];
    atomicAdd(gw4 + threadIdx.x, t);
  } else if (threadIdx.x == kH) {
    float t = 0.f;
    double a = 0.0, b = 0.0;
    for (int w = 0; w < nwb; ++w) {
      t += sgb[w];
      a += sl[w][0];
      b += sl[w][1];
    }
    atomicAdd(gb4, t);
    atomicAdd(loss, a);
    atomicAdd(loss + 1, b);
  }
}

// Adam on fp32 master parameters; optionally refreshes the bf16 copies used
// by the GEMMs: transposed wt[n*K + k] = p[k*128 + n] (forward) and row-major
// wn[k*128 + n] = p[k*128 + n] (backward through the layer).
__global__ void k_adam(float* __restrict__ p, const float* __restrict__ gr, float* __restrict__ m,
                       float* __restrict__ v, long long n, float lr, float b1, float b2, float eps, float c1,
                       float c2, uint16_t* __restrict__ wt, uint16_t* __restrict__ wn, int K) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float g = gr[i];
    const float mi = b1 * m[i] + (1.f - b1) * g;
    const float vi = b2 * v[i] + (1.f - b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    const float pi = p[i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
    p[i] = pi;
    if (wt || wn) {
      const long long k = i / kH, nn = i % kH;
      const __nv_bfloat16 b = __float2bfloat16_rn(pi);
      if (wt) wt[nn * K + k] = *reinterpret_cast<const uint16_t*>(&b);
      if (wn) wn[i] = *reinterpret_cast<const uint16_t*>(&b);
    }
  }
}

// ------------------------------------------------------------- features
// Inverse distances of the 15 atom pairs (i<j, combinations order of the
// reference's descriptor, tensorflow_descriptors/distance_descriptors.py:66-68),
// with sorted in the canonical atom order of dimer_sort_pairs, normalised
// (d - mu) * inv_sd into frow[0..15]; with TANG also the normalised
// directional derivative along vs (permuted with the descriptors) into
// trow[0..15].
template <bool TANG>
__device__ __forceinline__ void pair_features(const float (&xs)[18], const float (&vs)[18], int sorted,
                                              const float* __restrict__ mu, const float* __restrict__ inv_sd,
                                              float* __restrict__ frow, float* __restrict__ trow) {
  float ir[15], tg[15];
  int q = 0;
#pragma unroll
  for (int i = 0; i < 6; ++i) {
#pragma unroll
    for (int j = i + 1; j < 6; ++j) {
      const float dx = xs[3 * i] - xs[3 * j], dy = xs[3 * i + 1] - xs[3 * j + 1], dz = xs[3 * i + 2] - xs[3 * j + 2];
      const float r = rsqrtf(dx * dx + dy * dy + dz * dz);
      ir[q] = r;
      if constexpr (TANG) {
        const float dvx = vs[3 * i] - vs[3 * j], dvy = vs[3 * i + 1] - vs[3 * j + 1], dvz = vs[3 * i + 2] - vs[3 * j + 2];
        tg[q] = -(dx * dvx + dy * dvy + dz * dvz) * r * r * r;
      }
      ++q;
    }
  }
  if (sorted) dimer_sort_pairs<TANG>(ir, tg);
#pragma unroll
  for (int k = 0; k < 15; ++k) {
    frow[k] = (ir[k] - mu[k]) * inv_sd[k];
    if constexpr (TANG) trow[k] = tg[k] * inv_sd[k];
  }
  frow[15] = 0.f;
  if constexpr (TANG) trow[15] = 0.f;
}

// Descriptors (and with a direction v their derivative along v, and et =
// (dV/dx . v) / e_scale; a permutation of equivalent atoms leaves V
// unchanged) of n walkers.
template <typename T>
__global__ void k_features(const T* __restrict__ x, long long ldx, long long n, const float* __restrict__ mu,
                           const float* __restrict__ inv_sd, const T* __restrict__ vdir, const double* __restrict__ grad,
                           float e_scale, float* __restrict__ feat, float* __restrict__ tang, float* __restrict__ et,
                           int sorted) {
  for (long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x; s < n; s += (long long)gridDim.x * blockDim.x) {
    float xs[18], vs[18];
#pragma unroll
    for (int k = 0; k < 18; ++k) {
      xs[k] = (float)x[k * ldx + s];
      vs[k] = vdir ? (float)vdir[k * ldx + s] : 0.f;
    }
    if (tang)
      pair_features<true>(xs, vs, sorted, mu, inv_sd, feat + s * kIn, tang + s * kIn);
    else
      pair_features<false>(xs, vs, sorted, mu, inv_sd, feat + s * kIn, nullptr);
    if (et) {
      double d = 0.0;
#pragma unroll
      for (int k = 0; k < 18; ++k) d += grad[k * ldx + s] * (double)vs[k];
      et[s] = (float)(d / (double)e_scale);
    }
  }
}

// ------------------------------------------------------- training batches
// A training batch runs as one CUDA graph: its samples are read at the
// device-side offset ctl[1], the tangent directions are drawn on the device
// from the device step count ctl[0], and one Adam kernel updates every
// parameter, clears the gradients and advances ctl.
//
// Inputs of samples [off, off + B) of the data set (fp64 SoA [18][ld] x and
// grad, v[ld]), off = ctl[1]: descriptors and, along a random unit direction u
// of the 18 coordinates (18 Philox normals of (seed, step ctl[0], sample),
// normalised), their derivative, et = (dV/dx . u) / e_scale and the energy
// target e = (V - e_mean) / e_scale - b4.
__global__ void k_train_inputs(const double* __restrict__ x, const double* __restrict__ v,
                               const double* __restrict__ grad, long long ld, long long B,
                               const long long* __restrict__ ctl, unsigned long long seed,
                               const float* __restrict__ mu, const float* __restrict__ inv_sd, float e_mean,
                               float e_scale, const float* __restrict__ b4, int sorted, float* __restrict__ feat,
                               float* __restrict__ tang, float* __restrict__ et, float* __restrict__ e) {
  const long long step = ctl[0], off = ctl[1];
  const float b4v = *b4;
  for (long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x; s < B; s += (long long)gridDim.x * blockDim.x) {
    const long long j = off + s;
    float xs[18], u[18];
#pragma unroll
    for (int k = 0; k < 18; ++k) xs[k] = (float)x[k * ld + j];
    Rng rng(seed, (uint64_t)step, (uint64_t)s);
    float nn = 0.f;
#pragma unroll
    for (int k = 0; k < 18; k += 2) {
      rng.normal2_f32(u[k], u[k + 1]);
      nn = fmaf(u[k], u[k], fmaf(u[k + 1], u[k + 1], nn));
    }
    const float inv = rsqrtf(nn);
#pragma unroll
    for (int k = 0; k < 18; ++k) u[k] *= inv;
    pair_features<true>(xs, u, sorted, mu, inv_sd, feat + s * kIn, tang + s * kIn);
    double d = 0.0;
#pragma unroll
    for (int k = 0; k < 18; ++k) d += grad[k * ld + j] * (double)u[k];
    et[s] = (float)(d / (double)e_scale);
    e[s] = (float)((v[j] - (double)e_mean) / (double)e_scale) - b4v;
  }
}

// One Adam step on every parameter of the network (pyvibdmc's Keras
// training has no counterpart; Adam as Kingma & Ba 2015): the step t =
// ctl[0] + 1, the learning rate of the cosine schedule lr_min + (lr0 -
// lr_min) (1 + cos(pi k / steps)) / 2 at k = t - 1 - t0, the gradients
// cleared after use, the bf16 copies of the weight matrices refreshed; the
// last block to finish (ticket) advances ctl[0] and the batch offset ctl[1].
struct AdamAll {
  float* p[8];
  float* g[8];
  float* m[8];
  float* v[8];
  uint16_t* wt[8];
  uint16_t* wn[8];
  int k[8];
  long long start[9];
  int nq;
  float lr0, lr_min, b1, b2, eps;
  long long t0, steps, batch;
};

__global__ void __launch_bounds__(256) k_adam_all(const __grid_constant__ AdamAll A, long long* ctl,
                                                  unsigned int* ticket) {
  const long long t = ctl[0] + 1;
  const long long kk = t - 1 - A.t0;
  const float lr = A.lr_min + 0.5f * (A.lr0 - A.lr_min) *
                                  (1.f + cosf(3.14159265358979f * (float)kk / (float)(A.steps > 0 ? A.steps : 1)));
  const float c1 = 1.0f / (1.0f - powf(A.b1, (float)t)), c2 = 1.0f / (1.0f - powf(A.b2, (float)t));
  const long long total = A.start[A.nq];
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    int q = 0;
    while (q + 1 < A.nq && i >= A.start[q + 1]) ++q;
    const long long e = i - A.start[q];
    const float gr = A.g[q][e];
    const float mi = A.b1 * A.m[q][e] + (1.f - A.b1) * gr;
    const float vi = A.b2 * A.v[q][e] + (1.f - A.b2) * gr * gr;
    A.m[q][e] = mi;
    A.v[q][e] = vi;
    const float pi = A.p[q][e] - lr * (mi * c1) / (sqrtf(vi * c2) + A.eps);
    A.p[q][e] = pi;
    A.g[q][e] = 0.f;
    if (A.wt[q] || A.wn[q]) {
      const long long k = e / kH, nn = e % kH;
      const __nv_bfloat16 b = __float2bfloat16_rn(pi);
      if (A.wt[q]) A.wt[q][nn * A.k[q] + k] = *reinterpret_cast<const uint16_t*>(&b);
      if (A.wn[q]) A.wn[q][e] = *reinterpret_cast<const uint16_t*>(&b);
    }
  }
  __shared__ bool last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  __syncthreads();
  if (last && threadIdx.x == 0) {
    ctl[0] = t;
    ctl[1] += A.batch;
    *ticket = 0u;
  }
}

// ------------------------------------------------------------ inference
// Layer l of one warp's 16 rows: acc = A(h, 16 x K) W_l, then bias + SiLU and
// repack into next-layer A fragments.
__device__ __forceinline__ void hidden_layer(uint32_t (&a)[8][4], const uint16_t* Ws, const float* bs) {
  const int lane = threadIdx.x & 31, t = lane & 3;
  float acc[16][4];
#pragma unroll
  for (int j = 0; j < 16; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
#pragma unroll
  for (int kc = 0; kc < 8; ++kc) mma_row16(acc, a[kc], Ws, kPadH, kc);
#pragma unroll
  for (int kc = 0; kc < 8; ++kc) {
    const int c0 = 16 * kc + 2 * t, c1 = c0 + 8;
    const float* u = acc[2 * kc];
    const float* v = acc[2 * kc + 1];
    a[kc][0] = pack_bf16(silu(u[0] + bs[c0]), silu(u[1] + bs[c0 + 1]));
    a[kc][1] = pack_bf16(silu(u[2] + bs[c0]), silu(u[3] + bs[c0 + 1]));
    a[kc][2] = pack_bf16(silu(v[0] + bs[c1]), silu(v[1] + bs[c1 + 1]));
    a[kc][3] = pack_bf16(silu(v[2] + bs[c1]), silu(v[3] + bs[c1 + 1]));
  }
}

struct MlpSmem {
  uint16_t w1[kH * kPadI];
  uint16_t w2[kH * kPadH];
  uint16_t w3[kH * kPadH];
  float b1[kH], b2[kH], b3[kH], w4[kH];
  float feat[8][16][17];  // per warp: 16 walkers x 16 features (+1 pad)
};

__device__ void load_net(MlpSmem& sm, const gbdmc_mlp_t& net) {
  load_wt(sm.w1, net.w1t, kIn, kPadI);
  load_wt(sm.w2, net.w2t, kH, kPadH);
  load_wt(sm.w3, net.w3t, kH, kPadH);
  for (int i = threadIdx.x; i < kH; i += blockDim.x) {
    sm.b1[i] = net.b1[i];
    sm.b2[i] = net.b2[i];
    sm.b3[i] = net.b3[i];
    sm.w4[i] = net.w4[i];
  }
}

// Network output (normalised units) for the 16 feature rows of warp w; on
// return every lane of quad g holds rows g (e_lo) and g + 8 (e_hi).
__device__ __forceinline__ void mlp_forward16(const MlpSmem& sm, const gbdmc_mlp_t& net, int w, float& e_lo,
                                              float& e_hi) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  uint32_t a[8][4];
  {
    float acc[16][4];
#pragma unroll
    for (int j = 0; j < 16; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
    const float* fa = sm.feat[w][g];
    const float* fb = sm.feat[w][g + 8];
    const uint32_t a0[4] = {pack_bf16(fa[2 * t], fa[2 * t + 1]), pack_bf16(fb[2 * t], fb[2 * t + 1]),
                            pack_bf16(fa[2 * t + 8], fa[2 * t + 9]), pack_bf16(fb[2 * t + 8], fb[2 * t + 9])};
    mma_row16(acc, a0, sm.w1, kPadI, 0);
#pragma unroll
    for (int kc = 0; kc < 8; ++kc) {
      const int c0 = 16 * kc + 2 * t, c1 = c0 + 8;
      const float* u = acc[2 * kc];
      const float* v = acc[2 * kc + 1];
      a[kc][0] = pack_bf16(silu(u[0] + sm.b1[c0]), silu(u[1] + sm.b1[c0 + 1]));
      a[kc][1] = pack_bf16(silu(u[2] + sm.b1[c0]), silu(u[3] + sm.b1[c0 + 1]));
      a[kc][2] = pack_bf16(silu(v[0] + sm.b1[c1]), silu(v[1] + sm.b1[c1 + 1]));
      a[kc][3] = pack_bf16(silu(v[2] + sm.b1[c1]), silu(v[3] + sm.b1[c1 + 1]));
    }
  }
  hidden_layer(a, sm.w2, sm.b2);
  // layer 3 + head (fp32 dot with w4)
  float acc[16][4];
#pragma unroll
  for (int j = 0; j < 16; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
#pragma unroll
  for (int kc = 0; kc < 8; ++kc) mma_row16(acc, a[kc], sm.w3, kPadH, kc);
  float lo = 0.f, hi = 0.f;
#pragma unroll
  for (int j = 0; j < 16; ++j) {
    const int c = 8 * j + 2 * t;
    lo += silu(acc[j][0] + sm.b3[c]) * sm.w4[c] + silu(acc[j][1] + sm.b3[c + 1]) * sm.w4[c + 1];
    hi += silu(acc[j][2] + sm.b3[c]) * sm.w4[c] + silu(acc[j][3] + sm.b3[c + 1]) * sm.w4[c + 1];
  }
  lo += __shfl_xor_sync(0xffffffffu, lo, 1);
  lo += __shfl_xor_sync(0xffffffffu, lo, 2);
  hi += __shfl_xor_sync(0xffffffffu, hi, 1);
  hi += __shfl_xor_sync(0xffffffffu, hi, 2);
  e_lo = lo + net.b4;
  e_hi = hi + net.b4;
}

// Energies of n walkers (coordinates SoA, fp32 or fp64) from the surrogate.
template <typename T>
__global__ void __launch_bounds__(256) k_mlp_energy(const __grid_constant__ gbdmc_mlp_t net, const T* __restrict__ x,
                                                     long long ld, long long n, double* __restrict__ v,
                                                     int* __restrict__ outside, const __grid_constant__ FeatBox B) {
  extern __shared__ __align__(16) unsigned char smraw[];
  MlpSmem& sm = *reinterpret_cast<MlpSmem*>(smraw);
  load_net(sm, net);
  __syncthreads();
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3, w = threadIdx.x >> 5;
  for (long long base = (long long)blockIdx.x * 128 + 16 * w; base < n; base += (long long)gridDim.x * 128) {
    bool oob = false;
    if (lane < 16) {
      const long long i = base + lane;
      float xs[18];
#pragma unroll
      for (int k = 0; k < 18; ++k) xs[k] = i < n ? (float)x[k * ld + i] : (k < 3 ? 0.f : 1.f + k);
      oob = walker_features(xs, B, sm.feat[w][lane]) && i < n;
    }
    __syncwarp();
    float e_lo, e_hi;
    mlp_forward16(sm, net, w, e_lo, e_hi);
    const int row = g + 8 * t;
    if (t < 2) {
      const long long i = base + row;
      if (i < n) v[i] = (double)net.e_mean + (double)net.e_scale * (double)(t == 0 ? e_lo : e_hi);
    }
    const unsigned ob = __ballot_sync(0xffffffffu, oob);
    if (outside && lane < 16 && ((ob >> lane) & 1u)) outside[base + lane] = 1;
    __syncwarp();
  }
}

// ------------------------------------------------------- surrogate step
// Phase 1 of a surrogate DMC step (water dimer, fp32 walker coordinates):
// gather through idx and move (lanes 0-15 of each warp own one walker),
// descriptors, then the warp's 16-walker MLP forward on the tensor cores;
// writes V (hartree, fp64).  Walkers selected for the audit or outside the
// training box are appended to a per-step list (scratch) with their flag;
// k_mlp_audit gives them the analytic energy, so this kernel has no
// divergent fp64 work.  Tiles are 128 walkers (8 warps x 16).
__global__ void __launch_bounds__(256) k_mlp_move_energy(const __grid_constant__ gbdmc_sim_t S,
                                                          const __grid_constant__ RepTable T,
                                                          const __grid_constant__ gbdmc_mlp_t net,
                                                          const gbdmc_walkers_f32_t in, gbdmc_walkers_f32_t out,
                                                          gbdmc_ctrl_t* ctrls, int* list, unsigned char* flags,
                                                          const double* audit, const gbdmc_noise_t nz,
                                                          const __grid_constant__ FeatBox B) {
  extern __shared__ __align__(16) unsigned char smraw[];
  MlpSmem& sm = *reinterpret_cast<MlpSmem*>(smraw);
  const double corr = audit ? audit[4] + audit[8] : 0.0;  // online bias correction (hartree)
  load_net(sm, net);
  __syncthreads();
  const int64_t ld = S.ld;
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3, w = threadIdx.x >> 5;
  const int ntile = T.tile_off[T.nrep];
  for (int tile = blockIdx.x; tile < ntile; tile += gridDim.x) {
    const int r = replica_of(T, tile);
    gbdmc_ctrl_t* ctrl = ctrls + r;
    if (*(volatile int*)&ctrl->status) continue;
    const long long n = ctrl->n;
    const long long step = ctrl->step;
    const int64_t base = T.off[r];
    const int64_t i0 = (int64_t)(tile - T.tile_off[r]) * 128 + 16 * w;
    if (i0 >= n) continue;  // warp-uniform: no walkers in this warp's rows
    if (i0 == 0 && lane == 0) store_count_params(ctrl);
    if (lane < 16) {
      const int64_t i = i0 + lane;
      float xs[18];
      if (i < n) {
        const int64_t src = base + (in.idx ? (int64_t)in.idx[base + i] : i);
        const int64_t dst = base + i;
        Rng rng(S.seed, (uint64_t)step, (uint64_t)i, T.stream[r]);
        float z[18];
        if (S.noise_mode == GBDMC_NOISE_INJECTED) {
#pragma unroll
          for (int k = 0; k < 18; ++k) z[k] = (float)nz.normal[k * nz.ld_noise + dst];
        } else {
#pragma unroll
          for (int k = 0; k < 18; k += 2) rng.normal2_f32_fast(z[k], z[k + 1]);
        }
#pragma unroll
        for (int k = 0; k < 18; ++k) {
          xs[k] = in.x[k * ld + src] + (float)S.sigma[k / 3] * z[k];
          out.x[k * ld + dst] = xs[k];
        }
        if (out.who && in.who) out.who[dst] = in.who[src];
        const bool oob = walker_features(xs, B, sm.feat[w][lane]);
        const bool aud = audit_pick(
            splitmix32((uint32_t)i ^ (uint32_t)(step * 0x9E3779B9u) ^ (T.stream[r] * 0x85EBCA6Bu)), net.audit_every);
        const unsigned char fl = (oob ? 1 : 0) | (aud ? 2 : 0);
        if (fl) {
          const unsigned long long q = atomicAdd((unsigned long long*)&ctrl->reserved[2], 1ull);
          list[base + (int64_t)q] = (int)i;
          flags[dst] = fl;
        }
      } else {
#pragma unroll
        for (int k = 0; k < 18; ++k) xs[k] = (k < 3 ? 0.f : 1.f + k);
        walker_features(xs, B, sm.feat[w][lane]);
      }
    }
    __syncwarp();
    float e_lo, e_hi;
    mlp_forward16(sm, net, w, e_lo, e_hi);
    const int row = g + 8 * t;
    const int64_t i = i0 + row;
    if (t < 2 && i < n)
      out.v[base + i] = (double)net.e_mean + (double)net.e_scale * (double)(t == 0 ? e_lo : e_hi) - corr;
    __syncwarp();
  }
}

// Phase 2: the analytic energy (dimer_energy_f32) of the listed walkers:
// the audit subset and the out-of-box fallback, one walker per thread.  The
// lists of all replicas are walked as one: every block scans the replicas'
// list lengths into shared memory and the grid strides over the
// concatenated list (warp w of block b takes chunk w * gridDim + b, so a
// short list still spreads over every SM).  Audited differences
// V_nn - V_analytic are summed per block and added to audit[0..2]
// (fallbacks to audit[3]) with one atomic each per block.
__global__ void __launch_bounds__(128) k_mlp_audit(const __grid_constant__ gbdmc_sim_t S,
                                                    const __grid_constant__ RepTable T, gbdmc_walkers_f32_t out,
                                                    gbdmc_ctrl_t* ctrls, const int* list,
                                                    const unsigned char* flags, double* audit, float beta,
                                                    const __grid_constant__ StepF32 P, unsigned long long* tstat,
                                                    int ntile2, unsigned int* sync) {
  static_assert(GBDMC_MAX_REPLICAS <= 64, "two replicas per lane in the list-length scan");
  __shared__ long long pre[GBDMC_MAX_REPLICAS + 1];  // exclusive prefix of the list lengths
  pdl_wait();
  // the tile status words and tickets of this step's counting pass start cleared
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < ntile2; t += gridDim.x * blockDim.x) tstat[t] = 0ull;
  if (blockIdx.x == 0 && threadIdx.x < 2) sync[threadIdx.x] = 0u;
  const int64_t ld = S.ld;
  const double c_mix = *(volatile const double*)(audit + 4);  // mixed-average part of the correction
  const double c_used = c_mix + audit[8];                        // correction applied to this step's V_nn
  const int nrep = T.nrep;
  const int wpb = blockDim.x >> 5;
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    long long c[2] = {0, 0};
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int r = lane + 32 * h;
      if (r < nrep && *(volatile const int*)&ctrls[r].status == 0) {
        const long long m = *(volatile const long long*)&ctrls[r].reserved[2];
        c[h] = m < T.cap[r] ? m : T.cap[r];
      }
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const long long t = __shfl_up_sync(0xffffffffu, c[h], o);
        if (lane >= o) c[h] += t;
      }
    }
    const long long lo_total = __shfl_sync(0xffffffffu, c[0], 31);
    if (lane == 0) pre[0] = 0;
    if (lane < nrep) pre[lane + 1] = c[0];
    if (lane + 32 < nrep) pre[lane + 33] = c[1] + lo_total;
  }
  __syncthreads();
  const long long total = pre[nrep];
  double s_n = 0.0, s_d = 0.0, s_d2 = 0.0, s_fb = 0.0;
  const long long gw = (long long)(threadIdx.x >> 5) * gridDim.x + blockIdx.x;
  const long long nw = (long long)gridDim.x * wpb;
  for (long long jb = 32 * gw; jb < total; jb += 32 * nw) {
    const long long j = jb + (threadIdx.x & 31);
    if (j >= total) break;
    int r = 0, hi = nrep;  // largest r with pre[r] <= j (then j < pre[r + 1])
    while (hi - r > 1) {
      const int mid = (r + hi) >> 1;
      if (pre[mid] <= j) r = mid;
      else hi = mid;
    }
    const int64_t base = T.off[r];
    const int64_t dst = base + list[base + (j - pre[r])];
    float xs[18];
#pragma unroll
    for (int k = 0; k < 18; ++k) xs[k] = out.x[k * ld + dst];
    const double v = (double)dimer_energy_f32(xs, P.pes);
    const unsigned char fl = flags[dst];
    const double ke = out.ke ? (double)out.ke[dst] : 0.0;  // v holds V + KE with a trial
    if (fl & 2) {
      const double d = (out.v[dst] - ke + c_used) - v;  // error of the raw network energy
      s_n += 1.0;
      s_d += d;
      s_d2 += d * d;
    }
    if (fl & 1) s_fb += 1.0;
    out.v[dst] = v + ke;
  }
  {  // block sums of the audit statistics, one atomic per quantity
    __shared__ double red[4][4];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    s_n = warp_sum(s_n);
    s_d = warp_sum(s_d);
    s_d2 = warp_sum(s_d2);
    s_fb = warp_sum(s_fb);
    if (lane == 0) {
      red[w][0] = s_n;
      red[w][1] = s_d;
      red[w][2] = s_d2;
      red[w][3] = s_fb;
    }
    __syncthreads();
    if (threadIdx.x < 4) {
      double t = 0.0;
      for (int k = 0; k < wpb; ++k) t += red[k][threadIdx.x];
      if (t != 0.0) atomicAdd(audit + threadIdx.x, t);
    }
  }
  // last block: c_mix <- (1 - beta) c_mix + beta * (mean audited error of this
  // step); the next step applies c_mix + audit[8] (the pure-weighting offset
  // the host sets from forward-walking windows, 0 without them)
  __shared__ bool am_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned long long t = atomicAdd(reinterpret_cast<unsigned long long*>(audit + 7), 1ull);
    am_last = (t == (unsigned long long)gridDim.x - 1ull);
  }
  __syncthreads();
  if (am_last && threadIdx.x == 0) {
    __threadfence();
    const double cnt = *(volatile double*)(audit + 0) - audit[5];
    const double sum = *(volatile double*)(audit + 1) - audit[6];
    if (beta > 0.f && cnt > 0.0) audit[4] = (1.0 - (double)beta) * c_mix + (double)beta * (sum / cnt);
    audit[5] = audit[0];
    audit[6] = audit[1];
    *reinterpret_cast<unsigned long long*>(audit + 7) = 0ull;
  }
  if (am_last && S.trial.kind != GBDMC_TRIAL_NONE) {
    // dt_factor = accepted / N (pyvibdmc.py:603) for the weights of this step; effective time (:372-378)
    for (int r = threadIdx.x; r < T.nrep; r += blockDim.x) {
      gbdmc_ctrl_t* c = ctrls + r;
      if (*(volatile int*)&c->status) continue;
      const long long n = c->n, step = c->step;
      const long long na = *(volatile long long*)&c->n_acc;
      const double dte = S.dt * ((double)na / (double)n);
      c->dt_eff = dte;
      count_params(c)->y = (float)dte;
      c->eff_ts = (step == 0) ? dte : c->eff_ts + dte;
      if (step < S.hist.len) {
        const int64_t h = (int64_t)r * S.hist.len + step;
        if (S.hist.rejected) S.hist.rejected[h] = (int)(n - na);
        if (S.hist.eff_ts) S.hist.eff_ts[h] = c->eff_ts;
      }
      c->n_acc = 0;
    }
  }
}

// Step 0 of the surrogate run: energies (with audit/fallback) and vref.
__global__ void __launch_bounds__(256) k_mlp_init(const __grid_constant__ gbdmc_sim_t S,
                                                   const __grid_constant__ RepTable T,
                                                   const __grid_constant__ gbdmc_mlp_t net, gbdmc_walkers_f32_t W,
                                                   gbdmc_ctrl_t* ctrls, Partial* part,
                                                   const __grid_constant__ StepF32 P, const __grid_constant__ FeatBox B) {
  extern __shared__ __align__(16) unsigned char smraw[];
  MlpSmem& sm = *reinterpret_cast<MlpSmem*>(smraw);
  load_net(sm, net);
  __syncthreads();
  const int64_t ld = S.ld;
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3, w = threadIdx.x >> 5;
  const int ntile = T.tile_off[T.nrep];
  for (int tile = blockIdx.x; tile < ntile; tile += gridDim.x) {
    const int r = replica_of(T, tile);
    gbdmc_ctrl_t* ctrl = ctrls + r;
    const long long n = ctrl->n;
    const int64_t base = T.off[r];
    const int64_t i0 = (int64_t)(tile - T.tile_off[r]) * 128 + 16 * w;
    if (lane < 16) {
      const int64_t i = i0 + lane;
      float xs[18];
#pragma unroll
      for (int k = 0; k < 18; ++k) xs[k] = i < n ? W.x[k * ld + base + i] : (k < 3 ? 0.f : 1.f + k);
      walker_features(xs, B, sm.feat[w][lane]);
    }
    __syncwarp();
    float e_lo, e_hi;
    mlp_forward16(sm, net, w, e_lo, e_hi);
    Partial p = partial_zero();
    const int row = g + 8 * t;
    const int64_t i = i0 + row;
    if (t < 2 && i < n) {
      double xd[18], gd[18];
#pragma unroll
      for (int k = 0; k < 18; ++k) xd[k] = (double)W.x[k * ld + base + i];
      // step 0 uses the analytic energy for every walker (start structures are not yet sampled)
      double v = pes_dimer<false>(xd, S.pes.p, gd);
      (void)e_lo;
      (void)e_hi;
      if (S.trial.kind == GBDMC_TRIAL_DIMER_GAUSS) {  // psi_T, drift and local KE at the start (pyvibdmc.py:760-769)
        float xs[18], fx[18], lap;
#pragma unroll
        for (int k = 0; k < 18; ++k) xs[k] = W.x[k * ld + base + i];
        const float lp = dimer_trial_f32(xs, P, fx, lap);
        const float ke = -0.5f * lap;
#pragma unroll
        for (int k = 0; k < 18; ++k) W.f[k * ld + base + i] = fx[k];
        W.lnpsi[base + i] = lp;
        W.ke[base + i] = ke;
        v += (double)ke;
      }
      W.v[base + i] = v;
      p.s0 = v;
      p.c = 1;
    }
    p = block_reduce_partial<false>(p);
    if (threadIdx.x == 0) part[tile] = p;
    const int nt = T.tile_off[r + 1] - T.tile_off[r];
    if (last_tile(ctrl, nt)) {
      const Partial tt = reduce_partials<false>(part, T.tile_off[r], nt, nullptr);
      if (threadIdx.x == 0) {
        const double n0 = (double)T.n0[r];
        ctrl->vref = tt.s0 / (double)n - S.alpha * ((double)(n - T.n0[r]) / n0);
        ctrl->dt_eff = S.dt;  // k_count weights with dt_eff
        ctrl->reserved[2] = 0;
        ctrl->n_acc = 0;
        ctrl->ticket = 0;
      }
    }
  }
}

__global__ void __launch_bounds__(kMaxTPB) k_compact_f32(const __grid_constant__ gbdmc_sim_t S,
                                                          const __grid_constant__ RepTable T,
                                                          const gbdmc_walkers_f32_t in, gbdmc_walkers_f32_t out,
                                                          const gbdmc_ctrl_t* ctrls) {
  const int64_t ld = S.ld;
  const int ntile = T.tile_off[T.nrep];
  for (int tile = blockIdx.x; tile < ntile; tile += gridDim.x) {
    const int r = replica_of(T, tile);
    const long long n = ctrls[r].n;
    const int64_t i = (int64_t)(tile - T.tile_off[r]) * blockDim.x + threadIdx.x;
    if (i >= n) continue;
    const int64_t b = T.off[r];
    const int64_t src = b + (in.idx ? (int64_t)in.idx[b + i] : i);
#pragma unroll
    for (int k = 0; k < 18; ++k) out.x[k * ld + b + i] = in.x[k * ld + src];
    out.v[b + i] = in.v[src];
    if (in.who && out.who) out.who[b + i] = in.who[src];
    if (in.f && out.f) {
#pragma unroll
      for (int k = 0; k < 18; ++k) out.f[k * ld + b + i] = in.f[k * ld + src];
      out.lnpsi[b + i] = in.lnpsi[src];
      out.ke[b + i] = in.ke[src];
    }
  }
}

// ============================================================ host side
static int ew_grid(long long n) {
  long long g = (n + 255) / 256;
  const long long cap = 8LL * num_sms();
  return (int)(g < 1 ? 1 : (g > cap ? cap : g));
}

static int mlp_smem_bytes() { return (int)sizeof(MlpSmem); }

static int set_mlp_smem(const void* fn) {
  const cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, mlp_smem_bytes());
  if (e != cudaSuccess) {
    set_error("cudaFuncSetAttribute: %s", cudaGetErrorString(e));
    return GBDMC_ERR_CUDA;
  }
  return GBDMC_OK;
}

// ---------------------------------------------------- forward walking
// The descendant-weighted (pure-distribution) average of the surrogate's
// error delta = V_nn - V_analytic, the forward-walking estimator of the
// descendant weights of pyvibdmc.py:663-672 applied to delta.  At a window's
// start every live walker s of the compact population gets who[s] = s and
// delta[s]; the step kernels carry who to the copies; at the window's end
// summing delta[who] over the live population gives sum_s D_s delta_s, D_s
// the number of descendants of s.  Each block writes its partial (sum,
// count), replicas and walkers visited in a fixed order, so the host's sum
// in block order is reproducible.
constexpr int kFwThreads = 256;

template <bool BEGIN>
__global__ void __launch_bounds__(kFwThreads) k_fw(const __grid_constant__ RepTable T,
                                                   const gbdmc_ctrl_t* __restrict__ ctrls, const float* __restrict__ x,
                                                   int64_t ld, int32_t* __restrict__ who,
                                                   const double* __restrict__ vnn, const int32_t* __restrict__ outside,
                                                   const __grid_constant__ StepF32 P, double* __restrict__ delta,
                                                   double* __restrict__ part) {
  double s_d = 0.0, s_n = 0.0;
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, nth = (int64_t)gridDim.x * blockDim.x;
  for (int r = 0; r < T.nrep; ++r) {
    const int64_t cap = T.cap[r], off = T.off[r];
    int64_t n = ctrls[r].n;
    n = n < 0 ? 0 : (n > cap ? cap : n);
    for (int64_t i = tid; i < n; i += nth) {
      const int64_t s = off + i;
      double d;
      if constexpr (BEGIN) {
        float xs[18];
#pragma unroll
        for (int k = 0; k < 18; ++k) xs[k] = x[k * ld + s];
        d = outside[s] ? 0.0 : vnn[s] - (double)dimer_energy_f32(xs, P.pes);
        delta[s] = d;
        who[s] = (int32_t)s;
      } else {
        const int32_t a = who[s];
        if (a < 0 || (int64_t)a >= ld) continue;  // not in an open window: not counted
        d = delta[a];
      }
      s_d += d;
      s_n += 1.0;
    }
  }
  __shared__ double red[kFwThreads / 32][2];
  s_d = warp_sum(s_d);
  s_n = warp_sum(s_n);
  if ((threadIdx.x & 31) == 0) {
    red[threadIdx.x >> 5][0] = s_d;
    red[threadIdx.x >> 5][1] = s_n;
  }
  __syncthreads();
  if (threadIdx.x < 2) {
    double t = 0.0;
    for (int w = 0; w < kFwThreads / 32; ++w) t += red[w][threadIdx.x];
    part[2 * blockIdx.x + threadIdx.x] = t;
  }
}

static bool valid_net(const gbdmc_mlp_t* net) {
  return net && net->w1t && net->w2t && net->w3t && net->b1 && net->b2 && net->b3 && net->w4 &&
         (net->sort_atoms == 0 || net->sort_atoms == 1);
}

GBDMC_BOUNDS_READER(bounds_read_mlp)
}  // namespace gbdmc

using namespace gbdmc;

// Set by the tcgen05 training GEMMs when a bounded tensor-core wait gave up.
__device__ int g_tc_gemm_err;

static int* tc_gemm_err_ptr() {
  static std::mutex mu;
  static int* ptr[64] = {nullptr};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> lock(mu);
  if (!ptr[dev] && cudaGetSymbolAddress((void**)&ptr[dev], g_tc_gemm_err) != cudaSuccess) ptr[dev] = nullptr;
  return ptr[dev];
}

namespace {
// The mma.sync training GEMMs over npair (1 or 2) operand sets.
int launch_gemm_xw(const float* x0, const float* x1, long long m, int k, const uint16_t* wt, const float* b0,
                   const float* b1, float* y0, float* y1, int npair, cudaStream_t s) {
  long long g = (m + 127) / 128;
  if (g > 4LL * num_sms()) g = 4LL * num_sms();
  const dim3 grid((unsigned)g, (unsigned)npair);
  if (k == 16)
    k_gemm_xw<16><<<grid, 256, 0, s>>>(x0, x1, m, wt, b0, b1, y0, y1);
  else
    k_gemm_xw<128><<<grid, 256, 0, s>>>(x0, x1, m, wt, b0, b1, y0, y1);
  return check_launch("gbdmc_mlp_gemm");
}

int launch_gemm_tn(const float* x0, const float* d0, const float* x1, const float* d1, long long m, int k, float* g,
                   int npair, cudaStream_t s) {
  long long grid = (m + 63) / 64;
  if (grid > 2LL * num_sms()) grid = 2LL * num_sms();
  const dim3 gr((unsigned)grid, (unsigned)npair);
  if (k == 16)
    k_gemm_tn<16><<<gr, 256, 0, s>>>(x0, d0, x1, d1, m, g);
  else
    k_gemm_tn<128><<<gr, 256, 0, s>>>(x0, d0, x1, d1, m, g);
  return check_launch("gbdmc_mlp_gemm_tn");
}
}  // namespace

extern "C" int gbdmc_mlp_gemm(const float* x, int64_t m, int32_t k, const uint16_t* wt, const float* bias, float* y,
                              void* stream) {
  if (!x || !wt || !y || m < 0 || (k != 16 && k != 128)) {
    set_error("gbdmc_mlp_gemm: invalid arguments (k must be 16 or 128)");
    return GBDMC_ERR_ARG;
  }
  if (m == 0) return GBDMC_OK;
  return launch_gemm_xw(x, x, m, k, wt, bias, bias, y, y, 1, (cudaStream_t)stream);
}

extern "C" int gbdmc_mlp_gemm_tn(const float* x, const float* d, int64_t m, int32_t k, float* g, void* stream) {
  if (!x || !d || !g || m < 0 || (k != 16 && k != 128)) {
    set_error("gbdmc_mlp_gemm_tn: invalid arguments (k must be 16 or 128)");
    return GBDMC_ERR_ARG;
  }
  if (m == 0) return GBDMC_OK;
  return launch_gemm_tn(x, d, x, d, m, k, g, 1, (cudaStream_t)stream);
}

extern "C" int gbdmc_mlp_gemm_tc(const float* x, int64_t m, int32_t k, const uint16_t* wt, const float* bias, float* y,
                              void* stream) {
  if (!x || !wt || !y || m < 0 || (k != 16 && k != 128)) {
    set_error("gbdmc_mlp_gemm_tc: invalid arguments (k must be 16 or 128)");
    return GBDMC_ERR_ARG;
  }
  if (m == 0) return GBDMC_OK;
  int* err = tc_gemm_err_ptr();
  if (!err) {
    set_error("gbdmc_mlp_gemm_tc: no device status word");
    return GBDMC_ERR_CUDA;
  }
  return launch_tc_gemm_xw(x, x, m, k, wt, bias, bias, y, y, 1, err, (cudaStream_t)stream);
}

extern "C" int gbdmc_mlp_gemm_tn_tc(const float* x, const float* d, int64_t m, int32_t k, float* g, void* stream) {
  if (!x || !d || !g || m < 0 || (k != 16 && k != 128)) {
    set_error("gbdmc_mlp_gemm_tn_tc: invalid arguments (k must be 16 or 128)");
    return GBDMC_ERR_ARG;
  }
  if (m == 0) return GBDMC_OK;
  int* err = tc_gemm_err_ptr();
  if (!err) {
    set_error("gbdmc_mlp_gemm_tn_tc: no device status word");
    return GBDMC_ERR_CUDA;
  }
  return launch_tc_gemm_tn(x, d, x, d, m, k, g, 1, err, (cudaStream_t)stream);
}

extern "C" int gbdmc_mlp_gemm_pair(const float* x0, const float* x1, int64_t m, int32_t k, const uint16_t* wt,
                                   const float* bias0, const float* bias1, float* y0, float* y1, int32_t engine,
                                   void* stream) {
  if (!x0 || !x1 || !wt || !y0 || !y1 || m < 0 || (k != 16 && k != 128) || (engine != 0 && engine != 1)) {
    set_error("gbdmc_mlp_gemm_pair: invalid arguments (k must be 16 or 128, engine 0 or 1)");
    return GBDMC_ERR_ARG;
  }
  if (m == 0) return GBDMC_OK;
  if (engine == 0) return launch_gemm_xw(x0, x1, m, k, wt, bias0, bias1, y0, y1, 2, (cudaStream_t)stream);
  int* err = tc_gemm_err_ptr();
  if (!err) {
    set_error("gbdmc_mlp_gemm_pair: no device status word");
    return GBDMC_ERR_CUDA;
  }
  return launch_tc_gemm_xw(x0, x1, m, k, wt, bias0, bias1, y0, y1, 2, err, (cudaStream_t)stream);
}

extern "C" int gbdmc_mlp_gemm_tn_pair(const float* x0, const float* d0, const float* x1, const float* d1, int64_t m,
                                      int32_t k, float* g, int32_t engine, void* stream) {
  if (!x0 || !d0 || !x1 || !d1 || !g || m < 0 || (k != 16 && k != 128) || (engine != 0 && engine != 1)) {
    set_error("gbdmc_mlp_gemm_tn_pair: invalid arguments (k must be 16 or 128, engine 0 or 1)");
    return GBDMC_ERR_ARG;
  }
  if (m == 0) return GBDMC_OK;
  if (engine == 0) return launch_gemm_tn(x0, d0, x1, d1, m, k, g, 2, (cudaStream_t)stream);
  int* err = tc_gemm_err_ptr();
  if (!err) {
    set_error("gbdmc_mlp_gemm_tn_pair: no device status word");
    return GBDMC_ERR_CUDA;
  }
  return launch_tc_gemm_tn(x0, d0, x1, d1, m, k, g, 2, err, (cudaStream_t)stream);
}

extern "C" int gbdmc_mlp_gemm_status(int32_t clear) {
  int* err = tc_gemm_err_ptr();
  if (!err) return -1;
  int v = 0;
  if (cudaMemcpy(&v, err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
  if (clear && v) {
    const int z = 0;
    if (cudaMemcpy(err, &z, sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess) return -1;
  }
  return v;
}

extern "C" int gbdmc_mlp_silu_fwd(const float* z, const float* zt, float* h, float* ht, int64_t n, void* stream) {
  if (!z || !h || n < 0 || ((zt == nullptr) != (ht == nullptr))) {
    set_error("gbdmc_mlp_silu_fwd: invalid arguments");
    return GBDMC_ERR_ARG;
  }
  if (n == 0) return GBDMC_OK;
  k_silu_fwd<<<ew_grid(n), 256, 0, (cudaStream_t)stream>>>(z, zt, h, ht, n);
  return check_launch("gbdmc_mlp_silu_fwd");
}

extern "C" int gbdmc_mlp_silu_bwd(const float* z, const float* zt, const float* hb, const float* htb, float* zb,
                                  float* ztb, int64_t n, float* gbias, void* stream) {
  if (!z || !hb || !zb || n < 0 || n % kH || (zt && (!htb || !ztb))) {
    set_error("gbdmc_mlp_silu_bwd: invalid arguments (n a multiple of 128)");
    return GBDMC_ERR_ARG;
  }
  if (n == 0) return GBDMC_OK;
  const long long rows = n / kH;
  long long grid = (rows + 1) / 2;
  if (grid > 2LL * num_sms()) grid = 2LL * num_sms();
  k_silu_bwd<<<(int)grid, 256, 0, (cudaStream_t)stream>>>(z, zt, hb, htb, zb, ztb, rows, gbias);
  return check_launch("gbdmc_mlp_silu_bwd");
}

extern "C" int gbdmc_mlp_head(const float* h3, const float* ht3, const float* w4, float b4, const float* b4_dev,
                              const float* e, const float* et, int64_t m, float w_e, float w_f, float* h3b, float* ht3b,
                              float* gw4, float* gb4, double* loss, void* stream) {
  if (!h3 || !w4 || !e || !h3b || !gw4 || !gb4 || !loss || m < 1 || (ht3 && (!et || !ht3b))) {
    set_error("gbdmc_mlp_head: invalid arguments");
    return GBDMC_ERR_ARG;
  }
  long long grid = (m + 7) / 8;
  if (grid > num_sms()) grid = num_sms();
  k_head<<<(int)grid, 256, 0, (cudaStream_t)stream>>>(h3, ht3, w4, b4, b4_dev, e, et, m, w_e, w_f, h3b, ht3b, gw4,
                                                       gb4, loss);
  return check_launch("gbdmc_mlp_head");
}

extern "C" int gbdmc_mlp_train_inputs(const double* x, const double* v, const double* grad, int64_t ld, int64_t b,
                                      const int64_t* ctl, uint64_t seed, const float* mu, const float* inv_sd,
                                      float e_mean, float e_scale, const float* b4_dev, int32_t sort_atoms,
                                      float* feat, float* tang, float* et, float* e, void* stream) {
  if (!x || !v || !grad || !ctl || !mu || !inv_sd || !b4_dev || !feat || !tang || !et || !e || b < 1 || ld < b ||
      sort_atoms < 0 || sort_atoms > 1) {
    set_error("gbdmc_mlp_train_inputs: invalid arguments");
    return GBDMC_ERR_ARG;
  }
  k_train_inputs<<<ew_grid(b), 256, 0, (cudaStream_t)stream>>>(x, v, grad, ld, b, (const long long*)ctl, seed, mu,
                                                                 inv_sd, e_mean, e_scale, b4_dev, sort_atoms, feat,
                                                                 tang, et, e);
  return check_launch("gbdmc_mlp_train_inputs");
}

extern "C" int gbdmc_mlp_adam_all(const gbdmc_adam_param_t* params, int32_t nq, float lr0, float lr_min, float b1,
                                  float b2, float eps, int64_t t0, int64_t steps, int64_t batch, int64_t* ctl,
                                  uint32_t* ticket, void* stream) {
  if (!params || nq < 1 || nq > 8 || !ctl || !ticket || steps < 1 || t0 < 0) {
    set_error("gbdmc_mlp_adam_all: invalid arguments (1 to 8 parameters)");
    return GBDMC_ERR_ARG;
  }
  AdamAll A{};
  A.nq = nq;
  A.start[0] = 0;
  for (int q = 0; q < nq; ++q) {
    const gbdmc_adam_param_t& P = params[q];
    if (!P.p || !P.g || !P.m || !P.v || P.n < 1 || ((P.wt || P.wn) && P.n != (int64_t)P.k * kH)) {
      set_error("gbdmc_mlp_adam_all: invalid parameter %d", q);
      return GBDMC_ERR_ARG;
    }
    A.p[q] = P.p, A.g[q] = P.g, A.m[q] = P.m, A.v[q] = P.v, A.wt[q] = P.wt, A.wn[q] = P.wn, A.k[q] = P.k;
    A.start[q + 1] = A.start[q] + P.n;
  }
  A.lr0 = lr0, A.lr_min = lr_min, A.b1 = b1, A.b2 = b2, A.eps = eps;
  A.t0 = t0, A.steps = steps, A.batch = batch;
  long long grid = (A.start[nq] + 255) / 256;
  if (grid > 2LL * num_sms()) grid = 2LL * num_sms();
  k_adam_all<<<(int)grid, 256, 0, (cudaStream_t)stream>>>(A, (long long*)ctl, ticket);
  return check_launch("gbdmc_mlp_adam_all");
}

extern "C" int gbdmc_mlp_adam(float* p, const float* g, float* m, float* v, int64_t n, float lr, float b1, float b2,
                              float eps, int32_t t, uint16_t* wt, uint16_t* wn, int32_t k, void* stream) {
  if (!p || !g || !m || !v || n < 1 || t < 1 || ((wt || wn) && n != (int64_t)k * kH)) {
    set_error("gbdmc_mlp_adam: invalid arguments");
    return GBDMC_ERR_ARG;
  }
  const float c1 = 1.0f / (1.0f - powf(b1, (float)t)), c2 = 1.0f / (1.0f - powf(b2, (float)t));
  k_adam<<<ew_grid(n), 256, 0, (cudaStream_t)stream>>>(p, g, m, v, n, lr, b1, b2, eps, c1, c2, wt, wn, k);
  return check_launch("gbdmc_mlp_adam");
}

extern "C" int gbdmc_dimer_features(const double* x, int64_t ld, int64_t n, const float* mu, const float* inv_sd,
                                    const double* vdir, const double* grad, float e_scale, float* feat, float* tang,
                                    float* et, int32_t sort_atoms, void* stream) {
  if (!x || !mu || !inv_sd || !feat || n < 0 || ld < n || (vdir && !tang) || (et && (!vdir || !grad)) ||
      sort_atoms < 0 || sort_atoms > 1) {
    set_error("gbdmc_dimer_features: invalid arguments");
    return GBDMC_ERR_ARG;
  }
  if (n == 0) return GBDMC_OK;
  k_features<double><<<ew_grid(n), 256, 0, (cudaStream_t)stream>>>(x, ld, n, mu, inv_sd, vdir, grad, e_scale, feat,
                                                                     vdir ? tang : nullptr, et, sort_atoms);
  return check_launch("gbdmc_dimer_features");
}

extern "C" int gbdmc_mlp_energy(const gbdmc_mlp_t* net, const float* x, int64_t ld, int64_t n, double* v,
                                int32_t* outside, int32_t* status, void* stream) {
  if (valid_net(net) && n == 0 && ld >= 0) return GBDMC_OK;  // no walkers: nothing is read or written
  if (!valid_net(net) || !x || !v || n < 0 || ld < n || (net->engine == 1 && !status) || net->engine < 0 ||
      net->engine > 1) {
    set_error("gbdmc_mlp_energy: invalid arguments");
    return GBDMC_ERR_ARG;
  }
  if (net->engine == 1) return launch_mlp_tc_energy(*net, x, ld, n, v, outside, status, (cudaStream_t)stream);
  int rc = set_mlp_smem((const void*)k_mlp_energy<float>);
  if (rc) return rc;
  long long g = (n + 127) / 128;
  if (g > 2LL * num_sms()) g = 2LL * num_sms();
  k_mlp_energy<float><<<(int)g, 256, mlp_smem_bytes(), (cudaStream_t)stream>>>(*net, x, ld, n, v, outside,
                                                                                 feat_box(*net));
  return check_launch("gbdmc_mlp_energy");
}

// Replica table of the surrogate path: tiles of `tpb` walkers (128 for the
// MLP kernels: 8 warps x 16 or 128 threads x 1; 256 for counts and branching).
// Replica table of a surrogate run: the 6-atom dimer, discrete weighting,
// fp32 deviates, optionally the dimer trial; nrep == 0 means one replica
// spanning the whole ld.
static int mlp_table(const gbdmc_sim_t* S, const gbdmc_replica_t* reps, int nrep, RepTable& T, const char* what,
                     int tpb = 128) {
  if (!S || S->natoms != 6 || S->pes.kind != GBDMC_PES_DIMER || S->weighting != GBDMC_DISCRETE ||
      (S->trial.kind != GBDMC_TRIAL_NONE && S->trial.kind != GBDMC_TRIAL_DIMER_GAUSS) || S->ld < 1 ||
      S->ld > (int64_t)INT32_MAX || (nrep == 0 && S->n0 < 1) || nrep < 0 || (nrep > 0 && !reps)) {
    set_error("%s: the surrogate path runs the 6-atom dimer, discrete weighting, no trial or the dimer trial",
              what);
    return GBDMC_ERR_ARG;
  }
  if (S->noise_mode == GBDMC_NOISE_PHILOX64) {
    set_error("%s: the surrogate path draws fp32 deviates (PHILOX32 or INJECTED)", what);
    return GBDMC_ERR_ARG;
  }
  gbdmc_replica_t one{};
  if (nrep == 0) {
    one.off = 0;
    one.cap = S->ld;
    one.n0 = S->n0;
    one.stream = S->replica_id;
    reps = &one;
    nrep = 1;
  }
  gbdmc_sim_t S2 = *S;
  S2.block_threads = tpb;
  return build_table(S2, reps, nrep, T, what);
}

// Tiles of the scratch layout: enough for any tile width >= kMinTPB.
static int64_t mlp_scratch_tiles(const gbdmc_sim_t* S, const gbdmc_replica_t* reps, int nrep) {
  if (nrep == 0) return (S->ld + kMinTPB - 1) / kMinTPB;
  int64_t t = 0;
  for (int r = 0; r < nrep; ++r) t += (reps[r].cap + kMinTPB - 1) / kMinTPB;
  return t;
}

extern "C" int gbdmc_mlp_batch_init(const gbdmc_sim_t* S, const gbdmc_mlp_t* net, const gbdmc_replica_t* reps,
                                    int32_t nrep, const gbdmc_walkers_f32_t* w, gbdmc_ctrl_t* ctrl, void* scratch,
                                    void* stream) {
  RepTable T;
  int rc = mlp_table(S, reps, nrep, T, "gbdmc_mlp_batch_init");
  if (rc) return rc;
  if (!valid_net(net) || !w || !w->x || !w->v || !ctrl || !scratch) {
    set_error("gbdmc_mlp_batch_init: invalid arguments");
    return GBDMC_ERR_ARG;
  }
  if (S->trial.kind != GBDMC_TRIAL_NONE && (!w->f || !w->lnpsi || !w->ke)) {
    set_error("gbdmc_mlp_batch_init: a trial needs f/lnpsi/ke walker arrays");
    return GBDMC_ERR_ARG;
  }
  rc = set_mlp_smem((const void*)k_mlp_init);
  if (rc) return rc;
  const ScratchLayout L = scratch_layout(scratch, slot_extent(S->ld, reps, nrep), mlp_scratch_tiles(S, reps, nrep));
  int grid = T.tile_off[T.nrep];
  if (grid > 2 * num_sms()) grid = 2 * num_sms();
  k_mlp_init<<<grid, 256, mlp_smem_bytes(), (cudaStream_t)stream>>>(*S, T, *net, *w, ctrl, L.part, step_f32(*S),
                                                                     feat_box(*net));
  return check_launch("gbdmc_mlp_batch_init");
}

extern "C" int gbdmc_mlp_sim_init(const gbdmc_sim_t* S, const gbdmc_mlp_t* net, const gbdmc_walkers_f32_t* w,
                                  gbdmc_ctrl_t* ctrl, void* scratch, void* stream) {
  return gbdmc_mlp_batch_init(S, net, nullptr, 0, w, ctrl, scratch, stream);
}

// Blocks of the single-pass counting kernel: at most the resident blocks
// (the tiles are taken by ticket, so the grid need not cover them).
static int count_branch_grid(int ntile, bool injected) {
  static int occ[2] = {0, 0};
  int& o = occ[injected ? 1 : 0];
  if (o == 0) {
    const cudaError_t e = injected ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                                         &o, k_count_branch_f32<GBDMC_NOISE_INJECTED>, kMaxTPB, 0)
                                   : cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                                         &o, k_count_branch_f32<GBDMC_NOISE_PHILOX32>, kMaxTPB, 0);
    if (e != cudaSuccess || o < 1) o = 1;
  }
  const int g = num_sms() * o;
  return ntile < g ? ntile : g;
}

extern "C" int gbdmc_mlp_batch_step(const gbdmc_sim_t* S, const gbdmc_mlp_t* net, const gbdmc_replica_t* reps,
                                    int32_t nrep, const gbdmc_walkers_f32_t* src, const gbdmc_walkers_f32_t* dst,
                                    gbdmc_ctrl_t* ctrl, void* scratch, double* audit, const gbdmc_noise_t* noise,
                                    void* stream) {
  const char* what = "gbdmc_mlp_batch_step";
  RepTable T;
  int rc = mlp_table(S, reps, nrep, T, what);
  if (rc) return rc;
  if (!valid_net(net) || !src || !dst || !src->x || !dst->x || !dst->v || !dst->idx || src->x == dst->x || !ctrl ||
      !scratch || !audit) {
    set_error("%s: invalid arguments", what);
    return GBDMC_ERR_ARG;
  }
  gbdmc_noise_t nz{};
  if (S->noise_mode == GBDMC_NOISE_INJECTED) {
    if (!noise || !noise->normal || !noise->u_branch || noise->ld_noise < 1 || T.nrep != 1) {
      set_error("%s: injected noise needs normal/u_branch buffers and one replica", what);
      return GBDMC_ERR_ARG;
    }
    nz = *noise;
  }
  if (net->engine < 0 || net->engine > 1) {
    set_error("%s: engine must be 0 (mma.sync) or 1 (tcgen05)", what);
    return GBDMC_ERR_ARG;
  }
  if (S->trial.kind != GBDMC_TRIAL_NONE) {
    if (net->engine != 1 || !src->f || !src->lnpsi || !src->ke || !dst->f || !dst->lnpsi || !dst->ke ||
        (S->noise_mode == GBDMC_NOISE_INJECTED && !nz.u_accept)) {
      set_error("%s: importance sampling needs engine 1 (tcgen05), f/lnpsi/ke walker arrays and, with "
                "injected noise, acceptance uniforms", what);
      return GBDMC_ERR_ARG;
    }
  }
  rc = set_mlp_smem((const void*)k_mlp_move_energy);
  if (rc) return rc;
  const ScratchLayout L = scratch_layout(scratch, slot_extent(S->ld, reps, nrep), mlp_scratch_tiles(S, reps, nrep));
  cudaStream_t s = (cudaStream_t)stream;
  int grid = T.tile_off[T.nrep];
  if (grid > 2 * num_sms()) grid = 2 * num_sms();
  const bool prof = g_prof.on && g_prof.count < ProfState::kSlots;
  cudaEvent_t* ev = prof ? g_prof.ev[g_prof.count] : nullptr;
  if (prof) cudaEventRecord(ev[0], s);
  if (net->engine == 1) {
    rc = launch_mlp_tc_move_energy(*S, T, *net, *src, *dst, ctrl, L.list, L.flags, audit, nz, s);
    if (rc) return rc;
  } else {
    k_mlp_move_energy<<<grid, 256, mlp_smem_bytes(), s>>>(*S, T, *net, *src, *dst, ctrl, L.list, L.flags, audit,
                                                          nz, feat_box(*net));
  }
  if (prof) cudaEventRecord(ev[1], s);
  // expected list length: the audit share of the walkers (the out-of-box fallbacks are few);
  // the grid holds one pass of it (two to four 128-thread blocks per SM)
  long long slots = 0;
  for (int r = 0; r < T.nrep; ++r) slots += T.cap[r];
  const long long expect = net->audit_every > 0 ? slots / net->audit_every : 0;
  long long ab = (expect + 127) / 128;
  if (ab < 2LL * num_sms()) ab = 2LL * num_sms();
  if (ab > 4LL * num_sms()) ab = 4LL * num_sms();
  RepTable T2;  // counting and branching on kCBW-walker tiles (256 threads per tile)
  rc = mlp_table(S, reps, nrep, T2, what, kMaxTPB);
  if (rc) return rc;
  int ntile2 = 0;
  for (int r = 0; r < T2.nrep; ++r) {
    T2.tile_off[r] = ntile2;
    ntile2 += (int)((T2.cap[r] + kCBW - 1) / kCBW);
  }
  T2.tile_off[T2.nrep] = ntile2;
  unsigned long long* tstat = reinterpret_cast<unsigned long long*>(L.prefix);
  launch_pdl(k_mlp_audit, (int)ab, 128, s, *S, T, *dst, ctrl, L.list, L.flags, audit, net->bias_beta, step_f32(*S),
             tstat, ntile2, L.sync);
  // counting, finalisation and branching in one pass (tile tickets, decoupled look-back)
  if (S->noise_mode == GBDMC_NOISE_INJECTED)
    launch_pdl(k_count_branch_f32<GBDMC_NOISE_INJECTED>, count_branch_grid(ntile2, true), T2.tpb, s, *S, T2, dst->v,
               ctrl, L.part, tstat, L.sync, dst->idx, nz);
  else
    launch_pdl(k_count_branch_f32<GBDMC_NOISE_PHILOX32>, count_branch_grid(ntile2, false), T2.tpb, s, *S, T2,
               dst->v, ctrl, L.part, tstat, L.sync, dst->idx, nz);
  if (prof) {
    cudaEventRecord(ev[2], s);
    ++g_prof.count;
  }
  return check_launch(what);
}

extern "C" int gbdmc_mlp_sim_step(const gbdmc_sim_t* S, const gbdmc_mlp_t* net, const gbdmc_walkers_f32_t* src,
                                  const gbdmc_walkers_f32_t* dst, gbdmc_ctrl_t* ctrl, void* scratch, double* audit,
                                  const gbdmc_noise_t* noise, void* stream) {
  return gbdmc_mlp_batch_step(S, net, nullptr, 0, src, dst, ctrl, scratch, audit, noise, stream);
}

extern "C" int gbdmc_mlp_batch_compact(const gbdmc_sim_t* S, const gbdmc_replica_t* reps, int32_t nrep,
                                       const gbdmc_walkers_f32_t* in, const gbdmc_walkers_f32_t* out,
                                       const gbdmc_ctrl_t* ctrl, void* stream) {
  RepTable T;
  int rc = mlp_table(S, reps, nrep, T, "gbdmc_mlp_batch_compact");
  if (rc) return rc;
  if (!in || !out || !in->x || !out->x || !in->v || !out->v || in->x == out->x || !ctrl) {
    set_error("gbdmc_mlp_batch_compact: invalid arguments");
    return GBDMC_ERR_ARG;
  }
  k_compact_f32<<<grid_for(T), T.tpb, 0, (cudaStream_t)stream>>>(*S, T, *in, *out, ctrl);
  return check_launch("gbdmc_mlp_batch_compact");
}

extern "C" int gbdmc_mlp_compact(const gbdmc_sim_t* S, const gbdmc_walkers_f32_t* in, const gbdmc_walkers_f32_t* out,
                                 const gbdmc_ctrl_t* ctrl, void* stream) {
  return gbdmc_mlp_batch_compact(S, nullptr, 0, in, out, ctrl, stream);
}

extern "C" int gbdmc_mlp_fw_begin(const gbdmc_sim_t* S, const gbdmc_replica_t* reps, int32_t nrep,
                                  const gbdmc_walkers_f32_t* w, const gbdmc_ctrl_t* ctrl, const double* vnn,
                                  const int32_t* outside, double* delta, double* part, void* stream) {
  RepTable T;
  int rc = mlp_table(S, reps, nrep, T, "gbdmc_mlp_fw_begin");
  if (rc) return rc;
  if (!w || !w->x || !w->who || !ctrl || !vnn || !outside || !delta || !part) {
    set_error("gbdmc_mlp_fw_begin: invalid arguments");
    return GBDMC_ERR_ARG;
  }
  k_fw<true><<<GBDMC_FW_BLOCKS, kFwThreads, 0, (cudaStream_t)stream>>>(T, ctrl, w->x, S->ld, w->who, vnn, outside,
                                                                        step_f32(*S), delta, part);
  return check_launch("gbdmc_mlp_fw_begin");
}

extern "C" int gbdmc_mlp_fw_end(const gbdmc_sim_t* S, const gbdmc_replica_t* reps, int32_t nrep,
                                const gbdmc_walkers_f32_t* w, const gbdmc_ctrl_t* ctrl, const double* delta,
                                double* part, void* stream) {
  RepTable T;
  int rc = mlp_table(S, reps, nrep, T, "gbdmc_mlp_fw_end");
  if (rc) return rc;
  if (!w || !w->who || !ctrl || !delta || !part) {
    set_error("gbdmc_mlp_fw_end: invalid arguments");
    return GBDMC_ERR_ARG;
  }
  k_fw<false><<<GBDMC_FW_BLOCKS, kFwThreads, 0, (cudaStream_t)stream>>>(T, ctrl, nullptr, S->ld, w->who, nullptr,
                                                                         nullptr, step_f32(*S), const_cast<double*>(delta),
                                                                         part);
  return check_launch("gbdmc_mlp_fw_end");
}
