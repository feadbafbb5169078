// MLP surrogate forward on the 5th-generation tensor cores (tcgen05, sm_103a).
//
// A tile group of 128 threads processes tiles of 128 walkers, one walker per
// thread; a CTA holds G groups (G = 4 in the DMC step: 16 warps on the SM
// sharing one copy of the weights in shared memory, each group with its own
// activation buffer, mbarrier, named barrier and 128 TMEM columns).  The hidden layers are M=128 x N=128 x K tcgen05.mma instructions
// (kind::f16, BF16 operands, FP32 accumulation) issued by one thread:
//   A = activations of the tile, B = transposed weights, both in shared memory
//       in the canonical K-major no-swizzle layout (8-row x 16-byte core
//       matrices; K-adjacent cores contiguous, LBO = 128 B, SBO = KG*128 B);
//   D = a 128-lane x 128-column FP32 accumulator in tensor memory.
// The biases ride in the MMA: every A row ends in a constant block of 16
// columns (1, 1, 0, ..., 0) and every weight row in (b_hi, b_lo, 0, ..., 0),
// the bias split into two bf16 parts (~16 significant bits), so the
// accumulator holds W a + b and the epilogue adds nothing.
// Completion is signalled by tcgen05.commit to an mbarrier; every thread then
// reads its own walker's row (TMEM lane = thread) with tcgen05.ld, applies
// bias + SiLU and writes the BF16 row back as the next layer's A operand.
// Waits are bounded: a timeout sets GBDMC_ST_TIMEOUT, the CTA stops issuing,
// frees its tensor memory and returns.
#include "gbdmc_mlp_common.cuh"

namespace gbdmc {
namespace tc {

constexpr int kRows = 128;       // walkers per tile = MMA M = TMEM lanes
constexpr int kN = 128;          // hidden width = MMA N = TMEM columns
constexpr uint32_t kCols = 128;  // TMEM columns allocated per CTA
constexpr int kCore = 128;       // bytes of one 8 x 16-byte core matrix
constexpr int kThreads = 128;
constexpr int kKH = kN + 16;  // hidden-layer K: 128 activations + the constant block
constexpr int kKG = kKH / 8;  // core columns of an A buffer and of W2/W3 (18)
constexpr int kK1G = 4;       // core columns of W1: 16 features + the bias block

// Instruction descriptor, kind::f16: D fp32 (bits 4-5 = 1), A and B bf16
// (bits 7-9 = 1, 10-12 = 1), both K-major (bits 15, 16 = 0), N>>3 at 17, M>>4 at 24.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kN >> 3) << 17) |
                            ((uint32_t)(kRows >> 4) << 24);

template <int G>
struct TcSmemG {
  alignas(128) unsigned char w1[kN * 8 * kK1G * 2];  // N=128 x K=32: W1 | bias block
  alignas(128) unsigned char w2[kN * kKH * 2];       // N=128 x K=144: W2 | bias block
  alignas(128) unsigned char w3[kN * kKH * 2];
  alignas(128) unsigned char a[G][kRows * kKH * 2];  // per group: M=128 x K=144: activations | constants
  float w4[kN];
  alignas(8) unsigned long long mbar[G];
  uint32_t tmem_base;
};
constexpr int kGroups = 4;  // tile groups per CTA of the DMC step kernel
using TcSmem = TcSmemG<1>;
// the step kernel's shared memory (+1 KB alignment slack) within the 227 KB a CTA may use
static_assert(sizeof(TcSmemG<kGroups>) + 1024 <= 227 * 1024, "tile-group shared memory exceeds 227 KB");

// What one tile group owns: its activation buffer, mbarrier, TMEM columns,
// named barrier (bar.sync id over the group's 128 threads) and its thread index.
struct Grp {
  unsigned char* a;
  uint32_t mbar;
  uint32_t tmem;
  int bar;
  int lt;
};

__device__ __forceinline__ void group_sync(int bar) { asm volatile("bar.sync %0, 128;" ::"r"(bar) : "memory"); }
// OR of a predicate over the group (one barrier; the result is group-uniform)
__device__ __forceinline__ bool group_any(bool v, int bar) {
  int r;
  asm volatile(
      "{\n.reg .pred p, q;\nsetp.ne.s32 p, %1, 0;\nbar.red.or.pred q, %2, 128, p;\nselp.s32 %0, 1, 0, q;\n}\n"
      : "=r"(r)
      : "r"((int)v), "r"(bar)
      : "memory");
  return r != 0;
}
// byte offset of element (row, k) of a canonical K-major operand with KG core columns
__device__ __forceinline__ uint32_t canon_off(int row, int k, int KG) {
  return (uint32_t)(((row >> 3) * KG + (k >> 3)) * kCore + (row & 7) * 16 + (k & 7) * 2);
}

// tcgen05 shared-memory descriptor: start >> 4 (bits 0-13), LBO >> 4 (16-29),
// SBO >> 4 (32-45), version 1 (46-47), no swizzle (61-63 = 0).
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

__device__ __forceinline__ uint32_t saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void umma(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void umma_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
               : "memory");
}

__device__ __forceinline__ void mbar_init(uint32_t mbar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Bounded wait for the mbarrier phase `parity` to complete.
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
  for (int it = 0; it < (1 << 22); ++it) {
    uint32_t done;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(mbar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// 32 consecutive fp32 accumulator columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&r)[32]) {
  uint32_t u[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
      : "=r"(u[0]), "=r"(u[1]), "=r"(u[2]), "=r"(u[3]), "=r"(u[4]), "=r"(u[5]), "=r"(u[6]), "=r"(u[7]),
        "=r"(u[8]), "=r"(u[9]), "=r"(u[10]), "=r"(u[11]), "=r"(u[12]), "=r"(u[13]), "=r"(u[14]), "=r"(u[15]),
        "=r"(u[16]), "=r"(u[17]), "=r"(u[18]), "=r"(u[19]), "=r"(u[20]), "=r"(u[21]), "=r"(u[22]), "=r"(u[23]),
        "=r"(u[24]), "=r"(u[25]), "=r"(u[26]), "=r"(u[27]), "=r"(u[28]), "=r"(u[29]), "=r"(u[30]), "=r"(u[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int j = 0; j < 32; ++j) r[j] = __uint_as_float(u[j]);
}

// 8 bf16 weights times 1/2 (exact: a power of two on normal bf16 values)
__device__ __forceinline__ uint4 half_bf16x8(uint4 v) {
  const __nv_bfloat162 h = __float2bfloat162_rn(0.5f);
  uint32_t* w = reinterpret_cast<uint32_t*>(&v);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    __nv_bfloat162 b = *reinterpret_cast<__nv_bfloat162*>(&w[k]);
    b = __hmul2(b, h);
    w[k] = *reinterpret_cast<uint32_t*>(&b);
  }
  return v;
}

// bf16 bits of x (round to nearest even)
__device__ __forceinline__ uint32_t bf16_bits(float x) {
  const __nv_bfloat16 b = __float2bfloat16_rn(x);
  return (uint32_t)*reinterpret_cast<const uint16_t*>(&b);
}

// The bias block of weight row n: (b_hi, b_lo, 0, ..., 0) with b = hb the
// halved bias, b_hi = bf16(hb) and b_lo = bf16(hb - b_hi) (the difference is
// exact in fp32).  Two 16-byte chunks at columns kc .. kc + 15.
__device__ __forceinline__ void store_bias_block(unsigned char* w, int n, int kc, int KG, float hb) {
  const uint32_t hi = bf16_bits(hb);
  const uint32_t lo = bf16_bits(hb - __uint_as_float(hi << 16));
  *reinterpret_cast<uint4*>(w + canon_off(n, kc, KG)) = make_uint4(hi | (lo << 16), 0u, 0u, 0u);
  *reinterpret_cast<uint4*>(w + canon_off(n, kc + 8, KG)) = make_uint4(0u, 0u, 0u, 0u);
}

// The hidden layers' weights and biases are stored halved, so that each
// accumulator row is h = z/2 and the epilogue is silu_half(h).
template <int G>
__device__ void load_weights(TcSmemG<G>& sm, const gbdmc_mlp_t& net) {
  // Wt is n-major [128][K] in global; 16-byte chunks = 8 consecutive k of one row n
  for (int c = threadIdx.x; c < kN * 2; c += blockDim.x) {
    const int n = c >> 1, kg = c & 1;
    *reinterpret_cast<uint4*>(sm.w1 + canon_off(n, 8 * kg, kK1G)) =
        half_bf16x8(__ldg(reinterpret_cast<const uint4*>(net.w1t + n * 16 + 8 * kg)));
  }
  for (int c = threadIdx.x; c < kN * 16; c += blockDim.x) {
    const int n = c >> 4, kg = c & 15;
    *reinterpret_cast<uint4*>(sm.w2 + canon_off(n, 8 * kg, kKG)) =
        half_bf16x8(__ldg(reinterpret_cast<const uint4*>(net.w2t + n * kN + 8 * kg)));
    *reinterpret_cast<uint4*>(sm.w3 + canon_off(n, 8 * kg, kKG)) =
        half_bf16x8(__ldg(reinterpret_cast<const uint4*>(net.w3t + n * kN + 8 * kg)));
  }
  for (int n = threadIdx.x; n < kN; n += blockDim.x) {
    store_bias_block(sm.w1, n, 16, kK1G, 0.5f * net.b1[n]);
    store_bias_block(sm.w2, n, kN, kKG, 0.5f * net.b2[n]);
    store_bias_block(sm.w3, n, kN, kKG, 0.5f * net.b3[n]);
    sm.w4[n] = net.w4[n];
  }
}

// The constant block (1, 1, 0, ..., 0) of row `row` of an A buffer (written
// once; the epilogues only write columns 0 .. 127).
__device__ __forceinline__ void store_const_block(unsigned char* a, int row) {
  const uint32_t one = bf16_bits(1.f);
  *reinterpret_cast<uint4*>(a + canon_off(row, kN, kKG)) = make_uint4(one | (one << 16), 0u, 0u, 0u);
  *reinterpret_cast<uint4*>(a + canon_off(row, kN + 8, kKG)) = make_uint4(0u, 0u, 0u, 0u);
}

// SiLU of this thread's accumulator row (h = z/2 with the bias, see
// load_weights), written as the BF16 A row (columns 0 .. 127).
// The 32-column chunks are a rolled loop: sixteen warps at different points of
// the tile pipeline share the SM's instruction caches, and the fully unrolled
// epilogues tripled the kernel's code.
__device__ __forceinline__ void epilogue_to_a(const Grp& gp, uint32_t trow) {
  const int t = gp.lt;
#pragma unroll 1
  for (int c = 0; c < 4; ++c) {
    float r[32];
    tmem_ld32(trow + 32 * c, r);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      uint32_t p[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int j = 8 * q + 2 * e;
        p[e] = pack_bf16(silu_half(r[j]), silu_half(r[j + 1]));
      }
      *reinterpret_cast<uint4*>(gp.a + canon_off(t, 32 * c + 8 * q, kKG)) = make_uint4(p[0], p[1], p[2], p[3]);
    }
  }
}

// Issue the MMAs of one layer (thread 0) and wait for them.  A K-block of 16
// columns is 256 bytes further along a row of core matrices.  Layer 1 reads
// A's feature block (columns 0-15) and its constant block (128-143) against
// W1's two blocks; the hidden layers read all nine blocks.
__device__ __forceinline__ bool run_layer(const Grp& gp, uint32_t& phase, const unsigned char* w, bool first) {
  fence_proxy_async();
  tc_fence_before();
  group_sync(gp.bar);
  if (gp.lt == 0) {
    tc_fence_after();
    const uint32_t a0 = saddr(gp.a), b0 = saddr(w);
    if (first) {
      umma(gp.tmem, smem_desc(a0, kCore, kKG * kCore), smem_desc(b0, kCore, kK1G * kCore), 0u);
      umma(gp.tmem, smem_desc(a0 + 256u * (kN / 16), kCore, kKG * kCore), smem_desc(b0 + 256u, kCore, kK1G * kCore),
           1u);
    } else {
      for (int s = 0; s < kKG / 2; ++s)
        umma(gp.tmem, smem_desc(a0 + 256u * s, kCore, kKG * kCore), smem_desc(b0 + 256u * s, kCore, kKG * kCore),
             s > 0 ? 1u : 0u);
    }
    umma_commit(gp.mbar);
  }
  const bool ok = mbar_wait(gp.mbar, phase);
  phase ^= 1u;
  tc_fence_after();
  return ok;
}

// Network output (normalised, without b4) of this thread's feature row f.
// TMEM lane quarter of a warp = its warp index mod 4, which for a group of four
// aligned warps is the warp's index within the group.
template <int G>
__device__ __forceinline__ float forward_tile(TcSmemG<G>& sm, const Grp& gp, uint32_t& phase, const float (&f)[16],
                                              bool& ok) {
  const int t = gp.lt;
  const uint32_t trow = gp.tmem + ((uint32_t)(32 * (t >> 5)) << 16);
  {
    uint32_t p[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) p[q] = pack_bf16(f[2 * q], f[2 * q + 1]);
    *reinterpret_cast<uint4*>(gp.a + canon_off(t, 0, kKG)) = make_uint4(p[0], p[1], p[2], p[3]);
    *reinterpret_cast<uint4*>(gp.a + canon_off(t, 8, kKG)) = make_uint4(p[4], p[5], p[6], p[7]);
  }
  ok &= run_layer(gp, phase, sm.w1, true);
  epilogue_to_a(gp, trow);
  tc_fence_before();
  ok &= run_layer(gp, phase, sm.w2, false);
  epilogue_to_a(gp, trow);
  tc_fence_before();
  ok &= run_layer(gp, phase, sm.w3, false);
  float e = 0.f;
#pragma unroll 1
  for (int c = 0; c < 4; ++c) {
    float r[32];
    tmem_ld32(trow + 32 * c, r);
#pragma unroll
    for (int j = 0; j < 32; ++j) e += silu_half(r[j]) * sm.w4[32 * c + j];
  }
  tc_fence_before();
  group_sync(gp.bar);  // TMEM rows read and A free before the group's next tile
  return e;
}

// Weights into shared memory, G mbarriers, G x 128 TMEM columns (warp 0);
// returns the TMEM base address.
template <int G>
__device__ __forceinline__ uint32_t setup(TcSmemG<G>& sm, const gbdmc_mlp_t& net) {
  static_assert(G == 1 || G == 2 || G == 4, "TMEM allocations are powers of two of at least 32 columns");
  load_weights(sm, net);
  for (int i = threadIdx.x; i < G * kRows; i += blockDim.x) store_const_block(sm.a[i / kRows], i % kRows);
  if (threadIdx.x == 0)
    for (int g = 0; g < G; ++g) mbar_init(saddr(&sm.mbar[g]));
  if (threadIdx.x < 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(&sm.tmem_base)),
                 "r"(kCols * G)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_proxy_async();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  return sm.tmem_base;
}

template <int G>
__device__ __forceinline__ void teardown(uint32_t tmem) {
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (threadIdx.x < 32)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kCols * G) : "memory");
}

// Energies of n walkers (fp32 SoA coordinates) -- the tcgen05 twin of k_mlp_energy.
__global__ void __launch_bounds__(kThreads) k_mlp_tc_energy(const __grid_constant__ gbdmc_mlp_t net,
                                                             const float* __restrict__ x, long long ld, long long n,
                                                             double* __restrict__ v, int* __restrict__ outside,
                                                             int* __restrict__ err, const __grid_constant__ FeatBox B) {
  extern __shared__ __align__(1024) unsigned char smraw[];
  TcSmem& sm = *reinterpret_cast<TcSmem*>(smraw);
  uint32_t phase = 0;
  const uint32_t tmem = setup(sm, net);
  const Grp gp{sm.a[0], saddr(&sm.mbar[0]), tmem, 0, (int)threadIdx.x};
  bool ok = true;
  for (long long base = (long long)blockIdx.x * kRows; base < n; base += (long long)gridDim.x * kRows) {
    const long long i = base + threadIdx.x;
    float xs[18], f[16];
#pragma unroll
    for (int k = 0; k < 18; ++k) xs[k] = i < n ? x[k * ld + i] : (k < 3 ? 0.f : 1.f + k);
    const bool oob = walker_features(xs, B, f) && i < n;
    const float e = forward_tile(sm, gp, phase, f, ok);
    if (i < n) v[i] = (double)net.e_mean + (double)net.e_scale * (double)(e + net.b4);
    if (oob && outside) outside[i] = 1;
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) atomicExch(err, 1);
      break;
    }
  }
  teardown<1>(tmem);
}

// Phase 1 of a surrogate DMC step on tcgen05: gather + move + descriptors
// (one walker per thread), MLP forward, V; audit/out-of-box walkers are
// listed for k_mlp_audit exactly like the mma.sync path.
// The CTA holds kGroups tile groups; group g takes tiles blockIdx.x + g * gridDim.x,
// + gridDim.x * kGroups, ... (so a run of fewer tiles than 4 x SMs still spreads
// over all SMs).  Every decision that skips or ends a group's tile
// (replica stopped, tile beyond N, tensor-core timeout) is made uniform over
// the group with a barrier reduction, so the group's named barriers always
// see all of its 128 threads.
__global__ void __launch_bounds__(kThreads * kGroups) k_mlp_tc_move_energy(
    const __grid_constant__ gbdmc_sim_t S, const __grid_constant__ RepTable T, const __grid_constant__ gbdmc_mlp_t net,
    const gbdmc_walkers_f32_t in, gbdmc_walkers_f32_t out, gbdmc_ctrl_t* ctrls, int* list, unsigned char* flags,
    const double* audit, const gbdmc_noise_t nz, const __grid_constant__ StepF32 P,
    const __grid_constant__ FeatBox B) {
  extern __shared__ __align__(1024) unsigned char smraw[];
  TcSmemG<kGroups>& sm = *reinterpret_cast<TcSmemG<kGroups>*>(smraw);
  uint32_t phase = 0;
  // weights, mbarriers and TMEM first (inputs no kernel of the step writes),
  // then wait for the previous step's kernels (programmatic launch)
  const uint32_t tmem = setup(sm, net);
  pdl_wait();
  const double corr = audit ? audit[4] + audit[8] : 0.0;  // online bias correction (hartree)
  // V = (e_mean - corr) + e_scale (e + b4) (+ KE): the fp64 constants once per thread
  const double v_off = (double)net.e_mean - corr, v_scale = (double)net.e_scale;
  const int g = threadIdx.x >> 7;
  const Grp gp{sm.a[g], saddr(&sm.mbar[g]), tmem + (uint32_t)(g * kN), 1 + g, (int)(threadIdx.x & 127)};
  bool ok = true;
  const int64_t ld = S.ld;
  const int ntile = T.tile_off[T.nrep];
  for (int tile = blockIdx.x + g * gridDim.x; tile < ntile; tile += gridDim.x * kGroups) {
    const int r = replica_of(T, tile);
    gbdmc_ctrl_t* ctrl = ctrls + r;
    if (group_any(*(volatile int*)&ctrl->status != 0, gp.bar)) continue;  // replica stopped
    const long long n = ctrl->n;
    const long long step = ctrl->step;
    const int64_t base = T.off[r];
    const int64_t i0 = (int64_t)(tile - T.tile_off[r]) * kRows;
    if (i0 >= n) continue;  // group-uniform: n and the tile are the same for the whole group
    if (i0 == 0 && gp.lt == 0) store_count_params(ctrl);
    const int64_t i = i0 + gp.lt;
    float xs[18], f[16];
    bool acc = false;
    float ke = 0.f;
    if (i < n) {
      const int64_t src = base + (in.idx ? (int64_t)in.idx[base + i] : i);
      const int64_t dst = base + i;
      Rng rng(S.seed, (uint64_t)step, (uint64_t)i, T.stream[r]);
      const bool inj = S.noise_mode == GBDMC_NOISE_INJECTED;
      float z[18];
      if (S.trial.kind == GBDMC_TRIAL_DIMER_GAUSS) {
        // deviates first, then the walker's loads (measured faster here: the
        // trial's registers leave no room to hold both across the deviates)
        if (inj) {
#pragma unroll
          for (int k = 0; k < 18; ++k) z[k] = (float)nz.normal[k * nz.ld_noise + dst];
        } else {
#pragma unroll
          for (int k = 0; k < 18; k += 2) rng.normal2_f32_fast(z[k], z[k + 1]);
        }
        float fx[18];
#pragma unroll
        for (int k = 0; k < 18; ++k) {
          xs[k] = in.x[k * ld + src];
          fx[k] = in.f[k * ld + src];
        }
        float lp = in.lnpsi[src];
        ke = in.ke[src];
        // the acceptance uniform is drawn after the deviates (the stream order of the move)
        auto accept = [&](float met) {
          return inj ? (double)met > nz.u_accept[dst] : u53_below(rng.bits53(), met);
        };
        acc = is_move_f32(P, xs, fx, lp, ke, z, accept);
#pragma unroll
        for (int k = 0; k < 18; ++k) {
          out.x[k * ld + dst] = xs[k];
          out.f[k * ld + dst] = fx[k];
        }
        out.lnpsi[dst] = lp;
        out.ke[dst] = ke;
      } else {
        // the walker's loads first: their latency overlaps the deviates' arithmetic
#pragma unroll
        for (int k = 0; k < 18; ++k) xs[k] = in.x[k * ld + src];
        if (inj) {
#pragma unroll
          for (int k = 0; k < 18; ++k) z[k] = (float)nz.normal[k * nz.ld_noise + dst];
        } else {
#pragma unroll
          for (int k = 0; k < 18; k += 2) rng.normal2_f32_fast(z[k], z[k + 1]);
        }
#pragma unroll
        for (int k = 0; k < 18; ++k) {
          xs[k] += P.sigma[k / 3] * z[k];
          out.x[k * ld + dst] = xs[k];
        }
      }
      if (out.who && in.who) out.who[dst] = in.who[src];
      const bool oob = walker_features(xs, B, f);
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
      walker_features(xs, B, f);
    }
    if (S.trial.kind != GBDMC_TRIAL_NONE) {  // accepted moves of the replica (dt_eff = dt * accepted / N)
      const int nacc = __popc(__ballot_sync(0xffffffffu, acc));
      if ((gp.lt & 31) == 0 && nacc) atomicAdd((unsigned long long*)&ctrl->n_acc, (unsigned long long)nacc);
    }
    const float e = forward_tile(sm, gp, phase, f, ok);
    if (i < n) {
      const double v = v_off + v_scale * (double)(e + net.b4);
      out.v[base + i] = S.trial.kind != GBDMC_TRIAL_NONE ? v + (double)ke : v;
    }
    if (group_any(!ok, gp.bar)) {
      if (gp.lt == 0) atomicOr(&ctrl->status, GBDMC_ST_TIMEOUT);
      break;
    }
  }
  teardown<kGroups>(tmem);
}

// ------------------------------------------------------------ training GEMMs
// The GEMMs of a training step on the same tensor-core path: 128-thread CTAs,
// M = 128 x N = 128 MMAs with K = 16 per instruction, operands in shared
// memory in the canonical K-major layout, the fp32 accumulator in 128 TMEM
// columns, bounded mbarrier waits (a timeout sets *err and the CTA returns).

// Y[M x 128] = X[M x K] W[K x 128] (+ bias): tiles of 128 rows, one row per
// thread; CTA (x, y) takes output columns 64 y .. 64 y + 63 of tiles x, x +
// gridDim.x, ... (two CTAs per tile: twice the CTAs of a batch, half the
// epilogue each).  B = those 64 rows of Wt (n-major [128][K], bf16) staged
// once per CTA; A = the tile's rows of X rounded to bf16; the accumulator is
// 64 TMEM columns; the bias is added in the fp32 epilogue.
constexpr int kXwN = 64;
constexpr uint32_t kIdescN64 = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kXwN >> 3) << 17) |
                               ((uint32_t)(kRows >> 4) << 24);

template <int K>
struct XwSmem {
  alignas(128) unsigned char w[kXwN * K * 2];
  alignas(128) unsigned char a[kRows * K * 2];
  alignas(8) unsigned long long mbar;
  uint32_t tmem_base;
};

__device__ __forceinline__ uint32_t tc_alloc_setup(uint32_t* base_slot, unsigned long long* mbar,
                                                   uint32_t cols = kCols) {
  if (threadIdx.x == 0) mbar_init(saddr(mbar));
  if (threadIdx.x < 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(base_slot)),
                 "r"(cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_proxy_async();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  return *base_slot;
}

__device__ __forceinline__ void umma_n64(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(kIdescN64), "r"(accumulate)
      : "memory");
}

// blockIdx.z selects one of two operand sets that share W.
template <int K>
__global__ void __launch_bounds__(kThreads) k_tc_gemm_xw(const float* __restrict__ X0, const float* __restrict__ X1,
                                                         long long M, const uint16_t* __restrict__ Wt,
                                                         const float* __restrict__ bias0,
                                                         const float* __restrict__ bias1, float* __restrict__ Y0,
                                                         float* __restrict__ Y1, int* __restrict__ err) {
  const float* __restrict__ X = blockIdx.z ? X1 : X0;
  const float* __restrict__ bias = blockIdx.z ? bias1 : bias0;
  float* __restrict__ Y = blockIdx.z ? Y1 : Y0;
  constexpr int KG = K / 8;
  extern __shared__ __align__(1024) unsigned char smraw[];
  XwSmem<K>& sm = *reinterpret_cast<XwSmem<K>*>(smraw);
  const int t = threadIdx.x;
  const int n0 = kXwN * (int)blockIdx.y;  // this CTA's first output column
  for (int c = t; c < kXwN * KG; c += blockDim.x) {
    const int n = c / KG, kg = c % KG;
    *reinterpret_cast<uint4*>(sm.w + canon_off(n, 8 * kg, KG)) =
        __ldg(reinterpret_cast<const uint4*>(Wt + (size_t)(n0 + n) * K + 8 * kg));
  }
  const uint32_t tmem = tc_alloc_setup(&sm.tmem_base, &sm.mbar, kXwN);
  const uint32_t trow = tmem + ((uint32_t)(32 * (t >> 5)) << 16);
  uint32_t phase = 0;
  for (long long base = (long long)blockIdx.x * kRows; base < M; base += (long long)gridDim.x * kRows) {
    const long long r = base + t;
#pragma unroll
    for (int kg = 0; kg < KG; ++kg) {
      float4 lo = make_float4(0.f, 0.f, 0.f, 0.f), hi = lo;
      if (r < M) {
        lo = *reinterpret_cast<const float4*>(X + r * K + 8 * kg);
        hi = *reinterpret_cast<const float4*>(X + r * K + 8 * kg + 4);
      }
      *reinterpret_cast<uint4*>(sm.a + canon_off(t, 8 * kg, KG)) =
          make_uint4(pack_bf16(lo.x, lo.y), pack_bf16(lo.z, lo.w), pack_bf16(hi.x, hi.y), pack_bf16(hi.z, hi.w));
    }
    fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    if (t == 0) {
      tc_fence_after();
      const uint32_t a0 = saddr(sm.a), b0 = saddr(sm.w);
#pragma unroll
      for (int s = 0; s < K / 16; ++s)
        umma_n64(tmem, smem_desc(a0 + 256u * s, kCore, KG * kCore), smem_desc(b0 + 256u * s, kCore, KG * kCore),
                 s > 0 ? 1u : 0u);
      umma_commit(saddr(&sm.mbar));
    }
    const bool ok = mbar_wait(saddr(&sm.mbar), phase);
    phase ^= 1u;
    tc_fence_after();
    if (__syncthreads_or(!ok)) {
      if (t == 0) atomicExch(err, 1);
      break;
    }
#pragma unroll 1
    for (int c = 0; c < kXwN / 32; ++c) {
      float rr[32];
      tmem_ld32(trow + 32 * c, rr);
      if (r < M) {
#pragma unroll
        for (int j = 0; j < 32; j += 4) {
          const int col = n0 + 32 * c + j;
          float4 o = make_float4(rr[j], rr[j + 1], rr[j + 2], rr[j + 3]);
          if (bias) {
            o.x += bias[col];
            o.y += bias[col + 1];
            o.z += bias[col + 2];
            o.w += bias[col + 3];
          }
          *reinterpret_cast<float4*>(Y + r * kN + col) = o;
        }
      }
    }
    tc_fence_before();
    __syncthreads();  // TMEM rows read and A free before the next tile's MMAs
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (t < 32) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)kXwN)
                           : "memory");
}

// G[K x 128] += X[M x K]^T D[M x 128]: the sum over the M rows runs along the
// MMA's K.  A = X^T (rows = the K features; for K = 16 rows 16..127 stay
// zero), B = D^T (rows = the 128 outputs), both staged transposed in the
// canonical K-major layout 128 rows of X and D at a time: lane l of warp w
// loads column 32 w + l of 8 consecutive rows (each load a coalesced 128-byte
// row segment across the warp) and stores them as one 16-byte core-matrix
// row.  A CTA accumulates its chunks in TMEM and adds its K x 128 partial to
// G with fp32 vector atomics (four elements each).
struct TnSmem {
  alignas(128) unsigned char a[kRows * kRows * 2];
  alignas(128) unsigned char b[kN * kRows * 2];
  alignas(8) unsigned long long mbar;
  uint32_t tmem_base;
};

// 8 rows r0 .. r0 + 7 of column c of a row-major [rows][ld] fp32 matrix as
// 8 bf16 in one 16-byte value (rows at or past r_end read as 0).
__device__ __forceinline__ uint4 column8_bf16(const float* __restrict__ P, long long ld, long long r0,
                                              long long r_end, int c) {
  float v[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = (r0 + i < r_end) ? P[(r0 + i) * ld + c] : 0.f;
  return make_uint4(pack_bf16(v[0], v[1]), pack_bf16(v[2], v[3]), pack_bf16(v[4], v[5]), pack_bf16(v[6], v[7]));
}

// blockIdx.y selects one of two (X, D) pairs accumulated into the same G.
template <int K>
__global__ void __launch_bounds__(kThreads) k_tc_gemm_tn(const float* __restrict__ X0, const float* __restrict__ D0,
                                                         const float* __restrict__ X1, const float* __restrict__ D1,
                                                         long long M, long long rows_per_cta, float* __restrict__ G,
                                                         int* __restrict__ err) {
  const float* __restrict__ X = blockIdx.y ? X1 : X0;
  const float* __restrict__ D = blockIdx.y ? D1 : D0;
  constexpr int KG = kRows / 8;  // 16 core columns: 128 rows of X and D per chunk
  extern __shared__ __align__(1024) unsigned char smraw[];
  TnSmem& sm = *reinterpret_cast<TnSmem*>(smraw);
  const int t = threadIdx.x, w = t >> 5, l = t & 31;
  if (K < kRows)
    for (int c = t; c < kRows * kRows * 2 / 16; c += blockDim.x)
      reinterpret_cast<uint4*>(sm.a)[c] = make_uint4(0u, 0u, 0u, 0u);
  const uint32_t tmem = tc_alloc_setup(&sm.tmem_base, &sm.mbar);
  const uint32_t trow = tmem + ((uint32_t)(32 * w) << 16);
  const long long r_begin = (long long)blockIdx.x * rows_per_cta;
  const long long r_end = r_begin + rows_per_cta < M ? r_begin + rows_per_cta : M;
  uint32_t phase = 0;
  bool any = false, ok = true;
  for (long long c0 = r_begin; c0 < r_end; c0 += kRows) {
    // B = D^T: output column n = 32 w + l, the 16 blocks of 8 rows
#pragma unroll 8
    for (int sb = 0; sb < KG; ++sb)
      *reinterpret_cast<uint4*>(sm.b + canon_off(32 * w + l, 8 * sb, KG)) =
          column8_bf16(D, kN, c0 + 8 * sb, r_end, 32 * w + l);
    if (K == kRows) {
#pragma unroll 8
      for (int sb = 0; sb < KG; ++sb)
        *reinterpret_cast<uint4*>(sm.a + canon_off(32 * w + l, 8 * sb, KG)) =
            column8_bf16(X, K, c0 + 8 * sb, r_end, 32 * w + l);
    } else {  // K = 16: feature t % 16, blocks t / 16 and t / 16 + 8
      const int f = t % K;
      for (int sb = t / K; sb < KG; sb += kThreads / K)
        *reinterpret_cast<uint4*>(sm.a + canon_off(f, 8 * sb, KG)) = column8_bf16(X, K, c0 + 8 * sb, r_end, f);
    }
    fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    if (t == 0) {
      tc_fence_after();
      const uint32_t a0 = saddr(sm.a), b0 = saddr(sm.b);
#pragma unroll
      for (int s = 0; s < KG / 2; ++s)
        umma(tmem, smem_desc(a0 + 256u * s, kCore, KG * kCore), smem_desc(b0 + 256u * s, kCore, KG * kCore),
             (any || s > 0) ? 1u : 0u);
      umma_commit(saddr(&sm.mbar));
    }
    ok = mbar_wait(saddr(&sm.mbar), phase);
    phase ^= 1u;
    tc_fence_after();
    any = true;
    if (__syncthreads_or(!ok)) {
      if (t == 0) atomicExch(err, 1);
      break;
    }
  }
  if (any && ok) {
#pragma unroll 1
    for (int c = 0; c < 4; ++c) {
      float rr[32];
      tmem_ld32(trow + 32 * c, rr);
      if (t < K) {
#pragma unroll
        for (int j = 0; j < 32; j += 4)  // vector atomics: a quarter of the transactions
          atomicAdd(reinterpret_cast<float4*>(G + t * kN + 32 * c + j),
                    make_float4(rr[j], rr[j + 1], rr[j + 2], rr[j + 3]));
      }
    }
  }
  teardown<1>(tmem);
}

}  // namespace tc

int tc_smem_bytes() { return (int)sizeof(tc::TcSmem) + 1024; }
static int tc_group_smem_bytes() { return (int)sizeof(tc::TcSmemG<tc::kGroups>) + 1024; }

int launch_mlp_tc_energy(const gbdmc_mlp_t& net, const float* x, long long ld, long long n, double* v, int* outside,
                         int* err, cudaStream_t s) {
  const cudaError_t e =
      cudaFuncSetAttribute((const void*)tc::k_mlp_tc_energy, cudaFuncAttributeMaxDynamicSharedMemorySize, tc_smem_bytes());
  if (e != cudaSuccess) {
    set_error("cudaFuncSetAttribute: %s", cudaGetErrorString(e));
    return GBDMC_ERR_CUDA;
  }
  long long g = (n + tc::kRows - 1) / tc::kRows;
  if (g > 2LL * num_sms()) g = 2LL * num_sms();
  tc::k_mlp_tc_energy<<<(int)g, tc::kThreads, tc_smem_bytes(), s>>>(net, x, ld, n, v, outside, err, feat_box(net));
  return check_launch("gbdmc_mlp_energy (tcgen05)");
}

int launch_mlp_tc_move_energy(const gbdmc_sim_t& S, const RepTable& T, const gbdmc_mlp_t& net,
                              const gbdmc_walkers_f32_t& in, const gbdmc_walkers_f32_t& out, gbdmc_ctrl_t* ctrl,
                              int* list, unsigned char* flags, const double* audit, const gbdmc_noise_t& nz,
                              cudaStream_t s) {
  const cudaError_t e = cudaFuncSetAttribute((const void*)tc::k_mlp_tc_move_energy,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, tc_group_smem_bytes());
  if (e != cudaSuccess) {
    set_error("cudaFuncSetAttribute: %s", cudaGetErrorString(e));
    return GBDMC_ERR_CUDA;
  }
  // one CTA per SM (its shared memory and its 4 x 128 TMEM columns fill the SM)
  int g = T.tile_off[T.nrep];
  if (g > num_sms()) g = num_sms();
  launch_pdl_smem(tc::k_mlp_tc_move_energy, g, tc::kThreads * tc::kGroups, (size_t)tc_group_smem_bytes(), s, S, T,
                  net, in, out, ctrl, list, flags, audit, nz, step_f32(S), feat_box(net));
  return check_launch("gbdmc_mlp_sim_step (tcgen05)");
}

// The training GEMMs on tcgen05 (err: a device int set to 1 if a bounded
// tensor-core wait gave up; the caller's buffer).
int launch_tc_gemm_xw(const float* x0, const float* x1, long long m, int k, const uint16_t* wt, const float* b0,
                      const float* b1, float* y0, float* y1, int npair, int* err, cudaStream_t s) {
  // at least 70 KB of shared memory, so that at most three CTAs share an SM and
  // their 3 x 128 TMEM columns always fit (an allocation never waits)
  int smem = (int)(k == 16 ? sizeof(tc::XwSmem<16>) : sizeof(tc::XwSmem<128>)) + 1024;
  if (smem < 70 * 1024) smem = 70 * 1024;
  const void* f = k == 16 ? (const void*)tc::k_tc_gemm_xw<16> : (const void*)tc::k_tc_gemm_xw<128>;
  const cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) {
    set_error("cudaFuncSetAttribute: %s", cudaGetErrorString(e));
    return GBDMC_ERR_CUDA;
  }
  long long g = (m + tc::kRows - 1) / tc::kRows;
  if (g > 3LL * num_sms() / 2) g = 3LL * num_sms() / 2;
  // two CTAs per 128-row tile, 64 output columns each, per operand set
  const dim3 grid((unsigned)g, tc::kN / tc::kXwN, (unsigned)npair);
  if (k == 16)
    tc::k_tc_gemm_xw<16><<<grid, tc::kThreads, smem, s>>>(x0, x1, m, wt, b0, b1, y0, y1, err);
  else
    tc::k_tc_gemm_xw<128><<<grid, tc::kThreads, smem, s>>>(x0, x1, m, wt, b0, b1, y0, y1, err);
  return check_launch("gbdmc_mlp_gemm (tcgen05)");
}

int launch_tc_gemm_tn(const float* x0, const float* d0, const float* x1, const float* d1, long long m, int k,
                      float* g, int npair, int* err, cudaStream_t s) {
  int smem = (int)sizeof(tc::TnSmem) + 1024;
  if (smem < 70 * 1024) smem = 70 * 1024;  // at most three CTAs (3 x 128 TMEM columns) per SM
  const void* f = k == 16 ? (const void*)tc::k_tc_gemm_tn<16> : (const void*)tc::k_tc_gemm_tn<128>;
  const cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) {
    set_error("cudaFuncSetAttribute: %s", cudaGetErrorString(e));
    return GBDMC_ERR_CUDA;
  }
  // one 128-row chunk per CTA while the chunks of all operand sets fit three CTAs per SM
  const long long chunks = (m + tc::kRows - 1) / tc::kRows;
  const long long slots = 3LL * num_sms() / npair;
  long long per = 1;
  if (chunks > slots) per = (chunks + slots - 1) / slots;
  const long long grid = (chunks + per - 1) / per;
  const dim3 gr((unsigned)grid, (unsigned)npair);
  if (k == 16)
    tc::k_tc_gemm_tn<16><<<gr, tc::kThreads, smem, s>>>(x0, d0, x1, d1, m, per * tc::kRows, g, err);
  else
    tc::k_tc_gemm_tn<128><<<gr, tc::kThreads, smem, s>>>(x0, d0, x1, d1, m, per * tc::kRows, g, err);
  return check_launch("gbdmc_mlp_gemm_tn (tcgen05)");
}

GBDMC_BOUNDS_READER(bounds_read_mlp_tc)
}  // namespace gbdmc
