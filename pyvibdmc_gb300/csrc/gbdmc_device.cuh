// Device building blocks of the walker step: counter-based RNG, Gaussian
// deviates, the analytic potentials with their hand-written adjoints, the
// internal-coordinate trial wave function with its first/second Cartesian
// derivatives, and block reductions.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <math_constants.h>
#include "gbdmc.h"
#include "gbdmc_ps_pes.cuh"

namespace gbdmc {

// ------------------------------------------------------------------ Philox
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
// easy as 1, 2, 3", SC'11): 10 rounds of two 32x32->64 multiplies with the
// published multipliers and Weyl key increments.
struct U4 {
  uint32_t x, y, z, w;
};

__device__ __forceinline__ U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint32_t lo0 = M0 * c.x, hi0 = __umulhi(M0, c.x);
    const uint32_t lo1 = M1 * c.z, hi1 = __umulhi(M1, c.z);
    c = U4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
    k0 += W0;
    k1 += W1;
  }
  return c;
}

// Counter layouts.  Index streams (LIN false): (walker index, step low word,
// stream slot | replica << 8, step high word).  Lineage streams (LIN true, the
// multi-step kernel, whose walkers are named by a 64-bit lineage key instead
// of their position): (key low word, key high word, step low word, stream slot
// | replica << 8 | 1 << 31); the top bit keeps the two kinds of counters apart
// (replica ids stay below 2^23).
template <bool LIN>
struct RngT {
  uint32_t k0, k1, i, s_lo, s_hi, rep;  // LIN: i, s_hi = the lineage key's low and high words
  uint32_t slot;
  U4 buf;
  int used;
  __device__ RngT(uint64_t seed, uint64_t step, uint64_t walker, uint32_t replica = 0)
      : k0((uint32_t)seed), k1((uint32_t)(seed >> 32)), i((uint32_t)walker), s_lo((uint32_t)step),
        s_hi(LIN ? (uint32_t)(walker >> 32) : (uint32_t)(step >> 32)), rep(replica), slot(0), used(4) {}
  __device__ __forceinline__ U4 block() {
    U4 c;
    if constexpr (LIN)
      c = U4{i, s_hi, s_lo, slot | (rep << 8) | 0x80000000u};
    else
      c = U4{i, s_lo, slot | (rep << 8), s_hi ^ (uint32_t)(i >> 31)};
    ++slot;
    return philox4x32_10(c, k0, k1);
  }
  __device__ __forceinline__ uint32_t next32() {
    if (used == 4) {
      buf = block();
      used = 0;
    }
    const uint32_t v = used == 0 ? buf.x : used == 1 ? buf.y : used == 2 ? buf.z : buf.w;
    ++used;
    return v;
  }
  // the stream position after k 32-bit draws of a fresh generator
  __device__ __forceinline__ void skip32(uint32_t k) {
    slot += k / 4;
    used = 4;
    if (k % 4) {
      buf = block();
      used = (int)(k % 4);
    }
  }
  // uniform in [0,1) with 53 random bits
  // the 53 random bits m of uniform53() = m * 2^-53
  __device__ __forceinline__ uint64_t bits53() {
    const uint64_t hi = next32(), lo = next32();
    return (hi << 21) | (lo >> 11);
  }
  // uniform in [0,1) with 53 random bits
  __device__ __forceinline__ double uniform53() { return (double)bits53() * 0x1.0p-53; }
  // two standard normals, Box-Muller in fp32 (u1 in (0,1] from 32 bits)
  __device__ __forceinline__ void normal2_f32(float& z0, float& z1) {
    const uint32_t a = next32(), b = next32();
    const float u1 = fmaf((float)a, 0x1.0p-32f, 0x1.0p-33f);
    const float u2 = (float)(b >> 8) * 0x1.0p-24f;
    const float rad = sqrtf(-2.0f * logf(u1));
    float s, c;
    sincospif(2.0f * u2, &s, &c);
    z0 = rad * c;
    z1 = rad * s;
  }
  // two standard normals, Box-Muller from the same draws with the special-
  // function unit's approximations (lg2.approx, sqrt.approx, sin/cos.approx on
  // the angle reduced to [-pi, pi)): ~1e-6 absolute error, for the fp32
  // surrogate walkers, whose moves need no more
  __device__ __forceinline__ void normal2_f32_fast(float& z0, float& z1) {
    const uint32_t a = next32(), b = next32();
    const float u1 = fmaf((float)a, 0x1.0p-32f, 0x1.0p-33f);  // (0, 1]
    const float u2 = (float)(b >> 8) * 0x1.0p-24f;             // [0, 1)
    const float r2 = -1.38629436f * __log2f(u1);               // -2 ln u1 >= 0
    float rad;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(rad) : "f"(r2));
    const float th = fmaf(6.28318531f, u2, -3.14159265f);  // the angle 2 pi u2 - pi
    float s, c;
    __sincosf(th, &s, &c);
    z0 = -rad * c;  // cos(2 pi u2) = -cos(th)
    z1 = -rad * s;
  }
  // two standard normals, Box-Muller in fp64 (53-bit uniforms)
  __device__ __forceinline__ void normal2_f64(double& z0, double& z1) {
    const double u1 = 1.0 - uniform53();  // (0,1]
    const double u2 = uniform53();
    const double rad = sqrt(-2.0 * log(u1));
    double s, c;
    sincospi(2.0 * u2, &s, &c);
    z0 = rad * c;
    z1 = rad * s;
  }
};
using Rng = RngT<false>;
using RngL = RngT<true>;

// The lineage key of copy r of a walker with key k, made at step `step`:
// copy 0 keeps k, copy r >= 1 takes the SplitMix64 finaliser (Steele, Lea,
// Flood 2014; Vigna's constants) of k + r * 0x9E3779B97F4A7C15 + step *
// 0xD1B54A32D192ED03.  The step keeps a walker that branches at two steps
// from giving two children the same key; every walker's key stays distinct
// (up to 64-bit collisions).
__host__ __device__ __forceinline__ uint64_t lineage_key(uint64_t k, int r, uint64_t step) {
  if (r == 0) return k;
  uint64_t z = k + (uint64_t)r * 0x9E3779B97F4A7C15ull + step * 0xD1B54A32D192ED03ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// fp64 -> fp32 with round-to-nearest-even on the integer pipes only (the
// fp64 pipe runs a conversion at about the cost of two FMAs per warp).  Equal
// to the (float) conversion except that results below the normal fp32 range
// flush to a signed zero; overflow gives a signed infinity, NaN a quiet NaN.
__device__ __forceinline__ float d2f_rn_int(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const uint32_t hi = (uint32_t)(b >> 32), lo = (uint32_t)b;
  const uint32_t sign = hi & 0x80000000u;
  const int e = (int)((hi >> 20) & 0x7FFu);
  const uint32_t m = ((hi & 0xFFFFFu) << 3) | (lo >> 29);  // the top 23 of 52 mantissa bits
  const uint32_t rest = lo & 0x1FFFFFFFu;                    // the 29 dropped bits
  uint32_t f = sign | ((uint32_t)(e - 1023 + 127) << 23) | m;
  f += (rest > 0x10000000u || (rest == 0x10000000u && (m & 1u))) ? 1u : 0u;  // a carry moves into the exponent
  const bool nan = e == 0x7FF && ((hi & 0xFFFFFu) | lo) != 0u;
  f = e < 1023 - 126 ? sign : f;                               // below the normal range
  f = e > 1023 + 127 ? (nan ? (sign | 0x7FC00000u) : (sign | 0x7F800000u)) : f;
  return __uint_as_float(f);
}

// m * 2^-53 < f for the 53-bit integer m of Rng::bits53 and a float f, with
// integer operations only: the exact value of (double)uniform53() < (double)f.
// For 0 < f < 1, f = F * 2^(e - 150) with F the 24-bit significand and e the
// biased exponent, so m * 2^-53 < f  <=>  m * 2^(97 - e) < F.
__device__ __forceinline__ bool u53_below(uint64_t m, float f) {
  if (!(f > 0.f)) return false;  // uniforms are >= 0; NaN compares false
  if (f >= 1.f) return true;     // uniforms are < 1
  const uint32_t b = __float_as_uint(f);
  const int e = (int)(b >> 23);
  const uint64_t F = e ? ((b & 0x7FFFFFu) | 0x800000u) : b;
  const int s = (e ? e : 1) - 97;
  if (s >= 0) return m < (F << s);                       // s <= 29 since f < 1: F << s < 2^53
  if (m >= (1ull << 24) || -s >= 24) return m == 0;      // otherwise m * 2^-s >= 2^24 > F
  return (m << -s) < F;
}

// Programmatic dependent launch.  A kernel launched with programmatic stream
// serialisation may start while the previous kernel of its stream is still
// running; griddepcontrol.wait returns once that kernel has completed and its
// memory is visible (immediately when there is no programmatic dependency).
// Every such kernel calls pdl_wait() before its first global-memory access,
// then pdl_trigger() so that its own successor can be launched early.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// 32-bit integer hash (SplitMix32-style finaliser) for audit sampling.
__device__ __forceinline__ uint32_t splitmix32(uint32_t z) {
  z += 0x9E3779B9u;
  z = (z ^ (z >> 16)) * 0x85EBCA6Bu;
  z = (z ^ (z >> 13)) * 0xC2B2AE35u;
  return z ^ (z >> 16);
}

// Exact float -> double widening with integer operations only (the FP64 pipe
// of GB300 is narrow; a conversion costs about two DFMA slots there).  Valid
// for zero and normal floats, which is everything the fp32 Box-Muller below
// produces: |z| is either 0 or >= 2^-11.5 * |cospi(0.5 - 2^-23)| > 1e-10.
__device__ __forceinline__ double widen_f32(float f) {
  const uint32_t b = __float_as_uint(f);
  const uint32_t e = (b >> 23) & 0xFFu;
  const uint64_t sign = (uint64_t)(b & 0x80000000u) << 32;
  const uint64_t mag = ((uint64_t)(e + 896u) << 52) | ((uint64_t)(b & 0x7FFFFFu) << 29);
  return __longlong_as_double((long long)(sign | (e ? mag : 0ull)));
}

// Fill z[0..n) with standard normals for the chosen noise mode.
template <int NM, int N, class G>
__device__ __forceinline__ void gen_normals(G& g, double (&z)[N]) {
  if constexpr (NM == GBDMC_NOISE_PHILOX32) {
#pragma unroll
    for (int k = 0; k < N; k += 2) {
      float a, b;
      g.normal2_f32(a, b);
      z[k] = widen_f32(a);
      if (k + 1 < N) z[k + 1] = widen_f32(b);
    }
  } else {
#pragma unroll
    for (int k = 0; k < N; k += 2) {
      double a, b;
      g.normal2_f64(a, b);
      z[k] = a;
      if (k + 1 < N) z[k + 1] = b;
    }
  }
}

// ------------------------------------------------------------- potentials
// 1/sqrt(y) for y > 0, else 0 (rsqrt: one special-function seed and Newton
// steps, about a third of the FP64 cost of sqrt followed by a division).
__device__ __forceinline__ double rsqrt_guard(double y) { return y > 0.0 ? rsqrt(y) : 0.0; }

// Local-mode water: two Morse OH stretches, harmonic bend 1/2 k (th-th_e)^2,
// stretch-stretch coupling krr dr1 dr2.  Atoms (o, h1, h2) inside x[3*A].
// With G: accumulates dV/dx into g.
template <bool G, int A>
__device__ __forceinline__ double h2o_lm(const double (&x)[3 * A], const double* p, int o, int h1, int h2,
                                         double (&g)[3 * A]) {
  const double De = p[0], a = p[1], re = p[2], kth = p[3], the = p[4], krr = p[5];
  double d1[3], d2[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    d1[d] = x[3 * h1 + d] - x[3 * o + d];
    d2[d] = x[3 * h2 + d] - x[3 * o + d];
  }
  const double r1 = sqrt(d1[0] * d1[0] + d1[1] * d1[1] + d1[2] * d1[2]);
  const double r2 = sqrt(d2[0] * d2[0] + d2[1] * d2[1] + d2[2] * d2[2]);
  const double dot = d1[0] * d2[0] + d1[1] * d2[1] + d1[2] * d2[2];
  const double inv12 = 1.0 / (r1 * r2);
  double c = dot * inv12;
  c = fmin(1.0, fmax(-1.0, c));
  const double th = acos(c);
  const double dr1 = r1 - re, dr2 = r2 - re;
  const double x1 = exp(-a * dr1), x2 = exp(-a * dr2);
  const double e1 = 1.0 - x1, e2 = 1.0 - x2;
  const double dth = th - the;
  const double v = De * e1 * e1 + De * e2 * e2 + 0.5 * kth * dth * dth + krr * dr1 * dr2;
  if constexpr (G) {
    // adjoint: dV/dr1, dV/dr2, dV/dth, then chain rule through r1, r2, theta
    const double vr1 = 2.0 * De * e1 * a * x1 + krr * dr2;
    const double vr2 = 2.0 * De * e2 * a * x2 + krr * dr1;
    const double vth = kth * dth;
    const double s = -rsqrt_guard(1.0 - c * c);
    const double ir1 = 1.0 / r1, ir2 = 1.0 / r2;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const double e1d = d1[d] * ir1, e2d = d2[d] * ir2;
      const double dch1 = d2[d] * inv12 - c * ir1 * e1d;
      const double dch2 = d1[d] * inv12 - c * ir2 * e2d;
      const double gh1 = vr1 * e1d + vth * s * dch1;
      const double gh2 = vr2 * e2d + vth * s * dch2;
      g[3 * h1 + d] += gh1;
      g[3 * h2 + d] += gh2;
      g[3 * o + d] -= gh1 + gh2;
    }
  }
  return v;
}

template <bool G, int A>
__device__ __forceinline__ double pes_ho(const double (&x)[3 * A], const double* p, double (&g)[3 * A]) {
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 3 * A; ++k) s = s + x[k] * x[k];
  if constexpr (G) {
#pragma unroll
    for (int k = 0; k < 3 * A; ++k) g[k] += p[0] * x[k];
  }
  return 0.5 * p[0] * s;
}

// Water dimer: monomers (0,1,2) and (3,4,5) + O-O Lennard-Jones + 9
// intermolecular charge pairs.
template <bool G>
__device__ __forceinline__ double pes_dimer(const double (&x)[18], const double* p, double (&g)[18]) {
  double v = h2o_lm<G, 6>(x, p, 0, 1, 2, g) + h2o_lm<G, 6>(x, p, 3, 4, 5, g);
  const double eps = p[6], sig = p[7], qH = p[8], qO = p[9];
  {
    double d[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) d[k] = x[9 + k] - x[k];
    const double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    const double ir2 = 1.0 / r2;
    const double s2 = sig * sig * ir2;
    const double s6 = s2 * s2 * s2;
    v += 4.0 * eps * (s6 * s6 - s6);
    if constexpr (G) {
      const double f = 4.0 * eps * (-12.0 * s6 * s6 + 6.0 * s6) * ir2;  // (dV/dr)/r
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        g[9 + k] += f * d[k];
        g[k] -= f * d[k];
      }
    }
  }
  const double q[3] = {qO, qH, qH};
#pragma unroll
  for (int i = 0; i < 3; ++i) {
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      double d[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) d[k] = x[3 * (3 + j) + k] - x[3 * i + k];
      const double ir = rsqrt_guard(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
      const double qq = q[i] * q[j];
      v += qq * ir;
      if constexpr (G) {
        const double f = -qq * ir * ir * ir;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          g[3 * (3 + j) + k] += f * d[k];
          g[3 * i + k] -= f * d[k];
        }
      }
    }
  }
  return v;
}

// Partridge-Schwenke water (vibpot, h2opes_v2.f:393-492, with the internal
// coordinates of calc_hoh_pot, calc_h2o_pot.f:13-27).  V = P(x1, x2, x3)
// exp(-b1 (dr1^2 + dr2^2)) + c1 + V_OH(r1) + V_OH(r2) + V_HH(r_HH) with
// x_k = (r_k - re)/re, x3 = cos(theta) - cos(theta_e); cos(theta) is taken
// from the bond vectors directly (the reference evaluates acos, then cos),
// and r_HH is the H-H distance (the reference's law of cosines).  The
// polynomial P and its partial derivatives are generated code
// (gbdmc_ps_pes.cuh).  With G: adds dV/dx to g.
template <bool G, int A>
__device__ __forceinline__ double h2o_ps(const double (&x)[3 * A], int o, int h1, int h2, double (&g)[3 * A]) {
  using namespace ps;
  double v1[3], v2[3], u[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    v1[d] = x[3 * h1 + d] - x[3 * o + d];
    v2[d] = x[3 * h2 + d] - x[3 * o + d];
    u[d] = x[3 * h1 + d] - x[3 * h2 + d];
  }
  const double r1 = sqrt(v1[0] * v1[0] + v1[1] * v1[1] + v1[2] * v1[2]);
  const double r2 = sqrt(v2[0] * v2[0] + v2[1] * v2[1] + v2[2] * v2[2]);
  const double rhh = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
  const double ir12 = 1.0 / (r1 * r2);
  const double c = (v1[0] * v2[0] + v1[1] * v2[1] + v1[2] * v2[2]) * ir12;
  const double dr1 = r1 - k_reoh, dr2 = r2 - k_reoh;
  const double x1 = dr1 / k_reoh, x2 = dr2 / k_reoh, x3 = c - k_ce;
  const double vhh = k_phh1 * exp(-k_phh2 * rhh);
  const double ex1 = exp(-k_alphaoh * (r1 - k_roh)), ex2 = exp(-k_alphaoh * (r2 - k_roh));
  const double voh1 = k_deoh * ex1 * (ex1 - 2.0), voh2 = k_deoh * ex2 * (ex2 - 2.0);
  const double E = exp(-k_b1 * (dr1 * dr1 + dr2 * dr2));
  const double P = poly(x1, x2, x3);
  const double v = P * E + kC1 + voh1 + voh2 + vhh;
  if constexpr (G) {
    const double ire = 1.0 / k_reoh;
    const double vr1 = (dpoly1(x1, x2, x3) * ire - 2.0 * k_b1 * dr1 * P) * E +
                       k_deoh * (-k_alphaoh * ex1) * (2.0 * ex1 - 2.0);
    const double vr2 = (dpoly2(x1, x2, x3) * ire - 2.0 * k_b1 * dr2 * P) * E +
                       k_deoh * (-k_alphaoh * ex2) * (2.0 * ex2 - 2.0);
    const double vc = dpoly3(x1, x2, x3) * E;
    const double vrh = -k_phh2 * vhh / rhh;  // (dV/dr_HH) / r_HH
    const double ir1 = 1.0 / r1, ir2 = 1.0 / r2;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const double e1 = v1[d] * ir1, e2 = v2[d] * ir2;
      const double dc1 = (e2 - c * e1) * ir1, dc2 = (e1 - c * e2) * ir2;  // dcos/dx_h1, dcos/dx_h2
      const double gh1 = vr1 * e1 + vc * dc1 + vrh * u[d];
      const double gh2 = vr2 * e2 + vc * dc2 - vrh * u[d];
      g[3 * h1 + d] += gh1;
      g[3 * h2 + d] += gh2;
      g[3 * o + d] -= vr1 * e1 + vr2 * e2 + vc * (dc1 + dc2);
    }
  }
  return v;
}

template <int PK, int A, bool G>
__device__ __forceinline__ double pes(const double (&x)[3 * A], const gbdmc_pes_t& P, double (&g)[3 * A]) {
  if constexpr (PK == GBDMC_PES_HO) {
    return pes_ho<G, A>(x, P.p, g);
  } else if constexpr (PK == GBDMC_PES_H2O_LM) {
    static_assert(A == 3, "H2O local-mode PES has 3 atoms");
    return h2o_lm<G, 3>(x, P.p, 0, 1, 2, g);
  } else if constexpr (PK == GBDMC_PES_H2O_PS) {
    static_assert(A == 3, "Partridge-Schwenke PES has 3 atoms");
    return P.p[0] != 0.0 ? h2o_ps<G, 3>(x, 2, 0, 1, g) : h2o_ps<G, 3>(x, 0, 1, 2, g);
  } else {
    static_assert(A == 6, "dimer PES has 6 atoms");
    return pes_dimer<G>(x, P.p, g);
  }
}

// ----------------------------------------------------------- trial psi
// psi, d1 = (dpsi/dx)/psi, d2 = (d2psi/dx2)/psi per Cartesian component.
// Separable Cartesian Gaussian, p[a] = alpha of atom a.
template <int A>
__device__ __forceinline__ double trial_ho(const double (&x)[3 * A], const double* p, double (&d1)[3 * A],
                                           double (&d2)[3 * A]) {
  double arg = 0.0, norm = 1.0;
#pragma unroll
  for (int k = 0; k < 3 * A; ++k) {
    const double al = p[k / 3];
    arg += al * x[k] * x[k];
    norm *= sqrt(sqrt(al * (1.0 / CUDART_PI)));
    d1[k] = -al * x[k];
    d2[k] = d1[k] * d1[k] - al;
  }
  return norm * exp(-0.5 * arg);
}

// Product of Gaussians in (r1, r2, theta) of one water (O vertex).  The
// Cartesian chain rule: with L_q = -alpha_q (q - q_e),
//   d1_k = sum_q L_q dq/dx_k
//   d2_k = d1_k^2 + sum_q [ -alpha_q (dq/dx_k)^2 + L_q d2q/dx_k^2 ]
// which equals the ChainRuleHelper d2psidx2 sum for a direct-product psi.
// h2o_trial_terms adds the water's d ln psi / dx_k to f[] and its
// d2 ln psi / dx_k^2 to t[] for the atoms (o, h1, h2) of x, and returns the
// exponent -1/2 sum_q alpha_q (q - q_e)^2.  The fp64 path instantiates it
// with T = double and double parameters; the fp32 surrogate move has its own
// form (dimer_trial_f32), which sums the second derivatives as it goes.
template <typename T>
__device__ __forceinline__ T rsqrt_guard_t(T y) {
  return y > T(0) ? rsqrt(y) : T(0);
}

template <typename T, int N, typename P>
__device__ __forceinline__ T h2o_trial_terms(const T (&x)[N], const P* p, int o, int h1, int h2, T (&f)[N],
                                             T (&t)[N]) {
  const T a1 = (T)p[0], a2 = (T)p[1], ath = (T)p[2], r1e = (T)p[3], r2e = (T)p[4], the = (T)p[5];
  T v1[3], v2[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    v1[d] = x[3 * h1 + d] - x[3 * o + d];
    v2[d] = x[3 * h2 + d] - x[3 * o + d];
  }
  const T r1 = sqrt(v1[0] * v1[0] + v1[1] * v1[1] + v1[2] * v1[2]);
  const T r2 = sqrt(v2[0] * v2[0] + v2[1] * v2[1] + v2[2] * v2[2]);
  const T ir1 = T(1) / r1, ir2 = T(1) / r2;
  const T g = ir1 * ir2;
  T c = (v1[0] * v2[0] + v1[1] * v2[1] + v1[2] * v2[2]) * g;
  c = fmin(T(1), fmax(T(-1), c));
  const T th = acos(c);
  const T one_m_c2 = T(1) - c * c;
  const T s = -rsqrt_guard_t(one_m_c2);  // dtheta/dcos
  const T s2 = c * s * s * s;            // d2theta/dcos2 = -c/(1-c^2)^1.5
  const T L1 = -a1 * (r1 - r1e), L2 = -a2 * (r2 - r2e), Lt = -ath * (th - the);
  const T ir1s = ir1 * ir1, ir2s = ir2 * ir2;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const T e1 = v1[d] * ir1, e2 = v2[d] * ir2;
    // cos(theta) first derivatives
    const T dch1 = v2[d] * g - c * ir1 * e1;
    const T dch2 = v1[d] * g - c * ir2 * e2;
    const T dco = -(dch1 + dch2);
    // cos(theta) diagonal second derivatives
    const T d2ch1 = c * (T(3) * e1 * e1 - T(1)) * ir1s - T(2) * v2[d] * e1 * ir1s * ir2;
    const T d2ch2 = c * (T(3) * e2 * e2 - T(1)) * ir2s - T(2) * v1[d] * e2 * ir2s * ir1;
    const T h = e1 * ir1 + e2 * ir2;
    const T d2co = T(2) * g - T(2) * (v1[d] + v2[d]) * g * h +
                   c * (h * h + (T(2) * e1 * e1 - T(1)) * ir1s + (T(2) * e2 * e2 - T(1)) * ir2s);
    // theta derivatives
    const T dth_o = s * dco, dth_1 = s * dch1, dth_2 = s * dch2;
    const T d2th_o = s2 * dco * dco + s * d2co;
    const T d2th_1 = s2 * dch1 * dch1 + s * d2ch1;
    const T d2th_2 = s2 * dch2 * dch2 + s * d2ch2;
    // r derivatives
    const T d2r1 = (T(1) - e1 * e1) * ir1, d2r2 = (T(1) - e2 * e2) * ir2;
    // O: depends on r1 (-e1), r2 (-e2), theta
    f[3 * o + d] += -L1 * e1 - L2 * e2 + Lt * dth_o;
    t[3 * o + d] += -a1 * e1 * e1 - a2 * e2 * e2 - ath * dth_o * dth_o + L1 * d2r1 + L2 * d2r2 + Lt * d2th_o;
    // H1: r1 (+e1), theta
    f[3 * h1 + d] += L1 * e1 + Lt * dth_1;
    t[3 * h1 + d] += -a1 * e1 * e1 - ath * dth_1 * dth_1 + L1 * d2r1 + Lt * d2th_1;
    // H2: r2 (+e2), theta
    f[3 * h2 + d] += L2 * e2 + Lt * dth_2;
    t[3 * h2 + d] += -a2 * e2 * e2 - ath * dth_2 * dth_2 + L2 * d2r2 + Lt * d2th_2;
  }
  return T(-0.5) * (a1 * (r1 - r1e) * (r1 - r1e) + a2 * (r2 - r2e) * (r2 - r2e) + ath * (th - the) * (th - the));
}

template <int A>
__device__ __forceinline__ double trial_h2o(const double (&x)[3 * A], const double* p, double (&d1o)[3 * A],
                                            double (&d2o)[3 * A]) {
  double t[3 * A];
#pragma unroll
  for (int k = 0; k < 3 * A; ++k) d1o[k] = t[k] = 0.0;
  const double e = h2o_trial_terms(x, p, 0, 1, 2, d1o, t);
  const double n = sqrt(sqrt(p[0] * p[1] * p[2] * (1.0 / (CUDART_PI * CUDART_PI * CUDART_PI))));
#pragma unroll
  for (int k = 0; k < 3 * A; ++k) d2o[k] = d1o[k] * d1o[k] + t[k];
  return n * exp(e);
}

// Water dimer (O,H,H,O,H,H): the water trial of each monomer times a Gaussian
// in the O-O distance, exp(-1/2 alpha_R (R - R_e)^2);
// p = alpha_r1, alpha_r2, alpha_th, r1e, r2e, theta_e, alpha_R, R_e.
// Returns ln psi without the normalisation; d1 = d ln psi/dx,
// d2 = (d2 psi/dx2)/psi = d1^2 + d2 ln psi/dx2 per Cartesian component.
template <typename T, typename P>
__device__ __forceinline__ T dimer_trial_log(const T (&x)[18], const P* p, T (&d1)[18], T (&d2)[18]) {
  T t[18];
#pragma unroll
  for (int k = 0; k < 18; ++k) d1[k] = t[k] = T(0);
  T e = h2o_trial_terms(x, p, 0, 1, 2, d1, t) + h2o_trial_terms(x, p, 3, 4, 5, d1, t);
  const T aR = (T)p[6], Re = (T)p[7];
  T v[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) v[d] = x[9 + d] - x[d];
  const T R = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  const T iR = T(1) / R;
  const T LR = -aR * (R - Re);
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const T ed = v[d] * iR;
    const T tt = -aR * ed * ed + LR * (T(1) - ed * ed) * iR;
    d1[9 + d] += LR * ed;
    d1[d] -= LR * ed;
    t[9 + d] += tt;
    t[d] += tt;
  }
  e += T(-0.5) * aR * (R - Re) * (R - Re);
#pragma unroll
  for (int k = 0; k < 18; ++k) d2[k] = d1[k] * d1[k] + t[k];
  return e;
}

template <int A>
__device__ __forceinline__ double trial_dimer(const double (&x)[3 * A], const double* p, double (&d1)[3 * A],
                                              double (&d2)[3 * A]) {
  const double e = dimer_trial_log(x, p, d1, d2);
  const double n1 = sqrt(sqrt(p[0] * p[1] * p[2] * (1.0 / (CUDART_PI * CUDART_PI * CUDART_PI))));
  return n1 * n1 * sqrt(sqrt(p[6] * (1.0 / CUDART_PI))) * exp(e);
}

template <int TK, int A>
__device__ __forceinline__ double trial(const double (&x)[3 * A], const gbdmc_trial_t& T, double (&d1)[3 * A],
                                        double (&d2)[3 * A]) {
  if constexpr (TK == GBDMC_TRIAL_HO_GAUSS) {
    return trial_ho<A>(x, T.p, d1, d2);
  } else if constexpr (TK == GBDMC_TRIAL_DIMER_GAUSS) {
    static_assert(A == 6, "dimer trial has 6 atoms");
    return trial_dimer<A>(x, T.p, d1, d2);
  } else {
    static_assert(A == 3, "H2O trial has 3 atoms");
    return trial_h2o<A>(x, T.p, d1, d2);
  }
}

// ----------------------------------------------------------- reductions
template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}
// Order-preserving map of a double onto int64 (total order of the non-NaN
// values, -0 < +0); min/max then run on the integer pipes.  Self-inverse.
__device__ __forceinline__ long long dkey(double v) {
  const long long b = __double_as_longlong(v);
  return b ^ ((b >> 63) & 0x7FFFFFFFFFFFFFFFLL);
}
__device__ __forceinline__ double dkey_inv(long long k) {
  return __longlong_as_double(k ^ ((k >> 63) & 0x7FFFFFFFFFFFFFFFLL));
}
__device__ __forceinline__ long long warp_min_key(long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = min(v, (long long)__shfl_down_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ long long warp_max_key(long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = max(v, (long long)__shfl_down_sync(0xffffffffu, v, o));
  return v;
}
// Warp sums of a and b with five fp64 adds per lane instead of ten: after one
// exchange lanes 0-15 reduce a and lanes 16-31 reduce b.  Fixed order; the
// sums are returned in every lane.
__device__ __forceinline__ void warp_sum2(double& a, double& b) {
  const bool hi = (threadIdx.x & 16) != 0;
  double keep = hi ? b : a;
  const double send = hi ? a : b;
  keep += __shfl_xor_sync(0xffffffffu, send, 16);
#pragma unroll
  for (int o = 8; o > 0; o >>= 1) keep += __shfl_xor_sync(0xffffffffu, keep, o);
  a = __shfl_sync(0xffffffffu, keep, 0);
  b = __shfl_sync(0xffffffffu, keep, 16);
}

__device__ __forceinline__ double warp_min(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_down_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
  return v;
}

// Inclusive warp scan of ints.
__device__ __forceinline__ int warp_incl_scan(int v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

}  // namespace gbdmc
