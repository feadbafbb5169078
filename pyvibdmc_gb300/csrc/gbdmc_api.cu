// C-ABI plumbing (error reporting, version, scratch sizing) and the plug-in
// boundary kernels: potential energy (+ adjoint gradient) and trial wave
// function (+ first/second derivatives) of a batch of walkers.
#include <stdarg.h>
#include "gbdmc_device.cuh"
#include "gbdmc_internal.cuh"

namespace gbdmc {

constexpr int kEvalTPB = 128;  // threads per block of the plug-in evaluation kernels
static inline int eval_grid(int64_t n) { return (int)((n + kEvalTPB - 1) / kEvalTPB); }

static thread_local char g_err[512] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

int check_launch(const char* what) {
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("%s: %s", what, cudaGetErrorString(e));
    return GBDMC_ERR_CUDA;
  }
  return GBDMC_OK;
}

// V (and optionally dV/dx) for walkers i < n, SoA with leading dimension ld.
template <int PK, int A, bool G>
__global__ void __launch_bounds__(kEvalTPB) k_pes_eval(const gbdmc_pes_t P, const double* __restrict__ x, int64_t n,
                                                    int64_t ld, double* __restrict__ v, double* __restrict__ g) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double xr[3 * A], gr[3 * A];
#pragma unroll
  for (int k = 0; k < 3 * A; ++k) {
    xr[k] = x[k * ld + i];
    gr[k] = 0.0;
  }
  v[i] = pes<PK, A, G>(xr, P, gr);
  if constexpr (G) {
#pragma unroll
    for (int k = 0; k < 3 * A; ++k) g[k * ld + i] = gr[k];
  }
}

template <int TK, int A>
__global__ void __launch_bounds__(kEvalTPB) k_trial_eval(const gbdmc_trial_t T, const double* __restrict__ x, int64_t n,
                                                      int64_t ld, double* __restrict__ psi, double* __restrict__ d1,
                                                      double* __restrict__ d2) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double xr[3 * A], a[3 * A], b[3 * A];
#pragma unroll
  for (int k = 0; k < 3 * A; ++k) xr[k] = x[k * ld + i];
  psi[i] = trial<TK, A>(xr, T, a, b);
#pragma unroll
  for (int k = 0; k < 3 * A; ++k) {
    if (d1) d1[k * ld + i] = a[k];
    if (d2) d2[k * ld + i] = b[k];
  }
}

template <int PK, int A>
static void launch_pes(const gbdmc_pes_t& P, const double* x, int64_t n, int64_t ld, double* v, double* g,
                       cudaStream_t s) {
  const int G = eval_grid(n);
  if (g)
    k_pes_eval<PK, A, true><<<G, kEvalTPB, 0, s>>>(P, x, n, ld, v, g);
  else
    k_pes_eval<PK, A, false><<<G, kEvalTPB, 0, s>>>(P, x, n, ld, v, g);
}

}  // namespace gbdmc

using namespace gbdmc;

extern "C" int gbdmc_abi_version(void) { return GBDMC_ABI_VERSION; }

extern "C" const char* gbdmc_last_error(void) { return g_err; }

extern "C" int gbdmc_bounds_check_enabled(void) {
#ifdef GBDMC_BOUNDS_CHECK
  return 1;
#else
  return 0;
#endif
}

extern "C" uint32_t gbdmc_bounds_errors(int32_t clear) {
  if (cudaDeviceSynchronize() != cudaSuccess) return ~0u;
  return bounds_read_step(clear) | bounds_read_run(clear) | bounds_read_mlp(clear) | bounds_read_mlp_tc(clear);
}


extern "C" int gbdmc_pes_eval(const gbdmc_pes_t* pes, const double* x, int64_t n, int64_t ld, double* v,
                              double* grad, void* stream) {
  // no walkers: nothing is read or written (an empty array may have no address)
  if (pes && n == 0 && ld >= 0) return GBDMC_OK;
  if (!pes || !x || !v || n < 0 || ld < n) {
    set_error("gbdmc_pes_eval: invalid arguments (n=%lld ld=%lld)", (long long)n, (long long)ld);
    return GBDMC_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const int A = pes->natoms;
  switch (pes->kind) {
    case GBDMC_PES_HO:
      if (A == 1) launch_pes<GBDMC_PES_HO, 1>(*pes, x, n, ld, v, grad, s);
      else if (A == 2) launch_pes<GBDMC_PES_HO, 2>(*pes, x, n, ld, v, grad, s);
      else if (A == 3) launch_pes<GBDMC_PES_HO, 3>(*pes, x, n, ld, v, grad, s);
      else if (A == 6) launch_pes<GBDMC_PES_HO, 6>(*pes, x, n, ld, v, grad, s);
      else {
        set_error("gbdmc_pes_eval: HO supports 1, 2, 3 or 6 atoms (got %d)", A);
        return GBDMC_ERR_ARG;
      }
      break;
    case GBDMC_PES_H2O_LM:
      if (A != 3) {
        set_error("gbdmc_pes_eval: H2O local-mode PES needs 3 atoms (got %d)", A);
        return GBDMC_ERR_ARG;
      }
      launch_pes<GBDMC_PES_H2O_LM, 3>(*pes, x, n, ld, v, grad, s);
      break;
    case GBDMC_PES_H2O_PS:
      if (pes->natoms != 3) {
        set_error("gbdmc_pes_eval: the Partridge-Schwenke PES has 3 atoms");
        return GBDMC_ERR_ARG;
      }
      launch_pes<GBDMC_PES_H2O_PS, 3>(*pes, x, n, ld, v, grad, s);
      break;
    case GBDMC_PES_DIMER:
      if (A != 6) {
        set_error("gbdmc_pes_eval: dimer PES needs 6 atoms (got %d)", A);
        return GBDMC_ERR_ARG;
      }
      launch_pes<GBDMC_PES_DIMER, 6>(*pes, x, n, ld, v, grad, s);
      break;
    default:
      set_error("gbdmc_pes_eval: unknown PES kind %d", pes->kind);
      return GBDMC_ERR_ARG;
  }
  return check_launch("gbdmc_pes_eval");
}

extern "C" int gbdmc_trial_eval(const gbdmc_trial_t* t, const double* x, int64_t n, int64_t ld, double* psi,
                                double* d1, double* d2, void* stream) {
  if (t && n == 0 && ld >= 0) return GBDMC_OK;  // no walkers: nothing is read or written
  if (!t || !x || !psi || n < 0 || ld < n) {
    set_error("gbdmc_trial_eval: invalid arguments");
    return GBDMC_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const int G = eval_grid(n);
  const int A = t->natoms;
  if (t->kind == GBDMC_TRIAL_HO_GAUSS) {
    if (A == 1) k_trial_eval<GBDMC_TRIAL_HO_GAUSS, 1><<<G, kEvalTPB, 0, s>>>(*t, x, n, ld, psi, d1, d2);
    else if (A == 3) k_trial_eval<GBDMC_TRIAL_HO_GAUSS, 3><<<G, kEvalTPB, 0, s>>>(*t, x, n, ld, psi, d1, d2);
    else {
      set_error("gbdmc_trial_eval: HO trial supports 1 or 3 atoms (got %d)", A);
      return GBDMC_ERR_ARG;
    }
  } else if (t->kind == GBDMC_TRIAL_H2O_GAUSS) {
    if (A != 3) {
      set_error("gbdmc_trial_eval: H2O trial needs 3 atoms (got %d)", A);
      return GBDMC_ERR_ARG;
    }
    k_trial_eval<GBDMC_TRIAL_H2O_GAUSS, 3><<<G, kEvalTPB, 0, s>>>(*t, x, n, ld, psi, d1, d2);
  } else if (t->kind == GBDMC_TRIAL_DIMER_GAUSS) {
    if (A != 6) {
      set_error("gbdmc_trial_eval: dimer trial needs 6 atoms (got %d)", A);
      return GBDMC_ERR_ARG;
    }
    k_trial_eval<GBDMC_TRIAL_DIMER_GAUSS, 6><<<G, kEvalTPB, 0, s>>>(*t, x, n, ld, psi, d1, d2);
  } else {
    set_error("gbdmc_trial_eval: unknown trial kind %d", t->kind);
    return GBDMC_ERR_ARG;
  }
  return check_launch("gbdmc_trial_eval");
}

extern "C" size_t gbdmc_struct_size(int32_t which) {
  switch (which) {
    case 0: return sizeof(gbdmc_sim_t);
    case 1: return sizeof(gbdmc_walkers_t);
    case 2: return sizeof(gbdmc_ctrl_t);
    case 3: return sizeof(gbdmc_noise_t);
    case 4: return sizeof(gbdmc_pes_t);
    case 5: return sizeof(gbdmc_trial_t);
    case 6: return sizeof(gbdmc_history_t);
    case 7: return sizeof(gbdmc_replica_t);
    case 8: return sizeof(gbdmc_mlp_t);
    case 9: return sizeof(gbdmc_walkers_f32_t);
    case 10: return sizeof(gbdmc_adam_param_t);
    case 11: return sizeof(gbdmc_host_walkers_t);
  }
  return 0;
}

// ------------------------------------------------------------ measurement
namespace gbdmc {
ProfState g_prof;

// 8 independent DFMA chains per thread.
__global__ void __launch_bounds__(256) k_fp64_fma(double* sink, long long iters) {
  double a0 = threadIdx.x * 1e-9, a1 = a0 + 1e-9, a2 = a0 + 2e-9, a3 = a0 + 3e-9;
  double a4 = a0 + 4e-9, a5 = a0 + 5e-9, a6 = a0 + 6e-9, a7 = a0 + 7e-9;
  const double m = 0.999999999, c = 1e-12;
  for (long long i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      a0 = fma(a0, m, c); a1 = fma(a1, m, c); a2 = fma(a2, m, c); a3 = fma(a3, m, c);
      a4 = fma(a4, m, c); a5 = fma(a5, m, c); a6 = fma(a6, m, c); a7 = fma(a7, m, c);
    }
  }
  const double r = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
  if (r == 12345.678) sink[blockIdx.x] = r;  // keeps the chains live
}
}  // namespace gbdmc

extern "C" int gbdmc_prof_enable(int32_t on) {
  if (on && !g_prof.created) {
    for (int i = 0; i < ProfState::kSlots; ++i) {
      for (int j = 0; j < 3; ++j) {
        if (cudaEventCreate(&g_prof.ev[i][j]) != cudaSuccess) {
          set_error("gbdmc_prof_enable: cudaEventCreate failed");
          return GBDMC_ERR_CUDA;
        }
      }
    }
    g_prof.created = true;
  }
  g_prof.on = on != 0;
  g_prof.count = 0;
  return GBDMC_OK;
}

extern "C" int gbdmc_prof_read(double* move_ms, int64_t* move_n, double* scat_ms, int64_t* scat_n) {
  double a = 0.0, b = 0.0;
  const int n = g_prof.count < ProfState::kSlots ? g_prof.count : ProfState::kSlots;
  for (int i = 0; i < n; ++i) {
    float t0 = 0.f, t1 = 0.f;
    if (cudaEventSynchronize(g_prof.ev[i][2]) != cudaSuccess) {
      set_error("gbdmc_prof_read: cudaEventSynchronize failed");
      return GBDMC_ERR_CUDA;
    }
    cudaEventElapsedTime(&t0, g_prof.ev[i][0], g_prof.ev[i][1]);
    cudaEventElapsedTime(&t1, g_prof.ev[i][1], g_prof.ev[i][2]);
    a += t0;
    b += t1;
  }
  if (move_ms) *move_ms = a;
  if (scat_ms) *scat_ms = b;
  if (move_n) *move_n = n;
  if (scat_n) *scat_n = n;
  g_prof.count = 0;
  return GBDMC_OK;
}

extern "C" int gbdmc_fp64_fma_probe(double* sink, int64_t iters, int32_t blocks, double* flops, void* stream) {
  if (!sink || iters < 1 || blocks < 1) {
    set_error("gbdmc_fp64_fma_probe: invalid arguments");
    return GBDMC_ERR_ARG;
  }
  k_fp64_fma<<<blocks, 256, 0, (cudaStream_t)stream>>>(sink, iters);
  if (flops) *flops = 2.0 * 8 * 16 * (double)iters * 256.0 * (double)blocks;
  return check_launch("gbdmc_fp64_fma_probe");
}
