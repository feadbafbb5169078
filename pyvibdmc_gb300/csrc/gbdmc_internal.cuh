// Host/device helpers shared by the C-ABI translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>
#include "gbdmc.h"

namespace gbdmc {

constexpr int kMaxTPB = 256;  // largest tile (walkers per tile = threads per block)
constexpr int kMinTPB = 32;

// Compile-time bounds checking (-DGBDMC_BOUNDS_CHECK, the libgbdmc_bc.so
// build).  Every data-dependent index of the step kernels passes through
// GBDMC_BC(i, lo, hi, site): in the checked build an index outside [lo, hi)
// sets bit `site` of this translation unit's error word and is replaced by lo,
// so the access stays inside its buffer and the kernel carries on (it never
// traps); gbdmc_bounds_errors() returns the OR of the words.  In the normal
// build GBDMC_BC(i, ...) is i.
enum BoundsSite {
  kBcMoveGather = 0,     // gather index of the plain move outside the previous population
  kBcIsGather = 1,       // the same in the importance-sampled move
  kBcCompactGather = 2,  // the same in gbdmc_walkers_compact
  kBcExtGather = 3,      // the same in the move of gbdmc_sim_move
  kBcBranchWrite = 4,    // a copy past the replica's capacity (discrete branching)
  kBcContSlot = 5,       // continuous branching: a kill-list slot or argmax outside the population
  kBcRunShared = 6,      // multi-step kernel: a walker slot past the block's buffer
  kBcRunOut = 7,         // multi-step kernel: an output position past the capacity
  kBcSurrogateWrite = 8  // a copy past the capacity (surrogate single-pass branching)
};
#ifdef GBDMC_BOUNDS_CHECK
static __device__ unsigned g_bounds_word;
__device__ __forceinline__ long long bc_index(long long i, long long lo, long long hi, int site) {
  if (i < lo || i >= hi) {
    atomicOr(&g_bounds_word, 1u << site);
    return lo;
  }
  return i;
}
#define GBDMC_BC(i, lo, hi, site) ::gbdmc::bc_index((long long)(i), (long long)(lo), (long long)(hi), (site))
#define GBDMC_BOUNDS_READER(fn)                                                                   \
  unsigned fn(int clear) {                                                                        \
    unsigned v = 0;                                                                               \
    if (cudaMemcpyFromSymbol(&v, ::gbdmc::g_bounds_word, sizeof v) != cudaSuccess) return ~0u;   \
    if (clear) {                                                                                  \
      const unsigned z = 0;                                                                       \
      if (cudaMemcpyToSymbol(::gbdmc::g_bounds_word, &z, sizeof z) != cudaSuccess) return ~0u;    \
    }                                                                                             \
    return v;                                                                                     \
  }
#else
#define GBDMC_BC(i, lo, hi, site) (i)
#define GBDMC_BOUNDS_READER(fn) \
  unsigned fn(int) { return 0u; }
#endif
unsigned bounds_read_step(int clear);
unsigned bounds_read_run(int clear);
unsigned bounds_read_mlp(int clear);
unsigned bounds_read_mlp_tc(int clear);

// Per-tile partial results of a walker kernel (64 bytes).
struct Partial {
  long long c;       // sum of branch counts (or accepted moves)
  long long births;  // sum of max(c-1, 0)
  long long deaths;  // number of c == 0
  long long aux;
  double s0;         // sum of c*V (branching) / sum of V or V*w (init)
  double s1;         // sum of V (stats) / sum of w (init)
  double vmin;
  double vmax;
};
static_assert(sizeof(Partial) == 64, "Partial is 64 bytes");

// Replica table passed by value (__grid_constant__) to every step kernel.
struct RepTable {
  int32_t nrep;
  int32_t tpb;
  int32_t tile_off[GBDMC_MAX_REPLICAS + 1];  // first tile of each replica; [nrep] = total tiles
  int64_t off[GBDMC_MAX_REPLICAS];
  int64_t cap[GBDMC_MAX_REPLICAS];
  int64_t n0[GBDMC_MAX_REPLICAS];
  uint32_t stream[GBDMC_MAX_REPLICAS];
  float w_hi_f[GBDMC_MAX_REPLICAS];  // (n0 + n0/2) + 1 rounded down to fp32: float w > w_hi <=> w > w_hi_f
};

inline size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

// scratch layout: [Partial x tiles][int64 prefix x tiles][int32 counts x ld][int32 list x ld][uint8 flags x ld]
// [uint32 sync x 64]; the surrogate step's single-pass counting uses prefix[] as its tile status words and
// sync[0..1] as its tile ticket and exit counters
struct ScratchLayout {
  Partial* part;
  long long* prefix;
  int* counts;
  int* list;
  unsigned char* flags;
  unsigned int* sync;
  size_t bytes;
};

inline ScratchLayout scratch_layout(void* base, int64_t ld, int64_t max_tiles) {
  ScratchLayout L;
  size_t off = 0;
  char* b = (char*)base;
  L.part = (Partial*)(b + off);
  off += align256(sizeof(Partial) * (size_t)max_tiles);
  L.prefix = (long long*)(b + off);
  off += align256(sizeof(long long) * (size_t)max_tiles);
  L.counts = (int*)(b + off);
  off += align256(sizeof(int) * (size_t)ld);
  L.list = (int*)(b + off);
  off += align256(sizeof(int) * (size_t)ld);
  L.flags = (unsigned char*)(b + off);
  off += align256((size_t)ld);
  L.sync = (unsigned int*)(b + off);
  off += align256(64 * sizeof(unsigned int));
  L.bytes = off;
  return L;
}

// Slot extent of a replica table: the largest off + cap (the sim's ld for a
// single simulation, nrep == 0).  The scratch of a call is laid out over this
// extent, as the *_scratch_bytes functions size it, not over sim->ld: a batch
// may step a subset of the slots with a smaller scratch.
inline int64_t slot_extent(int64_t ld, const gbdmc_replica_t* reps, int nrep) {
  if (!reps || nrep < 1) return ld;
  int64_t e = 0;
  for (int r = 0; r < nrep; ++r) e = reps[r].off + reps[r].cap > e ? reps[r].off + reps[r].cap : e;
  return e;
}

// Upper bound of the tile count for any tile width >= kMinTPB.
inline int64_t max_tiles_for(const gbdmc_replica_t* reps, int nrep) {
  int64_t t = 0;
  for (int r = 0; r < nrep; ++r) t += (reps[r].cap + kMinTPB - 1) / kMinTPB;
  return t;
}

void set_error(const char* fmt, ...);
int check_launch(const char* what);

// Launch with programmatic stream serialisation: the kernel may start while
// its predecessor drains and must call pdl_wait() before it reads anything the
// predecessor writes; a failed launch is reported by the next check_launch.
template <typename... P, typename... Args>
inline void launch_pdl_smem(void (*kernel)(P...), int grid, int block, size_t smem, cudaStream_t s,
                            Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3((unsigned)block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  (void)cudaLaunchKernelEx(&cfg, kernel, static_cast<Args&&>(args)...);
}
template <typename... P, typename... Args>
inline void launch_pdl(void (*kernel)(P...), int grid, int block, cudaStream_t s, Args&&... args) {
  launch_pdl_smem(kernel, grid, block, 0, s, static_cast<Args&&>(args)...);
}

// Event-pair timing of the step kernels (gbdmc_prof_enable / gbdmc_prof_read).
struct ProfState {
  static constexpr int kSlots = 8192;
  bool on = false;
  bool created = false;
  int count = 0;
  cudaEvent_t ev[kSlots][3];
};
extern ProfState g_prof;

int num_sms();

// Host helpers of the step launchers shared between translation units.
int build_table(const gbdmc_sim_t& S, const gbdmc_replica_t* reps, int nrep, RepTable& T, const char* what);
int grid_for(const RepTable& T);
// Tiles per block iteration of the tile-batched branching pass (k_branch) and its grid.
struct TileBatch {
  int tpi, grid;
};
TileBatch tile_batch(const RepTable& T);
void launch_branch(const RepTable& T, int32_t* idx, const gbdmc_ctrl_t* ctrl, const long long* prefix,
                   const int* counts, cudaStream_t s);

// tcgen05 surrogate kernels (gbdmc_mlp_tc.cu)
int launch_mlp_tc_energy(const gbdmc_mlp_t& net, const float* x, long long ld, long long n, double* v, int* outside,
                         int* err, cudaStream_t s);
int launch_mlp_tc_move_energy(const gbdmc_sim_t& S, const RepTable& T, const gbdmc_mlp_t& net,
                              const gbdmc_walkers_f32_t& in, const gbdmc_walkers_f32_t& out, gbdmc_ctrl_t* ctrl,
                              int* list, unsigned char* flags, const double* audit, const gbdmc_noise_t& nz,
                              cudaStream_t s);
// the tcgen05 training GEMMs over npair (1 or 2) operand sets: set 1 is (x1, b1, y1) / (x1, d1)
int launch_tc_gemm_xw(const float* x0, const float* x1, long long m, int k, const uint16_t* wt, const float* b0,
                      const float* b1, float* y0, float* y1, int npair, int* err, cudaStream_t s);
int launch_tc_gemm_tn(const float* x0, const float* d0, const float* x1, const float* d1, long long m, int k,
                      float* g, int npair, int* err, cudaStream_t s);

}  // namespace gbdmc
