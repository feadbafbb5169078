// Host-side helpers shared by the C-ABI translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>
#include "gbdmc.h"

namespace gbdmc {

constexpr int kTPB = 256;  // threads per block of the per-walker kernels

// Per-block partial results of a walker kernel (64 bytes).
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

inline int grid_for(int64_t ld) { return (int)((ld + kTPB - 1) / kTPB); }

inline size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

// scratch layout: [Partial x G][int64 prefix x G][int32 counts x ld][int32 list x ld][uint8 flags x ld]
struct ScratchLayout {
  Partial* part;
  long long* prefix;
  int* counts;
  int* list;
  unsigned char* flags;
  size_t bytes;
};

inline ScratchLayout scratch_layout(void* base, int64_t ld) {
  ScratchLayout L;
  const int G = grid_for(ld);
  size_t off = 0;
  char* b = (char*)base;
  L.part = (Partial*)(b + off);
  off += align256(sizeof(Partial) * (size_t)G);
  L.prefix = (long long*)(b + off);
  off += align256(sizeof(long long) * (size_t)G);
  L.counts = (int*)(b + off);
  off += align256(sizeof(int) * (size_t)ld);
  L.list = (int*)(b + off);
  off += align256(sizeof(int) * (size_t)ld);
  L.flags = (unsigned char*)(b + off);
  off += align256((size_t)ld);
  L.bytes = off;
  return L;
}

void set_error(const char* fmt, ...);

// Event-pair timing of the step kernels (gbdmc_prof_enable / gbdmc_prof_read).
struct ProfState {
  static constexpr int kSlots = 8192;
  bool on = false;
  bool created = false;
  int count = 0;
  cudaEvent_t ev[kSlots][3];
};
extern ProfState g_prof;
int check_launch(const char* what);

}  // namespace gbdmc
