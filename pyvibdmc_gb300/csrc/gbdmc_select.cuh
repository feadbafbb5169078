// np.argpartition(w, kth) inside one CTA, in the order NumPy's portable
// introselect produces.
//
// The reference picks the walkers replaced above the upper continuous-weight
// threshold as np.argpartition(w, k)[:k] (pyvibdmc.py:443-445) and clones the
// current argmax into them in that order (_branch, :340-356), so the order of
// the list decides which walker is copied where.  NumPy's select
// (numpy/_core/src/npysort/selection.cpp: introselect_, dumb_select_,
// median3_swap_, unguarded_partition_, median_of_median5_, median5_) is the
// algorithm restated here; the CPU oracle restates it line by line
// (argpartition_introselect) and a CPU test pins that restatement against
// np.argpartition itself with NumPy's SIMD select switched off.
//
// The permutation t[] (int per walker) lives in global scratch.  The
// quickselect partitions run block-wide: Hoare's unguarded partition swaps the
// j-th element >= pivot met from the left with the j-th element <= pivot met
// from the right for as long as the two stay apart, so with
//   L = ascending positions p > ll0 with !(w[p] < pivot),
//   R = descending positions q < hh0 with !(pivot < w[q]),
// the swapped pairs are (L[j], R[j]) for j < m* = #{j : L[j] < R[j]}, and the
// final pointers follow from L and R around m* (see block_partition).  Both
// lists come from block scans; the swaps are disjoint, so they run in
// parallel.  The median-of-medians pivot that NumPy takes once 2 msb(num)
// partitions have not finished (only for adversarial inputs) is computed by
// thread 0 sequentially, nested selections included.
#pragma once
#include <climits>
#include "gbdmc_internal.cuh"

namespace gbdmc {

constexpr int kSelCTA = 1024;

__device__ __forceinline__ int sel_msb(long long n) {
  int d = 0;
  while (n > 1) {
    n >>= 1;
    ++d;
  }
  return d;
}

__device__ __forceinline__ void sel_swap(int* t, long long i, long long j) {
  const int a = t[i];
  t[i] = t[j];
  t[j] = a;
}

// ---------------------------------------------- sequential (thread 0 only)
__device__ void seq_dumb_select(const double* w, int* t, long long off, long long num, long long k) {
  for (long long i = 0; i <= k; ++i) {
    long long mi = i;
    double mv = w[t[off + i]];
    for (long long q = i + 1; q < num; ++q) {
      const double x = w[t[off + q]];
      if (x < mv) {
        mi = q;
        mv = x;
      }
    }
    sel_swap(t, off + i, off + mi);
  }
}

__device__ void seq_median3_swap(const double* w, int* t, long long low, long long mid, long long high) {
  if (w[t[high]] < w[t[mid]]) sel_swap(t, high, mid);
  if (w[t[high]] < w[t[low]]) sel_swap(t, high, low);
  if (w[t[low]] < w[t[mid]]) sel_swap(t, low, mid);
  sel_swap(t, mid, low + 1);
}

__device__ int seq_median5(const double* w, int* t, long long o) {
  if (w[t[o + 1]] < w[t[o + 0]]) sel_swap(t, o + 1, o + 0);
  if (w[t[o + 4]] < w[t[o + 3]]) sel_swap(t, o + 4, o + 3);
  if (w[t[o + 3]] < w[t[o + 0]]) sel_swap(t, o + 3, o + 0);
  if (w[t[o + 4]] < w[t[o + 1]]) sel_swap(t, o + 4, o + 1);
  if (w[t[o + 2]] < w[t[o + 1]]) sel_swap(t, o + 2, o + 1);
  if (w[t[o + 3]] < w[t[o + 2]]) return w[t[o + 3]] < w[t[o + 1]] ? 1 : 3;
  return 2;
}

// median5 of each group of five in [off, off + num), moved to the front
// (the first half of median_of_median5_); returns the number of medians.
__device__ long long seq_median_groups(const double* w, int* t, long long off, long long num) {
  const long long nmed = num / 5;
  for (long long i = 0; i < nmed; ++i) {
    const int m = seq_median5(w, t, off + 5 * i);
    sel_swap(t, off + 5 * i + m, off + i);
  }
  return nmed;
}

__device__ void seq_unguarded_partition(const double* w, int* t, double pv, long long& ll, long long& hh) {
  for (;;) {
    do {
      ++ll;
    } while (w[t[ll]] < pv);
    do {
      --hh;
    } while (pv < w[t[hh]]);
    if (hh < ll) break;
    sel_swap(t, ll, hh);
  }
}

// introselect_ on t[off, off + num) for kth, with the nested selections of
// median_of_median5_ kept on an explicit stack in shared memory (each level is
// a fifth of its parent, so 16 levels cover any int32 size).  Called by one
// thread of the block.  Returns false only if the stack would overflow, which
// no size below 5^16 reaches.
struct SelFrame {
  long long off, num, kth, low, high, ll, hh, nmed;
  int depth, state;  // state 0: entry, 1: loop head, 2: median of medians returned
};

__device__ bool seq_introselect(const double* w, int* t, long long off0, long long num0, long long kth0) {
  __shared__ SelFrame st[16];
  int sp = 0;
  st[0] = SelFrame{off0, num0, kth0, 0, num0 - 1, 0, 0, 0, 0, 0};
  while (sp >= 0) {
    SelFrame& f = st[sp];
    const long long o = f.off;
    if (f.state == 0) {
      if (f.kth - f.low < 3) {
        seq_dumb_select(w, t, o + f.low, f.high - f.low + 1, f.kth - f.low);
        --sp;
        continue;
      }
      if (f.kth == f.num - 1) {  // inexact type: the last maximum to the end
        long long mi = f.low;
        double mv = w[t[o + f.low]];
        for (long long q = f.low + 1; q < f.num; ++q) {
          const double x = w[t[o + q]];
          if (!(x < mv)) {
            mi = q;
            mv = x;
          }
        }
        sel_swap(t, o + f.kth, o + mi);
        --sp;
        continue;
      }
      f.depth = 2 * sel_msb(f.num);
      f.state = 1;
    }
    if (f.state == 1) {
      if (!(f.low + 1 < f.high)) {
        if (f.high == f.low + 1 && w[t[o + f.high]] < w[t[o + f.low]]) sel_swap(t, o + f.high, o + f.low);
        --sp;
        continue;
      }
      f.ll = f.low + 1;
      f.hh = f.high;
      if (f.depth > 0 || f.hh - f.ll < 5) {
        seq_median3_swap(w, t, o + f.low, o + f.low + (f.high - f.low) / 2, o + f.high);
      } else {
        f.nmed = seq_median_groups(w, t, o + f.ll, f.hh - f.ll);
        f.state = 2;
        if (f.nmed > 2) {
          if (sp + 1 >= 16) return false;
          st[sp + 1] = SelFrame{o + f.ll, f.nmed, f.nmed / 2, 0, f.nmed - 1, 0, 0, 0, 0, 0};
          ++sp;
          continue;
        }
      }
    }
    if (f.state == 2) {  // the median of the medians sits at ll + nmed/2
      const long long mid = f.ll + f.nmed / 2;
      sel_swap(t, o + mid, o + f.low);
      f.ll -= 1;
      f.hh += 1;
      f.state = 1;
    }
    f.depth -= 1;
    long long ll = o + f.ll, hh = o + f.hh;
    seq_unguarded_partition(w, t, w[t[o + f.low]], ll, hh);
    sel_swap(t, o + f.low, hh);
    ll -= o;
    hh -= o;
    if (hh >= f.kth) f.high = hh - 1;
    if (hh <= f.kth) f.low = ll;
  }
  return true;
}

// --------------------------------------------------------- block helpers
// Inclusive block scan of an int (kSelCTA threads); `tot` receives the sum.
__device__ __forceinline__ int sel_block_scan(int v, int& tot) {
  __shared__ int ws[kSelCTA / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) ws[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int s = ws[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    ws[lane] = s;
  }
  __syncthreads();
  const int res = x + (wid ? ws[wid - 1] : 0);
  tot = ws[kSelCTA / 32 - 1];
  __syncthreads();
  return res;
}

__device__ __forceinline__ long long sel_block_sum(long long v) {
  __shared__ long long ws[kSelCTA / 32];
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) ws[wid] = v;
  __syncthreads();
  if (wid == 0) {
    long long s = warp_sum(ws[lane]);
    if (lane == 0) ws[0] = s;
  }
  __syncthreads();
  const long long r = ws[0];
  __syncthreads();
  return r;
}

// Position of the minimum (MAX: maximum) of w[t[q]] over q in [from, n):
// the first one on ties, the last one with LAST.
template <bool MAX, bool LAST>
__device__ long long sel_block_argext(const double* w, const int* t, long long from, long long n) {
  __shared__ double sv[kSelCTA / 32];
  __shared__ long long si[kSelCTA / 32];
  double bv = 0.0;
  long long bi = -1;
  for (long long q = from + threadIdx.x; q < n; q += kSelCTA) {
    const double x = w[t[q]];
    if (bi < 0 || (MAX ? x > bv : x < bv) || (LAST && x == bv)) {
      bv = x;
      bi = q;
    }
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int pass = 0; pass < 2; ++pass) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double ov = __shfl_down_sync(0xffffffffu, bv, o);
      const long long oi = __shfl_down_sync(0xffffffffu, bi, o);
      if (oi >= 0 && (bi < 0 || (MAX ? ov > bv : ov < bv) || (ov == bv && (LAST ? oi > bi : oi < bi)))) {
        bv = ov;
        bi = oi;
      }
    }
    if (pass == 1) break;
    if (lane == 0) {
      sv[wid] = bv;
      si[wid] = bi;
    }
    __syncthreads();
    if (wid != 0) break;
    bv = sv[lane];
    bi = si[lane];
  }
  if (threadIdx.x == 0) si[0] = bi;
  __syncthreads();
  const long long r = si[0];
  __syncthreads();
  return r;
}

// Hoare's unguarded partition of t[low..high] around pv = w[t[low]],
// starting from the pointers (ll0, hh0); returns the final (ll, hh) in
// out[0..1] (shared) after applying every swap.  Lpos (n ints) and fl (n
// bytes) are scratch.
__device__ void block_partition(const double* w, int* t, long long low, long long high, long long ll0,
                                long long hh0, int* Lpos, unsigned char* fl, long long* out) {
  __shared__ long long s_run[2];
  const double pv = w[t[low]];
  // pass 1: element classes (bit 0: a left stop, bit 1: a right stop) and their totals
  long long cl = 0, cr = 0;
  for (long long p = low + threadIdx.x; p <= high; p += kSelCTA) {
    const double x = w[t[p]];
    const int ge = (p > ll0 && !(x < pv)) ? 1 : 0;
    const int le = (p < hh0 && !(pv < x)) ? 1 : 0;
    fl[p] = (unsigned char)(ge | (le << 1));
    cl += ge;
    cr += le;
  }
  const long long totL = sel_block_sum(cl);
  const long long totR = sel_block_sum(cr);
  // pass 2: left stops in ascending order (Lpos) and m* = #{j : L[j] < R[j]}.
  // L[j] = p < R[j] <=> at least j+1 right stops lie above p <=> j+1 <= totR - #right stops <= p
  if (threadIdx.x == 0) s_run[0] = s_run[1] = 0;
  __syncthreads();
  long long mcount = 0;
  for (long long c = low; c <= high; c += kSelCTA) {
    const long long p = c + threadIdx.x;
    const int f = p <= high ? fl[p] : 0;
    const int ge = f & 1, le = (f >> 1) & 1;
    int tot;
    const int inc = sel_block_scan(ge | (le << 16), tot);
    const long long rl = s_run[0] + ((inc & 0xffff) - ge);  // rank among left stops
    const long long cle = s_run[1] + (inc >> 16);           // right stops at positions <= p
    if (ge) {
      Lpos[rl] = (int)p;
      if (rl + 1 <= totR - cle) ++mcount;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      s_run[0] += tot & 0xffff;
      s_run[1] += tot >> 16;
    }
    __syncthreads();
  }
  const long long mstar = sel_block_sum(mcount);
  // pass 3: right stop with descending rank j < m* swaps with L[j]; record R around m*
  __shared__ long long s_r[3];  // R[m*-1], R[m*], R[m*+1]
  if (threadIdx.x == 0) {
    s_run[1] = 0;
    s_r[0] = LLONG_MAX;  // R[-1] = +inf
    s_r[1] = s_r[2] = LLONG_MIN;
  }
  __syncthreads();
  for (long long c = low; c <= high; c += kSelCTA) {
    const long long p = c + threadIdx.x;
    const int le = p <= high ? (fl[p] >> 1) & 1 : 0;
    int tot;
    const int inc = sel_block_scan(le, tot);
    if (le) {
      const long long j = totR - 1 - (s_run[1] + inc - 1);
      if (j < mstar) sel_swap(t, p, Lpos[j]);
      if (j >= mstar - 1 && j <= mstar + 1) s_r[j - mstar + 1] = p;
    }
    __syncthreads();
    if (threadIdx.x == 0) s_run[1] += tot;
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    auto Lj = [&](long long j) -> long long {
      if (j < 0) return LLONG_MIN;
      if (j >= totL) return LLONG_MAX;
      return Lpos[j];
    };
    long long ll, hh;
    if (mstar < totL && mstar < totR && Lj(mstar) == s_r[1]) {  // the pointers met on an element equal to pv
      ll = min(Lj(mstar + 1), s_r[0]);
      hh = max(s_r[2], Lj(mstar - 1));
    } else {
      ll = min(Lj(mstar), s_r[0]);
      hh = max(s_r[1], Lj(mstar - 1));
    }
    out[0] = ll;
    out[1] = hh;
  }
  __syncthreads();
}

// np.argpartition(w[0..n), kth) into t[0..n) (t is overwritten), 0 <= kth < n.
// Only the first kth entries of the result are used by the caller; the last
// selection-sort pass of dumb_select_, which touches positions >= kth only,
// is left out.  Returns false if the nested selection stack would overflow.
__device__ bool block_argpartition(const double* w, int* t, long long n, long long kth, int* Lpos,
                                   unsigned char* fl) {
  __shared__ long long s_b[4];
  __shared__ int s_ok;
  for (long long i = threadIdx.x; i < n; i += kSelCTA) t[i] = (int)i;
  if (threadIdx.x == 0) s_ok = 1;
  __syncthreads();
  if (kth < 3) {  // dumb_select_
    for (long long i = 0; i < kth; ++i) {
      const long long m = sel_block_argext<false, false>(w, t, i, n);
      if (threadIdx.x == 0) sel_swap(t, i, m);
      __syncthreads();
    }
    return true;
  }
  if (kth == n - 1) {
    const long long m = sel_block_argext<true, true>(w, t, 0, n);
    if (threadIdx.x == 0) sel_swap(t, kth, m);
    __syncthreads();
    return true;
  }
  long long low = 0, high = n - 1;
  int depth = 2 * sel_msb(n);
  while (low + 1 < high) {
    long long ll0 = low + 1, hh0 = high;
    if (depth > 0 || hh0 - ll0 < 5) {
      if (threadIdx.x == 0) seq_median3_swap(w, t, low, low + (high - low) / 2, high);
    } else {
      if (threadIdx.x == 0) {
        const long long nmed = seq_median_groups(w, t, ll0, hh0 - ll0);
        if (nmed > 2 && !seq_introselect(w, t, ll0, nmed, nmed / 2)) s_ok = 0;
        sel_swap(t, ll0 + nmed / 2, low);
      }
      ll0 -= 1;
      hh0 += 1;
    }
    --depth;
    __syncthreads();
    if (!s_ok) return false;
    block_partition(w, t, low, high, ll0, hh0, Lpos, fl, s_b);
    const long long ll = s_b[0], hh = s_b[1];
    if (threadIdx.x == 0) sel_swap(t, low, hh);
    __syncthreads();
    if (hh >= kth) high = hh - 1;
    if (hh <= kth) low = ll;
  }
  if (threadIdx.x == 0 && high == low + 1 && w[t[high]] < w[t[low]]) sel_swap(t, high, low);
  __syncthreads();
  return true;
}

}  // namespace gbdmc
