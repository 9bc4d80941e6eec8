// hss_block.cuh -- block-wide helpers shared by the merge kernels (one CTA
// per merge): exclusive scan, maximum, stable merge sort of (value, slot) pairs.
#pragma once
#include "hss_common.cuh"

namespace hss {

// Block-wide exclusive scan of one 64-bit value per thread (MT threads).
template <int MT>
__device__ __forceinline__ unsigned long long block_scan64(unsigned long long v,
                                                           unsigned long long *tot) {
  __shared__ unsigned long long ws[MT / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  unsigned long long x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    unsigned long long y = __shfl_up_sync(HSS_FULL, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) ws[w] = x;
  __syncthreads();
  if (w == 0) {
    unsigned long long t = (lane < MT / 32) ? ws[lane] : 0ull;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      unsigned long long y = __shfl_up_sync(HSS_FULL, t, o);
      if (lane >= o) t += y;
    }
    if (lane < MT / 32) ws[lane] = t;
  }
  __syncthreads();
  const unsigned long long base = (w > 0) ? ws[w - 1] : 0ull;
  if (tot) *tot = ws[MT / 32 - 1];
  const unsigned long long r = base + x - v;
  __syncthreads();
  return r;
}

template <int MT>
__device__ __forceinline__ double block_max(double v) {
  __shared__ double ws[MT / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  v = warp_max(v);
  if (lane == 0) ws[w] = v;
  __syncthreads();
  double r = ws[0];
  for (int i = 1; i < MT / 32; ++i) r = fmax(r, ws[i]);
  __syncthreads();
  return r;
}

// Stable bottom-up merge sort of (v, p) pairs of length len by one CTA, with
// scratch (tv, tp) of the same length; each pass places every element by a
// binary search in the partner run (merge path).
__device__ __forceinline__ void block_sort_pairs(double *v, int *p, double *tv, int *tp, int len) {
  bool in_tmp = false;
  for (int width = 1; width < len; width <<= 1) {
    const double *sv = in_tmp ? tv : v;
    const int *sp = in_tmp ? tp : p;
    double *dv = in_tmp ? v : tv;
    int *dp = in_tmp ? p : tp;
    for (int i = threadIdx.x; i < len; i += blockDim.x) {
      const int run = i / width, start = (run & ~1) * width;
      const int mid = min(start + width, len), end = min(start + 2 * width, len);
      const double x = sv[i];
      int pos;
      if ((run & 1) == 0) {
        int lo = mid, hi = end;
        while (lo < hi) { int md = (lo + hi) >> 1; if (sv[md] < x) lo = md + 1; else hi = md; }
        pos = (i - start) + (lo - mid);
      } else {
        int lo = start, hi = mid;
        while (lo < hi) { int md = (lo + hi) >> 1; if (sv[md] <= x) lo = md + 1; else hi = md; }
        pos = (i - mid) + (lo - start);
      }
      dv[start + pos] = x;
      dp[start + pos] = sp[i];
    }
    __syncthreads();
    in_tmp = !in_tmp;
  }
  if (in_tmp) {
    for (int i = threadIdx.x; i < len; i += blockDim.x) { v[i] = tv[i]; p[i] = tp[i]; }
    __syncthreads();
  }
}

}  // namespace hss
