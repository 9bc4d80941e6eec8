// hss_common.cuh -- shared device helpers for the sm_103a HSS merge kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define HSS_EPS 1.1102230246251565e-16   /* 2^-53, LAPACK DLAMCH('Epsilon') */
#define HSS_WARP 32
#define HSS_FULL 0xffffffffu

// ---- warp all-reduce (butterfly: every lane ends with the same bits) --------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(HSS_FULL, v, o);
  return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(HSS_FULL, v, o));
  return v;
}
__device__ __forceinline__ int warp_sum_int(int v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(HSS_FULL, v, o);
  return v;
}

// 1/x from the estimate y of the PTX instruction rcp.approx.ftz.f64 and one
// second-order correction: with e = 1 - x y (one fma, exact to ~2^-75),
// 1/x = y / (1 - e) = y (1 + e + e^2 + e^3 + ...), so y + y (e + e^2)
// leaves |e|^3 (far below an ulp for the estimate's accuracy) plus the final
// fma's rounding: within one ulp of 1/x for normal, finite, nonzero x (x = 0
// or infinite gives NaN).  Four FP64 instructions instead of a correctly
// rounded divide: the pole sums are FP64-pipe bound.
__device__ __forceinline__ double rcp_nr(double x) {
  double y;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
  const double e = fma(-x, y, 1.0);
  return fma(y, fma(e, e, e), y);
}

// a / b within 1.5 ulp through rcp_nr (four FP64 instructions instead of a
// correctly rounded divide) for the FP64-pipe bound loops; b = 0 gives NaN.
__device__ __forceinline__ double qdiv(double a, double b) { return a * rcp_nr(b); }

// (value, index) argmax with "first index wins" ties -- Fortran MAXLOC order.
struct ArgMax {
  double v;
  int i;
};
__device__ __forceinline__ ArgMax argmax_merge(ArgMax a, ArgMax b) {
  if (b.v > a.v || (b.v == a.v && b.i < a.i)) return b;
  return a;
}
__device__ __forceinline__ ArgMax warp_argmax(ArgMax a) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    ArgMax b;
    b.v = __shfl_xor_sync(HSS_FULL, a.v, o);
    b.i = __shfl_xor_sync(HSS_FULL, a.i, o);
    a = argmax_merge(a, b);
  }
  return a;
}

// Differences of the old poles F and new roots lam = F + DIFL, formed from
// DIFL/DIFR so that no cancellation occurs near the poles
// (SRC/CauchyHssEig.f90:470-568, computfd / computdd).
//   fd(p, q) = F_p - lam_q ;  dd(p, q) = lam_p - lam_q
// Singular-value mode (sq = true, the SVD merge of MDLASD3/MDLASD8): F holds
// the poles d, lam = sigma with DIFL/DIFR = sigma - d, and the differences are
// of squares, d_p^2 - sigma_q^2 = (d_p - sigma_q)(d_p + sigma_q), each factor
// formed without cancellation (as DLASD8 does).
struct PoleDiff {
  const double *__restrict__ F;
  const double *__restrict__ difl;
  const double *__restrict__ difr;
  bool sq = false;
  __device__ __forceinline__ double fd(int p, int q) const {
    const double lin = p <= q ? (__ldg(F + p) - __ldg(F + q)) - __ldg(difl + q)
                              : (__ldg(F + p) - __ldg(F + q + 1)) - __ldg(difr + q);
    return sq ? lin * (__ldg(F + p) + (__ldg(F + q) + __ldg(difl + q))) : lin;
  }
  // a - b for two pole values (a^2 - b^2 in singular-value mode)
  __device__ __forceinline__ double fv(double a, double b) const {
    return sq ? (a - b) * (a + b) : a - b;
  }
  __device__ __forceinline__ double dd(int p, int q) const {
    const double lin = p < q ? (__ldg(F + p + 1) - __ldg(F + q)) + __ldg(difr + p) - __ldg(difl + q)
                             : (__ldg(F + p) - __ldg(F + q + 1)) + __ldg(difl + p) - __ldg(difr + q);
    return sq ? lin * ((__ldg(F + p) + __ldg(difl + p)) + (__ldg(F + q) + __ldg(difl + q))) : lin;
  }
};

// Merge of root r in a level batch: merge m owns positions [s[m], s[m] + K[m])
// of the level arrays; off is the prefix sum of K (P + 1 entries).
__device__ __forceinline__ int find_merge(const int *__restrict__ off, int P, int r) {
  int lo = 0, hi = P;  // off[lo] <= r < off[hi]
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (__ldg(off + mid) <= r) lo = mid; else hi = mid;
  }
  return lo;
}

// Device status words written by kernels; the host maps them to INFO > 0.
enum HssStatus : int {
  HSS_OK = 0,
  HSS_SECULAR_NOCONV = 1,   // a secular root hit the iteration cap
  HSS_LEAF_NOCONV = 2,      // a leaf QL iteration hit its cap
  HSS_BAD_INPUT = 3,        // NaN / non-increasing poles
};
