// leaf.cu -- batched eigensolver for the DC leaves (the DSTEQR('I') calls of
// SRC/mdlaed0.f90:262-266).
//
// One thread per leaf of size m <= 32, up to 32 leaves per CTA.  Each thread runs the
// implicit QL iteration with a Wilkinson shift (Golub & Van Loan, Matrix
// Computations, sec. 8.3) on its own leaf, rotating the columns of its
// eigenvector block, then sorts the eigenpairs ascending (selection sort, as
// DSTEQR ends).  GB300's FP64 pipe is narrow, so no FP64 instruction is
// replicated across lanes: every lane does distinct work.  Per-leaf storage
// lives in shared memory interleaved by lane ([row][col][lane]), so the 32
// lanes of a warp always touch 32 consecutive words (no bank conflicts).  The
// rank-one cuts of the divide step (mdlaed0.f90:213-219) are applied on load:
// d(first) -= |e(left cut)|, d(last) -= |e(right cut)|.
#include "hss_common.cuh"
#include "hss_kernels.h"

#include <algorithm>

namespace hss {

constexpr int LEAF_MAX = 32;

__global__ void __launch_bounds__(32)
k_leaf_ql(int nleaf, const int *__restrict__ lstart, const int *__restrict__ lsize, int mmax,
          int nblk, const double *__restrict__ d, const double *__restrict__ e,
          double *__restrict__ Q, long long ldq, double *__restrict__ Dp,
          int *__restrict__ perm, int *__restrict__ status, int2 *__restrict__ sup) {
  extern __shared__ double sm[];
  const int lane = threadIdx.x, LW = blockDim.x;
  const int leaf = blockIdx.x * LW + lane;
  const bool active = leaf < nleaf;
  double *D = sm;                    // D[i*LW + lane]
  double *E = sm + mmax * LW;        // E[i*LW + lane]
  double *Z = sm + 2 * mmax * LW;    // Z[(r*mmax + c)*LW + lane]
#define DD(i) D[(i) * LW + lane]
#define EE(i) E[(i) * LW + lane]
#define ZZ(r, c) Z[((r) * mmax + (c)) * LW + lane]
  int s = 0, m = 0;
  if (active) {
    s = lstart[leaf];
    m = lsize[leaf];
    for (int i = 0; i < m; ++i) {
      double dv = d[s + i];
      if (i == 0 && s > 0) dv -= fabs(e[s - 1]);
      if (i == m - 1 && s + m < nblk) dv -= fabs(e[s + m - 1]);
      DD(i) = dv;
      EE(i) = (i < m - 1) ? e[s + i] : 0.0;
      for (int c = 0; c < m; ++c) ZZ(i, c) = (i == c) ? 1.0 : 0.0;
    }
  }
  int bad = 0;
  for (int l = 0; l < m && !bad; ++l) {
    int iter = 0;
    while (true) {
      int mm = l;
      for (; mm < m - 1; ++mm)
        if (fabs(EE(mm)) <= HSS_EPS * (fabs(DD(mm)) + fabs(DD(mm + 1)))) break;
      if (mm == l) break;
      if (++iter > 30 * m) { bad = 1; break; }
      // operands are O(||T||) after the block scaling, so plain sqrt is safe
      double g = (DD(l + 1) - DD(l)) / (2.0 * EE(l));
      double r = sqrt(fma(g, g, 1.0));
      g = DD(mm) - DD(l) + EE(l) / (g + copysign(r, g));
      double sn = 1.0, cs = 1.0, p = 0.0;
      bool early = false;
      for (int i = mm - 1; i >= l; --i) {
        const double f = sn * EE(i), b = cs * EE(i);
        r = sqrt(fma(f, f, g * g));
        EE(i + 1) = r;
        if (r == 0.0) {
          DD(i + 1) -= p;
          EE(mm) = 0.0;
          early = true;
          break;
        }
        const double rinv = 1.0 / r;
        sn = f * rinv;
        cs = g * rinv;
        g = DD(i + 1) - p;
        r = (DD(i) - g) * sn + 2.0 * cs * b;
        p = sn * r;
        DD(i + 1) = g + p;
        g = cs * r - b;
        for (int k = 0; k < m; ++k) {  // rotate columns i, i+1
          const double zi = ZZ(k, i), zi1 = ZZ(k, i + 1);
          ZZ(k, i + 1) = sn * zi + cs * zi1;
          ZZ(k, i) = cs * zi - sn * zi1;
        }
      }
      if (early) continue;
      DD(l) -= p;
      EE(l) = g;
      EE(mm) = 0.0;
    }
  }
  // selection sort ascending, moving columns
  for (int i = 0; i < m - 1; ++i) {
    int k = i;
    double pmin = DD(i);
    for (int j = i + 1; j < m; ++j)
      if (DD(j) < pmin) { k = j; pmin = DD(j); }
    if (k != i) {
      DD(k) = DD(i);
      DD(i) = pmin;
      for (int r = 0; r < m; ++r) {
        const double t = ZZ(r, i);
        ZZ(r, i) = ZZ(r, k);
        ZZ(r, k) = t;
      }
    }
  }
  if (active) {
    for (int i = 0; i < m; ++i) {
      Dp[s + i] = DD(i);
      perm[s + i] = s + i;
      if (sup) sup[s + i] = make_int2(s, s + m);  // rows the column is written on
    }
    if (bad) atomicMax(status, HSS_LEAF_NOCONV);
  }
  __syncthreads();
  // write the blocks: lanes over rows, one leaf at a time (coalesced columns)
  for (int q = 0; q < LW; ++q) {
    const int lf = blockIdx.x * LW + q;
    if (lf >= nleaf) break;
    const int s2 = lstart[lf], m2 = lsize[lf];
    for (int c = 0; c < m2; ++c)
      for (int r = lane; r < m2; r += LW) Q[(long long)(s2 + c) * ldq + s2 + r] = Z[(r * mmax + c) * LW + q];
  }
#undef DD
#undef EE
#undef ZZ
}

void launch_leaf(int nleaf, const int *lstart, const int *lsize, int mmax, int nblk,
                 const double *d, const double *e, double *Q, long long ldq, double *Dp, int *perm,
                 int *status, cudaStream_t st, int2 *sup) {
  if (nleaf <= 0) return;
  mmax = std::max(1, std::min(mmax, LEAF_MAX));
  // leaves per CTA: enough CTAs to cover the SMs, and the block within smem
  int lw = 32;
  while (lw > 8 && (nleaf + lw - 1) / lw < 2 * 148) lw /= 2;
  while (lw > 1 && (size_t)(mmax * mmax + 2 * mmax) * lw * sizeof(double) > 200 * 1024) lw /= 2;
  const size_t smem = (size_t)(mmax * mmax + 2 * mmax) * lw * sizeof(double);
  static size_t attr = 0;
  if (smem > 48 * 1024 && smem > attr) {
    cudaFuncSetAttribute(k_leaf_ql, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    attr = smem;
  }
  k_leaf_ql<<<(nleaf + lw - 1) / lw, lw, smem, st>>>(nleaf, lstart, lsize, mmax, nblk, d, e, Q, ldq,
                                                      Dp, perm, status, sup);
}

}  // namespace hss
