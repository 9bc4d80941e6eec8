// leaf.cu -- batched eigensolver for the DC leaves (the DSTEQR('I') calls of
// SRC/mdlaed0.f90:262-266).
//
// One warp per leaf of size m <= 32.  The implicit QL iteration with a
// Wilkinson shift (Golub & Van Loan, Matrix Computations, sec. 8.3) runs its
// scalar recurrence identically on every lane from shared memory; lane k owns
// row k of the eigenvector block and applies each Givens rotation to it.
// Eigenpairs are finally sorted ascending (selection sort, as DSTEQR ends).
// The rank-one cuts of the divide step (mdlaed0.f90:213-219) are applied on
// load: d(first) -= |e(left cut)|, d(last) -= |e(right cut)|.
#include "hss_common.cuh"
#include "hss_kernels.h"

namespace hss {

constexpr int LEAF_MAX = 32;
constexpr int LEAF_WARPS = 4;

__global__ void __launch_bounds__(LEAF_WARPS * 32)
k_leaf_ql(int nleaf, const int *__restrict__ lstart, const int *__restrict__ lsize,
          int nblk, const double *__restrict__ d, const double *__restrict__ e,
          double *__restrict__ Q, long long ldq, double *__restrict__ Dp,
          int *__restrict__ perm, int *__restrict__ status) {
  __shared__ double sd[LEAF_WARPS][LEAF_MAX + 1];
  __shared__ double se[LEAF_WARPS][LEAF_MAX + 1];
  __shared__ double sz[LEAF_WARPS][LEAF_MAX][LEAF_MAX + 1];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int leaf = blockIdx.x * LEAF_WARPS + w;
  if (leaf >= nleaf) return;
  const int s = __ldg(lstart + leaf), m = __ldg(lsize + leaf);
  double *D = sd[w], *E = se[w];
  double(*Z)[LEAF_MAX + 1] = sz[w];
  if (lane < m) {
    double dv = __ldg(d + s + lane);
    if (lane == 0 && s > 0) dv -= fabs(__ldg(e + s - 1));
    if (lane == m - 1 && s + m < nblk) dv -= fabs(__ldg(e + s + m - 1));
    D[lane] = dv;
    E[lane] = (lane < m - 1) ? __ldg(e + s + lane) : 0.0;
    for (int c = 0; c < m; ++c) Z[lane][c] = (c == lane) ? 1.0 : 0.0;
  }
  __syncwarp();
  int bad = 0;
  for (int l = 0; l < m; ++l) {
    int iter = 0;
    while (true) {
      int mm = l;
      for (; mm < m - 1; ++mm) {
        const double dd = fabs(D[mm]) + fabs(D[mm + 1]);
        if (fabs(E[mm]) <= HSS_EPS * dd) break;
      }
      if (mm == l) break;
      if (++iter > 30 * m) { bad = 1; break; }
      // Wilkinson-type shift from the leading 2x2 block
      double g = (D[l + 1] - D[l]) / (2.0 * E[l]);
      double r = hypot(g, 1.0);
      g = D[mm] - D[l] + E[l] / (g + copysign(r, g));
      double sn = 1.0, cs = 1.0, p = 0.0;
      int i = mm - 1;
      bool early = false;
      for (; i >= l; --i) {
        const double f = sn * E[i], b = cs * E[i];
        r = hypot(f, g);
        if (lane == 0) E[i + 1] = r;
        if (r == 0.0) {
          __syncwarp();
          if (lane == 0) { D[i + 1] -= p; E[mm] = 0.0; }
          early = true;
          break;
        }
        sn = f / r;
        cs = g / r;
        g = D[i + 1] - p;
        r = (D[i] - g) * sn + 2.0 * cs * b;
        p = sn * r;
        __syncwarp();
        if (lane == 0) D[i + 1] = g + p;
        g = cs * r - b;
        if (lane < m) {  // rotate columns i, i+1 of row `lane`
          const double zi = Z[lane][i], zi1 = Z[lane][i + 1];
          Z[lane][i + 1] = sn * zi + cs * zi1;
          Z[lane][i] = cs * zi - sn * zi1;
        }
        __syncwarp();
      }
      __syncwarp();
      if (early) continue;
      if (lane == 0) { D[l] -= p; E[l] = g; E[mm] = 0.0; }
      __syncwarp();
    }
    if (bad) break;
  }
  __syncwarp();
  // selection sort ascending, moving columns
  for (int i = 0; i < m - 1; ++i) {
    int k = i;
    double pmin = D[i];
    for (int j = i + 1; j < m; ++j)
      if (D[j] < pmin) { k = j; pmin = D[j]; }
    __syncwarp();
    if (k != i) {
      if (lane == 0) { D[k] = D[i]; D[i] = pmin; }
      if (lane < m) {
        const double t = Z[lane][i];
        Z[lane][i] = Z[lane][k];
        Z[lane][k] = t;
      }
    }
    __syncwarp();
  }
  // write the m x m block at Q(s, s), eigenvalues and identity order
  for (int c = 0; c < m; ++c)
    if (lane < m) Q[(long long)(s + c) * ldq + s + lane] = Z[lane][c];
  if (lane < m) {
    Dp[s + lane] = D[lane];
    perm[s + lane] = s + lane;
  }
  if (bad && lane == 0) atomicMax(status, HSS_LEAF_NOCONV);
}

void launch_leaf(int nleaf, const int *lstart, const int *lsize, int nblk, const double *d,
                 const double *e, double *Q, long long ldq, double *Dp, int *perm, int *status,
                 cudaStream_t st) {
  if (nleaf <= 0) return;
  dim3 grid((nleaf + LEAF_WARPS - 1) / LEAF_WARPS);
  k_leaf_ql<<<grid, LEAF_WARPS * 32, 0, st>>>(nleaf, lstart, lsize, nblk, d, e, Q, ldq, Dp, perm,
                                              status);
}

}  // namespace hss
