// band.cu -- symmetric banded divide and conquer (MDSBEVD, SRC/mdsbevd.f90:183).
//
// The band matrix (upper storage, LAPACK layout: A(i,j) = AB(kd+i-j, j) for
// j-kd <= i <= j, 0-based) is cut between consecutive leaves.  At the cut
// after row c the coupling block B(r, q) = A(c-kd+1+r, c+1+q) (kd x kd, lower
// triangular) is split by its SVD B = U S V^T (mdsbevd.f90:291-297):
//   A = diag(A_1 - [0 0; 0 U S U^T], A_2 - [V S V^T 0; 0 0])
//       + sum_k s_k w_k w_k^T,  w_k = [u_k in the last kd rows of block 1;
//                                       v_k in the first kd rows of block 2]
// (DSymSplit, SRC/BasicMM.f90:1195-1311).  Every leaf is then a small dense
// symmetric eigenproblem (DSYEVD at mdsbevd.f90:304-313) and every merge is
// kd rank-one updates (MDSBED1, SRC/mdsbed1.f90:2) driven by Z = Q^T [w_1 ..
// w_kd] (mdsbed1.f90:174-186), whose later columns are carried through each
// update's Givens rotations and eigenvector matrix.
//
// Kernels here: the per-cut SVDs (one-sided Jacobi, Hestenes 1958), the leaf
// eigensolves (cyclic Jacobi, Rutishauser's rotation formulas), the Z matrix
// of a level, and the transformation of Z's remaining columns by an update.
#include "hss_common.cuh"
#include "hss_kernels.h"

namespace hss {

constexpr int BAND_LEAF_MAX = 64;
constexpr int BAND_KD_MAX = 32;
constexpr int JACOBI_SWEEPS = 60;

__device__ __forceinline__ double band_at(const double *AB, long long ldab, int kd, int i, int j) {
  // A(i, j) of the symmetric band matrix from upper storage (0 outside the band)
  if (i > j) { const int t = i; i = j; j = t; }
  if (j - i > kd) return 0.0;
  return AB[(long long)j * ldab + (kd + i - j)];
}

// One warp per cut: B = U S V^T by one-sided Jacobi on the columns of B; S
// sorted descending.  cut_row[c] = last row of the block above cut c.
// Outputs per cut (column-major kd x kd): U, V; S (kd).
__global__ void __launch_bounds__(32)
k_band_cut_svd(int ncut, const int *__restrict__ cut_row, int kd, const double *__restrict__ AB,
               long long ldab, double *__restrict__ Uc, double *__restrict__ Vc,
               double *__restrict__ Sc, int *__restrict__ status) {
  __shared__ double B[BAND_KD_MAX][BAND_KD_MAX + 1];
  __shared__ double V[BAND_KD_MAX][BAND_KD_MAX + 1];
  __shared__ double sig[BAND_KD_MAX];
  __shared__ int ord[BAND_KD_MAX];
  const int lane = threadIdx.x;
  for (int cut = blockIdx.x; cut < ncut; cut += gridDim.x) {
    const int c = cut_row[cut];
    for (int q = 0; q < kd; ++q) {
      if (lane < kd) {
        B[lane][q] = band_at(AB, ldab, kd, c - kd + 1 + lane, c + 1 + q);
        V[lane][q] = (lane == q) ? 1.0 : 0.0;
      }
    }
    __syncwarp();
    bool conv = false;
    for (int sweep = 0; sweep < JACOBI_SWEEPS && !conv; ++sweep) {
      conv = true;
      for (int p = 0; p < kd - 1; ++p)
        for (int q = p + 1; q < kd; ++q) {
          const double bp = lane < kd ? B[lane][p] : 0.0, bq = lane < kd ? B[lane][q] : 0.0;
          const double al = warp_sum(bp * bp), be = warp_sum(bq * bq), ga = warp_sum(bp * bq);
          // converged pair: |cos angle| below 4 kd ulps (a rotation leaves a few
          // ulps behind, so a tighter test would cycle)
          if (ga == 0.0 || fabs(ga) <= 4.0 * kd * HSS_EPS * sqrt(al * be)) continue;
          conv = false;
          const double ze = (be - al) / (2.0 * ga);
          const double t = copysign(1.0, ze) / (fabs(ze) + sqrt(1.0 + ze * ze));
          const double cs = 1.0 / sqrt(1.0 + t * t), sn = cs * t;
          if (lane < kd) {
            B[lane][p] = cs * bp - sn * bq;
            B[lane][q] = sn * bp + cs * bq;
            const double vp = V[lane][p], vq = V[lane][q];
            V[lane][p] = cs * vp - sn * vq;
            V[lane][q] = sn * vp + cs * vq;
          }
          __syncwarp();
        }
    }
    if (!conv && lane == 0) atomicMax(status, HSS_LEAF_NOCONV);
    for (int q = 0; q < kd; ++q) {
      const double b = lane < kd ? B[lane][q] : 0.0;
      const double s2 = warp_sum(b * b);
      if (lane == 0) sig[q] = sqrt(s2);
    }
    __syncwarp();
    if (lane == 0) {  // order by singular value, descending (stable)
      for (int q = 0; q < kd; ++q) ord[q] = q;
      for (int a = 0; a < kd; ++a) {
        int best = a;
        for (int b = a + 1; b < kd; ++b)
          if (sig[ord[b]] > sig[ord[best]]) best = b;
        const int t = ord[a]; ord[a] = ord[best]; ord[best] = t;
      }
    }
    __syncwarp();
    if (lane < kd) {
      for (int k = 0; k < kd; ++k) {
        const int q = ord[k];
        const double s = sig[q];
        const long long o = (long long)cut * kd * kd + (long long)k * kd + lane;
        Uc[o] = s > 0.0 ? B[lane][q] / s : 0.0;
        Vc[o] = V[lane][q];
      }
    }
    if (lane == 0)
      for (int k = 0; k < kd; ++k) Sc[(long long)cut * kd + k] = sig[ord[k]];
    __syncwarp();
  }
}

// One warp per leaf: assemble the dense m x m block (band part minus the
// corrections of the cuts above and below it), cyclic Jacobi to diagonal,
// eigenpairs sorted ascending into the leaf's slots (Q columns, Dp, perm).
// cut_above[l] / cut_below[l]: index of the cut at the leaf's top / bottom
// edge, or -1.  Shared memory: two m x (m + 1) arrays.
__global__ void __launch_bounds__(32)
k_band_leaf(int nleaf, const int *__restrict__ lstart, const int *__restrict__ lsize,
            const int *__restrict__ cut_above, const int *__restrict__ cut_below, int mmax, int kd,
            const double *__restrict__ AB, long long ldab, const double *__restrict__ Uc,
            const double *__restrict__ Vc, const double *__restrict__ Sc, double *__restrict__ Q,
            long long ldq, double *__restrict__ Dp, int *__restrict__ perm,
            int *__restrict__ status) {
  extern __shared__ double bsm[];
  const int ld = mmax + 1;
  double *A = bsm, *Vv = bsm + mmax * ld;
  __shared__ int ord[BAND_LEAF_MAX];
  const int lane = threadIdx.x;
  for (int leaf = blockIdx.x; leaf < nleaf; leaf += gridDim.x) {
    const int s = lstart[leaf], m = lsize[leaf];
    const int ca = cut_above[leaf], cb = cut_below[leaf];
    for (int r = lane; r < m; r += 32)
      for (int c = 0; c < m; ++c) {
        double a = band_at(AB, ldab, kd, s + r, s + c);
        if (ca >= 0 && r < kd && c < kd) {  // - V S V^T on the first kd rows
          const double *Vk = Vc + (long long)ca * kd * kd;
          const double *Sk = Sc + (long long)ca * kd;
          double t = 0.0;
          for (int k = 0; k < kd; ++k) t = fma(Vk[k * kd + r] * Sk[k], Vk[k * kd + c], t);
          a -= t;
        }
        if (cb >= 0 && r >= m - kd && c >= m - kd) {  // - U S U^T on the last kd rows
          const double *Uk = Uc + (long long)cb * kd * kd;
          const double *Sk = Sc + (long long)cb * kd;
          const int rr = r - (m - kd), cc = c - (m - kd);
          double t = 0.0;
          for (int k = 0; k < kd; ++k) t = fma(Uk[k * kd + rr] * Sk[k], Uk[k * kd + cc], t);
          a -= t;
        }
        A[r * ld + c] = a;
        Vv[r * ld + c] = (r == c) ? 1.0 : 0.0;
      }
    __syncwarp();
    double fro = 0.0;
    for (int r = lane; r < m; r += 32)
      for (int c = 0; c < m; ++c) fro += A[r * ld + c] * A[r * ld + c];
    fro = sqrt(warp_sum(fro));
    // skip a rotation when |a_pq| is below 1e-17 ||A||_F (moves eigenvalues by
    // < m 1e-17 ||A||) or below m ulps of sqrt(|a_pp a_qq|) (relative accuracy)
    const double small = 1e-17 * fro, rel = (double)m * HSS_EPS;
    bool conv = false;
    for (int sweep = 0; sweep < JACOBI_SWEEPS && !conv; ++sweep) {
      conv = true;
      for (int p = 0; p < m - 1; ++p)
        for (int q = p + 1; q < m; ++q) {
          const double apq = A[p * ld + q], app = A[p * ld + p], aqq = A[q * ld + q];
          if (fabs(apq) <= small || fabs(apq) <= rel * sqrt(fabs(app * aqq))) continue;
          conv = false;
          const double th = (aqq - app) / (2.0 * apq);
          const double t = copysign(1.0, th) / (fabs(th) + sqrt(1.0 + th * th));
          const double cs = 1.0 / sqrt(1.0 + t * t), sn = cs * t;
          __syncwarp();
          for (int r = lane; r < m; r += 32) {  // A <- A J, V <- V J (columns p, q)
            const double xp = A[r * ld + p], xq = A[r * ld + q];
            A[r * ld + p] = cs * xp - sn * xq;
            A[r * ld + q] = sn * xp + cs * xq;
            const double vp = Vv[r * ld + p], vq = Vv[r * ld + q];
            Vv[r * ld + p] = cs * vp - sn * vq;
            Vv[r * ld + q] = sn * vp + cs * vq;
          }
          __syncwarp();
          for (int r = lane; r < m; r += 32) {  // A <- J^T A (rows p, q)
            const double xp = A[p * ld + r], xq = A[q * ld + r];
            A[p * ld + r] = cs * xp - sn * xq;
            A[q * ld + r] = sn * xp + cs * xq;
          }
          __syncwarp();
          if (lane == 0) {
            A[p * ld + p] = app - t * apq;
            A[q * ld + q] = aqq + t * apq;
            A[p * ld + q] = 0.0;
            A[q * ld + p] = 0.0;
          }
          __syncwarp();
        }
    }
    if (!conv && lane == 0) atomicMax(status, HSS_LEAF_NOCONV);
    if (lane == 0) {  // ascending order of the eigenvalues (stable)
      for (int i = 0; i < m; ++i) ord[i] = i;
      for (int a = 0; a < m; ++a) {
        int best = a;
        for (int b = a + 1; b < m; ++b)
          if (A[ord[b] * ld + ord[b]] < A[ord[best] * ld + ord[best]]) best = b;
        const int t = ord[a]; ord[a] = ord[best]; ord[best] = t;
      }
    }
    __syncwarp();
    for (int c = 0; c < m; ++c) {
      const int src = ord[c];
      for (int r = lane; r < m; r += 32) Q[(long long)(s + c) * ldq + s + r] = Vv[r * ld + src];
    }
    for (int c = lane; c < m; c += 32) {
      Dp[s + c] = A[ord[c] * ld + ord[c]];
      perm[s + c] = s + c;
    }
    __syncwarp();
  }
}

// Z[k * zld + slot] = w_k^T Q[:, slot] for every slot of every merge of a
// level (mdsbed1.f90:174-186): top slots see U (rows s+n1-kd .. s+n1-1),
// bottom slots V (rows s+n1 .. s+n1+kd-1) of the merge's cut.
__global__ void k_band_z(int P, const int *__restrict__ ms, const int *__restrict__ mn,
                         const int *__restrict__ mn1, const int *__restrict__ mcut, int kd,
                         const double *__restrict__ Q, long long ldq, const double *__restrict__ Uc,
                         const double *__restrict__ Vc, double *__restrict__ Z, long long zld) {
  for (int m = blockIdx.y; m < P; m += gridDim.y) {
    const int s = ms[m], n = mn[m], n1 = mn1[m], cut = mcut[m];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
      const int slot = s + i;
      const bool top = i < n1;
      const int base = top ? s + n1 - kd : s + n1;
      const double *W = (top ? Uc : Vc) + (long long)cut * kd * kd;
      const double *col = Q + (long long)slot * ldq + base;
      for (int k = 0; k < kd; ++k) {
        double acc = 0.0;
        for (int r = 0; r < kd; ++r) acc = fma(col[r], W[k * kd + r], acc);
        Z[k * zld + slot] = acc;
      }
    }
  }
}

// The update's eigenvector matrix applied to the remaining Z columns: for
// root j of merge m, Zt[c][slot_j] = sum_i S_ij Z[c][slot_i], S_ij =
// zhat_i alpha_j / (d_i - lam_j) (warp per root, as the alpha kernel).
__global__ void k_band_zupdate(LevelView lv, const double *__restrict__ dl,
                               const double *__restrict__ difl, const double *__restrict__ difr,
                               const double *__restrict__ zhat, const double *__restrict__ alpha,
                               const int *__restrict__ ndslot, const double *__restrict__ Z,
                               int nrest, long long zld, double *__restrict__ Zt) {
  const int lane = threadIdx.x & 31;
  const int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (r >= __ldg(lv.rootoff + lv.P)) return;
  const int m = find_merge(lv.rootoff, lv.P, r);
  const int j = r - __ldg(lv.rootoff + m);
  const int s = __ldg(lv.s + m);
  const int K = __ldg(lv.K + m);
  PoleDiff P{dl + s, difl + s, difr + s};
  const double aj = alpha[s + j];
  for (int c = 0; c < nrest; ++c) {
    double acc = 0.0;
    for (int i = lane; i < K; i += HSS_WARP)
      acc = fma(__ldg(zhat + s + i) / P.fd(i, j), Z[c * zld + ndslot[s + i]], acc);
    acc = warp_sum(acc);
    if (lane == 0) Zt[c * zld + ndslot[s + j]] = acc * aj;
  }
}

__global__ void k_band_zcopy(LevelView lv, const int *__restrict__ ndslot, int nrest, long long zld,
                             const double *__restrict__ Zt, double *__restrict__ Z) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= __ldg(lv.rootoff + lv.P)) return;
  const int m = find_merge(lv.rootoff, lv.P, r);
  const int j = r - __ldg(lv.rootoff + m);
  const int slot = ndslot[__ldg(lv.s + m) + j];
  for (int c = 0; c < nrest; ++c) Z[c * zld + slot] = Zt[c * zld + slot];
}

// ---------------------------------------------------------------- launch --
static inline int band_warp_grid(int total, int threads) {
  return (int)(((long long)total * 32 + threads - 1) / threads);
}

void launch_band_cut_svd(int ncut, const int *cut_row, int kd, const double *AB, long long ldab,
                         double *Uc, double *Vc, double *Sc, int *status, cudaStream_t st) {
  if (ncut <= 0 || kd <= 0) return;
  k_band_cut_svd<<<std::min(ncut, 65535), 32, 0, st>>>(ncut, cut_row, kd, AB, ldab, Uc, Vc, Sc,
                                                        status);
}

void launch_band_leaf(int nleaf, const int *lstart, const int *lsize, const int *cut_above,
                      const int *cut_below, int mmax, int kd, const double *AB, long long ldab,
                      const double *Uc, const double *Vc, const double *Sc, double *Q,
                      long long ldq, double *Dp, int *perm, int *status, cudaStream_t st) {
  if (nleaf <= 0) return;
  const size_t smem = sizeof(double) * 2 * (size_t)mmax * (mmax + 1);
  static size_t attr = 0;
  if (smem > 48 * 1024 && smem > attr) {
    cudaFuncSetAttribute(k_band_leaf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    attr = smem;
  }
  k_band_leaf<<<std::min(nleaf, 65535), 32, smem, st>>>(nleaf, lstart, lsize, cut_above,
                                                         cut_below, mmax, kd, AB, ldab, Uc, Vc,
                                                         Sc, Q, ldq, Dp, perm, status);
}

void launch_band_z(int P, int maxn, const int *ms, const int *mn, const int *mn1, const int *mcut,
                   int kd, const double *Q, long long ldq, const double *Uc, const double *Vc,
                   double *Z, long long zld, cudaStream_t st) {
  if (P <= 0 || kd <= 0) return;
  dim3 grid((maxn + 255) / 256, std::min(P, 65535));
  k_band_z<<<grid, 256, 0, st>>>(P, ms, mn, mn1, mcut, kd, Q, ldq, Uc, Vc, Z, zld);
}

void launch_band_zupdate(const LevelView &lv, int total, const double *dl, const double *difl,
                         const double *difr, const double *zhat, const double *alpha,
                         const int *ndslot, double *Z, int nrest, long long zld, double *Zt,
                         cudaStream_t st) {
  if (total <= 0 || nrest <= 0) return;
  k_band_zupdate<<<band_warp_grid(total, 256), 256, 0, st>>>(lv, dl, difl, difr, zhat, alpha, ndslot,
                                                        Z, nrest, zld, Zt);
  k_band_zcopy<<<(total + 255) / 256, 256, 0, st>>>(lv, ndslot, nrest, zld, Zt, Z);
}

}  // namespace hss
