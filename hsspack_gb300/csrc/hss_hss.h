// hss_hss.h -- the HSS path of one merge (MDLAED3 + DHSSEVC, SRC/mdlaed3.f90:124-261,
// SRC/CauchyHssEig.f90:2444-2598).
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

namespace hss {

struct HssError {
  std::string msg;
};

// One HSS merge of a DC level.  Poles/roots/weights are the merge's slices of
// the level arrays (already offset); ndslot lists the Q slots of the K
// non-deflated columns; Q is block-relative with leading dimension ldq and the
// merge's rows/columns start at s.
struct HssMergeArgs {
  int s, n, K;
  int leaf;
  double tol;
  int precision;
  const double *dl, *difl, *difr, *zhat;
  double *alpha;
  const int *ndslot;
  double *Q;
  long long ldq;
  int2 *sup = nullptr;  // rows each Q column holds data on (nullptr: all)
};

// Returns the number of kernels launched; *rank receives the largest HSS rank.
int hss_merge(const HssMergeArgs &a, int *rank, cudaStream_t st);

// One bidiagonal SVD merge with K >= bsmlz: U and V updated through two HSS
// products (the merge's rows s .. s+N-1 of U, s .. s+M-1 of V; leading dim ld).
struct SvdHssArgs {
  int s, N, M, K;
  int leaf;
  double tol;
  int precision;
  const double *dl, *difl, *difr, *zhat;  // the merge's slices (sigma mode)
  const int *ndslot;
  double *U, *V;
  long long ld;
};
int svd_hss_merge(const SvdHssArgs &a, int *rank, cudaStream_t st);

// CauchyHssMM on device arrays: B (n x ncb, ldb) <- C B, C_ij = u_i v_j / (D_i - F_j).
int hss_cauchyhssmm_core(int n, const double *D, const double *F, const double *u,
                         const double *v, int ni, double tol, int precision, double *B,
                         long long ldb, int ncb, int *rank, float *times, cudaStream_t st);

// DHSSEVC on caller arrays: Q(0:nrows, 0:K) <- Q * C.  sq: singular-value
// mode, C(i,j) = u_i v_j / (F_i^2 - sigma_j^2) with sigma_j = F_j + DIFL_j;
// swap_rho: the RRLU's strong-swap threshold (the eigen module's 1.5, the SVD
// module's 1.1).
int hss_dhssevc_core(int K, int ni, double tol, int precision, const double *F, const double *u,
                     const double *v, const double *difl, const double *difr, double *Q,
                     long long ldq, int nrows, int *rank, cudaStream_t st,
                     float *times = nullptr, bool sq = false, double swap_rho = 1.5);

// SvdHssUpdat (SRC/SvdHssUpdat.f90:1-178) on device arrays: the singular values
// and right singular vectors of [A; a^T] from A's.  f (n, ascending): A's
// singular values; z (n): V^T a; vt (n x n, ldvt): V^T (rows are the right
// singular vectors).  On return d[0..K) holds the K new singular values of the
// non-deflated problem (ascending) and d[K..n) the deflated ones, f and z are
// as MDLASD20 / MDLASD31 leave them, and vt's rows are the updated right
// singular vectors in the order of d.  Returns K (the secular equation's
// order); *rank: the largest HSS rank (K when the product ran densely).
int svd_update_core(int n, double *d, double *f, double *z, double *vt, long long ldvt, double tol,
                    int ni, int precision, int *rank, int *status, float *times,
                    cudaStream_t st);

// DHSSMM / DHSSMML on device arrays (mat2hss.cu): A (n x n, lda) compressed to
// HSS by truncated SVD (leaf ni, absolute tolerance tol); side 0: B (n x k,
// ldb) <- A_hss B; side 1: B (k x n, ldb) <- B A_hss.  times[0..1]:
// construction / multiplication (ms); *rank: largest HSS rank (n if a node
// outgrew the compression kernels and A was applied densely).
int hss_dhssmm_core(int n, const double *A, long long lda, double *B, long long ldb, int k,
                    double tol, int ni, int side, int precision, int *rank, float *times,
                    cudaStream_t st);

// Right singular vectors (singular value > tol, decreasing) of column-major
// tall matrices by TSQR, pivoted QR and one-sided Jacobi (mat2hss.cu).
std::vector<int> tall_right_bases(const std::vector<const double *> &X,
                                  const std::vector<int> &rows, const std::vector<int> &ncol,
                                  const std::vector<long long> &ld, const std::vector<double *> &P,
                                  const std::vector<double *> &PT, double tol, cudaStream_t st);

}  // namespace hss
