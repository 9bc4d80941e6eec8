// hss_hss.h -- the HSS path of one merge (MDLAED3 + DHSSEVC, SRC/mdlaed3.f90:124-261,
// SRC/CauchyHssEig.f90:2444-2598).
#pragma once
#include <cuda_runtime.h>

#include <string>

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

// DHSSEVC on caller arrays: Q(0:nrows, 0:K) <- Q * C.
int hss_dhssevc_core(int K, int ni, double tol, int precision, const double *F, const double *u,
                     const double *v, const double *difl, const double *difr, double *Q,
                     long long ldq, int nrows, int *rank, cudaStream_t st,
                     float *times = nullptr);

// DHSSMM / DHSSMML on device arrays (mat2hss.cu): A (n x n, lda) compressed to
// HSS by truncated SVD (leaf ni, absolute tolerance tol); side 0: B (n x k,
// ldb) <- A_hss B; side 1: B (k x n, ldb) <- B A_hss.  times[0..1]:
// construction / multiplication (ms); *rank: largest HSS rank (n if a node
// outgrew the compression kernels and A was applied densely).
int hss_dhssmm_core(int n, const double *A, long long lda, double *B, long long ldb, int k,
                    double tol, int ni, int side, int precision, int *rank, float *times,
                    cudaStream_t st);

}  // namespace hss
