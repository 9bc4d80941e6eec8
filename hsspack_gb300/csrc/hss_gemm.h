// hss_gemm.h -- problem descriptor and launch wrappers shared by the host driver.
#pragma once
#include <cuda_runtime.h>

namespace hss {

// C (M x N, ldc) = A (M x K, lda) * B (K x N, ldb) [+ C if beta]; column-major.
struct GemmDesc {
  const double *A;
  const double *B;
  double *C;
  int lda, ldb, ldc;
  int M, N, K;
  int beta;
  int tile0;  // first flattened tile index of this problem
};

int gemm_tiles(int M, int N);
void launch_gemm_f64(int nprob, int total_tiles, const GemmDesc *d_probs, cudaStream_t st);

}  // namespace hss
