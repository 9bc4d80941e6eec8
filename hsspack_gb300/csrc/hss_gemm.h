// hss_gemm.h -- problem descriptor and launch wrappers shared by the host driver.
#pragma once
#include <cuda_runtime.h>

#include <vector>

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

// one operand of the split-BF16 GEMM: `rows` vectors of length `inner`
// (A: rows of an M x K column-major matrix; B: columns of a K x N matrix)
struct SplitProb {
  const double *src;
  int ld, rows, inner, ktiles;
  void *dst;   // digit planes, pre-tiled
  int *expo;   // per row / column exponent
  unsigned long long *mbits;  // per row / column largest |x| as bits (zeroed)
  int w0;      // first flattened work item (panel x k chunk) of this operand
};

int gemm_tiles(int M, int N);
void launch_gemm_f64(int nprob, int total_tiles, const GemmDesc *d_probs, cudaStream_t st);
// FP64-accurate products on the BF16 tensor cores (digit-plane splitting);
// d_err receives 1/2 if a bounded wait timed out.
void launch_gemm_split(const std::vector<GemmDesc> &probs, int *d_err, cudaStream_t st);
// the same products with the operands split inside each CTA (many small and
// medium products): no plane buffers in global memory
void launch_gemm_fused(const std::vector<GemmDesc> &probs, int *d_err, cudaStream_t st);
// largest N and K of the element kernel for small products (0: 128)
void set_small_nk(int v);
// products with M*N*K >= 2^v and M >= set_split_min_m take the split path (0: 15)
void set_split_min_log2(int v);
// smallest M of a split product (0: 128)
void set_split_min_m(int v);
// 0: staged digit planes (default); 1: split inside the product kernel
void set_gemm_path(int v);
// precision 0: FP64 CUDA cores, 1: split BF16 tensor cores
void launch_gemm(const std::vector<GemmDesc> &probs, int precision, cudaStream_t st);

}  // namespace hss
