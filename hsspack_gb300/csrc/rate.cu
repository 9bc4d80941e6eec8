// rate.cu -- the FP64 fused multiply-add rate of the GPU, measured by a kernel.
//
// The FP64-bound stages (secular pole sums, Loewner products, the FP64 GEMM)
// are reported against this measured rate rather than a nominal figure.  Each
// thread runs eight independent FMA chains (enough to cover the FP64 pipe's
// latency), every SM holds several CTAs, and the host times one launch with
// CUDA events on the caller's stream; 2 flops per FMA.
#include <cuda_runtime.h>

#include "../../include/hsspack_gb300.h"

namespace hss {

__global__ void __launch_bounds__(256) k_fp64_fma_rate(int iters, double x, double y, double *out) {
  double a0 = 1e-3 * threadIdx.x, a1 = a0 + 0.1, a2 = a0 + 0.2, a3 = a0 + 0.3;
  double a4 = a0 + 0.4, a5 = a0 + 0.5, a6 = a0 + 0.6, a7 = a0 + 0.7;
#pragma unroll 4
  for (int i = 0; i < iters; ++i) {
    a0 = fma(a0, x, y); a1 = fma(a1, x, y); a2 = fma(a2, x, y); a3 = fma(a3, x, y);
    a4 = fma(a4, x, y); a5 = fma(a5, x, y); a6 = fma(a6, x, y); a7 = fma(a7, x, y);
  }
  const double s = ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
  // never true for the arguments the host passes; keeps the chains live
  if (s == -1.0) out[blockIdx.x] = s;
}

}  // namespace hss

extern "C" int hss_fp64_fma_rate(int blocks, int iters, float *ms, double *tflops, void *stream) {
  if (blocks <= 0 || iters <= 0 || !ms || !tflops) return -1;
  cudaStream_t st = (cudaStream_t)stream;
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess) return 1000000;
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return 1000000;
  }
  hss::k_fp64_fma_rate<<<blocks, 256, 0, st>>>(iters, 0.999999, 1e-6, nullptr);  // warm-up
  cudaEventRecord(e0, st);
  hss::k_fp64_fma_rate<<<blocks, 256, 0, st>>>(iters, 0.999999, 1e-6, nullptr);
  cudaEventRecord(e1, st);
  cudaError_t e = cudaEventSynchronize(e1);
  if (e == cudaSuccess) e = cudaGetLastError();
  float t = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (e != cudaSuccess) return 1000000;
  *ms = t;
  *tflops = 2.0 * 8.0 * 256.0 * (double)blocks * (double)iters / (t * 1e-3) / 1e12;
  return 0;
}
