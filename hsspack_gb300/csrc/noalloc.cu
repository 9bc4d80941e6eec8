// noalloc.cu -- Loewner rebuild of z and the column scalings alpha with no
// device allocation, for callers that must not let a library allocate.
//
// Some callers own all device memory up front -- a framework whose caching
// allocator has reserved the whole GPU, or a real-time pipeline that forbids
// allocation after start-up -- and cannot let a library call cudaMalloc on its
// hot path.  hss_lowner_noalloc_dev is the Loewner stage (the same kernels as
// hss_lowner_dev) with its scratch -- the rebuilt z_hat and the one-problem
// level descriptor -- in this file's statically sized device arrays instead of
// the library's growing buffer pool.
//
// * Limit: k <= NOALLOC_MAX_K = 65536 roots, i.e. 512 KB of z_hat scratch,
//   resident on every device that loads the library for the life of the
//   process.  A larger k returns -1 with a message in hss_last_error().
// * Set-up: every call resolves the scratch addresses in the current context
//   with cudaGetSymbolAddress, so no address outlives a context (after
//   cudaDeviceReset the next call finds the new context's copy).  The first
//   call on a device, with that device current, may also load the module on
//   it; make that first call at set-up time, before any stream capture, and
//   likewise the first call after a context reset.  Later calls only look the
//   addresses up.
// * Sharing: every call on a device uses the same scratch, which keeps the
//   last call's contents.  Calls whose kernels overlapped on the GPU would race
//   on it; this entry point serialises its callers with a lock and waits for
//   its stream before returning, so its own calls do not overlap.
// * Zeroing: each call writes every scratch element it reads (the descriptor
//   by k_noalloc_view, z_hat by the Loewner kernel) before reading it, so
//   nothing has to start at zero and nothing is cleared between calls.
// * No cudaMalloc, cudaFree or allocating library routine is called.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "../../include/hsspack_gb300.h"
#include "hss_kernels.h"

namespace hss {

constexpr int NOALLOC_MAX_K = 65536;

static __device__ __align__(256) double g_noalloc_zhat[NOALLOC_MAX_K];
static __device__ __align__(256) int g_noalloc_view[4];  // s, K, rootoff[0], rootoff[1]
static __device__ __align__(256) double g_noalloc_rho[1];

struct NoallocScratch {
  double *zhat = nullptr;
  int *view = nullptr;
  double *rho = nullptr;
};

static std::mutex g_noalloc_mu;

// One merge covering positions [0, k): s = 0, K = k, rootoff = {0, k}.
__global__ void k_noalloc_view(int *view, double *rho, int k) {
  view[0] = 0;
  view[1] = k;
  view[2] = 0;
  view[3] = k;
  rho[0] = 1.0;
}

static int noalloc_fail(const char *what, cudaError_t e) {
  char msg[256];
  snprintf(msg, sizeof msg, "hss_lowner_noalloc_dev: %s (%s)", what, cudaGetErrorString(e));
  set_last_error(msg);
  return 1000000;
}

// An error after the first launch: wait for what was queued on the stream, so
// no kernel of this call still uses the shared scratch once the lock is gone.
static int noalloc_fail_after_launch(const char *what, cudaError_t e, cudaStream_t st) {
  (void)cudaStreamSynchronize(st);
  return noalloc_fail(what, e);
}

}  // namespace hss

using namespace hss;

extern "C" int hss_lowner_noalloc_dev(int k, const double *dlamda, const double *difl,
                                      const double *difr, double *z, double *alpha, void *stream) {
  std::lock_guard<std::mutex> g(g_noalloc_mu);
  if (k < 0 || k > NOALLOC_MAX_K) {
    char msg[160];
    snprintf(msg, sizeof msg,
             "hss_lowner_noalloc_dev: k = %d outside 0..%d (the size of its static scratch)", k,
             NOALLOC_MAX_K);
    set_last_error(msg);
    return -1;
  }
  if (k == 0) return 0;
  cudaError_t e;
  // the addresses of this device's copy of the scratch in the current context
  NoallocScratch sc;
  e = cudaGetSymbolAddress((void **)&sc.zhat, g_noalloc_zhat);
  if (e != cudaSuccess) return noalloc_fail("cudaGetSymbolAddress(z_hat scratch) failed", e);
  e = cudaGetSymbolAddress((void **)&sc.view, g_noalloc_view);
  if (e != cudaSuccess) return noalloc_fail("cudaGetSymbolAddress(descriptor) failed", e);
  e = cudaGetSymbolAddress((void **)&sc.rho, g_noalloc_rho);
  if (e != cudaSuccess) return noalloc_fail("cudaGetSymbolAddress(rho) failed", e);
  cudaStream_t st = (cudaStream_t)stream;
  k_noalloc_view<<<1, 1, 0, st>>>(sc.view, sc.rho, k);
  e = cudaGetLastError();
  if (e != cudaSuccess) return noalloc_fail_after_launch("descriptor kernel failed to launch", e, st);
  const LevelView lv{sc.view, sc.view + 1, sc.rho, sc.view + 2, 1};
  launch_lowner(lv, k, dlamda, difl, difr, z, sc.zhat, st);
  launch_alpha(lv, k, dlamda, difl, difr, sc.zhat, alpha, st);
  e = cudaMemcpyAsync(z, sc.zhat, sizeof(double) * k, cudaMemcpyDeviceToDevice, st);
  if (e != cudaSuccess) return noalloc_fail_after_launch("copy of z_hat failed", e, st);
  e = cudaStreamSynchronize(st);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return noalloc_fail("kernel failed", e);
  return 0;
}
