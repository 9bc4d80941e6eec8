// hss_build.cu -- HSS path of a merge (interim: dense Cauchy-like product).
#include <vector>

#include "hss_common.cuh"
#include "hss_gemm.h"
#include "hss_hss.h"
#include "hss_kernels.h"
#include "hss_pool.h"

namespace hss {

#define HCK(x)                                                             \
  do {                                                                     \
    cudaError_t e_ = (x);                                                  \
    if (e_ != cudaSuccess) throw HssError{std::string(#x) + ": " + cudaGetErrorString(e_)}; \
  } while (0)

static LevelView single_view(int K, cudaStream_t st) {
  int *v = pool<int>("hss_view", 4);
  double *r = pool<double>("hss_view_rho", 1);
  int hv[4] = {0, K, 0, K};
  HCK(cudaMemcpyAsync(v, hv, sizeof hv, cudaMemcpyHostToDevice, st));
  double one = 1.0;
  HCK(cudaMemcpyAsync(r, &one, sizeof one, cudaMemcpyHostToDevice, st));
  // s = v[0], K = v[1], rootoff = v[2..3]
  return LevelView{v, v + 1, r, v + 2, 1};
}

static void dense_product(int K, const double *F, const double *u, const double *v,
                          const double *difl, const double *difr, const double *X, long long ldx,
                          int nrows, double *Y, long long ldy, cudaStream_t st) {
  double *C = pool<double>("hss_denseC", (size_t)K * K);
  launch_cauchy_eig(K, F, u, v, difl, difr, C, st);
  GemmDesc g{X, C, Y, (int)ldx, K, (int)ldy, nrows, K, K, 0, 0};
  GemmDesc *dg = pool<GemmDesc>("hss_gemm1", 1);
  HCK(cudaMemcpyAsync(dg, &g, sizeof g, cudaMemcpyHostToDevice, st));
  launch_gemm_f64(1, gemm_tiles(nrows, K), dg, st);
}

int hss_merge(const HssMergeArgs &a, int *rank, cudaStream_t st) {
  LevelView lv = single_view(a.K, st);
  launch_alpha(lv, a.K, a.dl, a.difl, a.difr, a.zhat, a.alpha, st);
  // gather the non-deflated columns into X (n x K)
  double *X = pool<double>("hss_X", (size_t)a.n * a.K);
  double *T = pool<double>("hss_T", (size_t)a.n * a.K);
  int *dv = pool<int>("hss_gview", 4);
  int hv[4] = {a.s, a.n, 0, a.K};
  HCK(cudaMemcpyAsync(dv, hv, sizeof hv, cudaMemcpyHostToDevice, st));
  long long *boff = pool<long long>("hss_boff", 1);
  long long zero = 0;
  HCK(cudaMemcpyAsync(boff, &zero, sizeof zero, cudaMemcpyHostToDevice, st));
  // the gather/scatter kernels index the level arrays with s; pass ndslot - s
  launch_gather(1, a.K, a.n, dv, dv + 1, dv + 2, a.ndslot - a.s, nullptr, boff, a.Q, a.ldq, X, st);
  dense_product(a.K, a.dl, a.zhat, a.alpha, a.difl, a.difr, X, a.n, a.n, T, a.n, st);
  launch_scatter(1, a.K, a.n, dv, dv + 1, dv + 2, a.ndslot - a.s, boff, T, a.Q, a.ldq, st);
  *rank = a.K;
  return 5;
}

int hss_dhssevc_core(int K, int ni, double tol, int precision, const double *F, const double *u,
                     const double *v, const double *difl, const double *difr, double *Q,
                     long long ldq, int nrows, int *rank, cudaStream_t st) {
  (void)ni; (void)tol; (void)precision;
  double *T = pool<double>("hss_T", (size_t)nrows * K);
  dense_product(K, F, u, v, difl, difr, Q, ldq, nrows, T, nrows, st);
  HCK(cudaMemcpy2DAsync(Q, ldq * sizeof(double), T, nrows * sizeof(double), nrows * sizeof(double), K,
                        cudaMemcpyDeviceToDevice, st));
  *rank = K;
  return 0;
}

}  // namespace hss
