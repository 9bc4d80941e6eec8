// gemm_f64.cu -- grouped FP64 GEMM: C_p = A_p * B_p (+ C_p) for a list of
// problems launched together (the dense merge update Q2*S of LAPACK DLAED3 and
// the per-level products of the HSS multiply, SRC/ConstructHssd.f90:1394-1630).
//
// 64x64 output tile per CTA, 16-deep K slices double-buffered in shared
// memory, 256 threads with a 4x4 register tile each (DFMA).  Problems and
// their tiles are flattened; a CTA finds its problem by binary search on the
// tile prefix.  All operands column-major.
#include "hss_common.cuh"
#include "hss_gemm.h"
#include "hss_pool.h"

namespace hss {

constexpr int BM = 64, BN = 64, BK = 16, GT = 256;

__global__ void __launch_bounds__(GT)
k_gemm_f64(int nprob, const GemmDesc *__restrict__ probs) {
  __shared__ double As[2][BK][BM + 2];
  __shared__ double Bs[2][BK][BN + 2];
  // locate problem
  int lo = 0, hi = nprob;
  const int b = blockIdx.x;
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (probs[mid].tile0 <= b) lo = mid; else hi = mid;
  }
  const GemmDesc P = probs[lo];
  const int t = b - P.tile0;
  const int tm = (P.M + BM - 1) / BM;
  const int m0 = (t % tm) * BM, n0 = (t / tm) * BN;
  const int tid = threadIdx.x;
  const int tx = tid % 16, ty = tid / 16;  // thread owns rows tx*4.., cols ty*4..
  double acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;
  const int nk = (P.K + BK - 1) / BK;
  auto load = [&](int buf, int kb) {
    const int k0 = kb * BK;
    // A tile: BM x BK, 1024 values, 4 per thread (column-major: row fastest)
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int idx = tid + r * GT;
      const int row = idx % BM, kk = idx / BM;
      const int gr = m0 + row, gk = k0 + kk;
      As[buf][kk][row] = (gr < P.M && gk < P.K) ? P.A[(long long)gk * P.lda + gr] : 0.0;
    }
    // B tile: BK x BN
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int idx = tid + r * GT;
      const int kk = idx % BK, col = idx / BK;
      const int gk = k0 + kk, gc = n0 + col;
      Bs[buf][kk][col] = (gk < P.K && gc < P.N) ? P.B[(long long)gc * P.ldb + gk] : 0.0;
    }
  };
  if (nk > 0) load(0, 0);
  __syncthreads();
  for (int kb = 0; kb < nk; ++kb) {
    const int cur = kb & 1;
    if (kb + 1 < nk) load(cur ^ 1, kb + 1);
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      double a[4], bb[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[cur][kk][tx * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) bb[j] = Bs[cur][kk][ty * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], bb[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int gc = n0 + ty * 4 + j;
    if (gc >= P.N) continue;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int gr = m0 + tx * 4 + i;
      if (gr >= P.M) continue;
      double *c = P.C + (long long)gc * P.ldc + gr;
      *c = P.beta ? *c + acc[i][j] : acc[i][j];
    }
  }
}

int gemm_tiles(int M, int N) { return ((M + BM - 1) / BM) * ((N + BN - 1) / BN); }

// Small products (N, K <= 32: the lowest DC levels): one thread per output
// element, the K-term dot product from L1 (a 64 x 64 tile would be mostly
// empty).  Problem p owns outputs [eoff[p], eoff[p+1]).
__global__ void __launch_bounds__(256)
k_gemm_small(int nprob, const GemmDesc *__restrict__ probs, const long long *__restrict__ eoff) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= eoff[nprob]) return;
  int lo = 0, hi = nprob;
  while (hi - lo > 1) { const int mid = (lo + hi) >> 1; if (eoff[mid] <= idx) lo = mid; else hi = mid; }
  const GemmDesc P = probs[lo];
  const long long e = idx - eoff[lo];
  const int i = (int)(e % P.M), j = (int)(e / P.M);
  const double *a = P.A + i, *b = P.B + (long long)j * P.ldb;
  double acc = 0.0;
  for (int k = 0; k < P.K; ++k) acc = fma(__ldg(a + (long long)k * P.lda), __ldg(b + k), acc);
  double *c = P.C + (long long)j * P.ldc + i;
  *c = P.beta ? *c + acc : acc;
}

// largest N and K taken by the element kernel (hss_config.small_nk; 0: 128,
// measured faster than 64 x 64 FP64 tiles for the DC merges' K <= 128)
static int g_small_nk = 128;
void set_small_nk(int v) { g_small_nk = v > 0 ? v : 128; }

// split-BF16 thresholds (hss_config.split_min_log2, split_min_m):
// M*N*K >= 2^g_split_log2 and M >= g_split_m
static int g_split_log2 = 15;
void set_split_min_log2(int v) { g_split_log2 = v > 0 ? v : 15; }
static int g_split_m = 128;
void set_split_min_m(int v) { g_split_m = v > 0 ? v : 128; }
// 0: digit planes written to global memory first, then the TMA-fed product
// kernel; 1: operands split inside each CTA of the product kernel
// (hss_config.gemm_path; the staged form measures faster on the DC shapes)
static int g_gemm_path = 0;
void set_gemm_path(int v) { g_gemm_path = v == 1 ? 1 : 0; }

void launch_gemm_f64(int nprob, int total_tiles, const GemmDesc *d_probs, cudaStream_t st) {
  if (nprob <= 0 || total_tiles <= 0) return;
  k_gemm_f64<<<total_tiles, GT, 0, st>>>(nprob, d_probs);
}

void launch_gemm(const std::vector<GemmDesc> &probs, int precision, cudaStream_t st) {
  if (probs.empty()) return;
  // one pass: tensor-core splitting pays off once a product has enough MACs
  // per operand byte (precision 1); the rest stay on the FP64 pipe, small
  // ones (N, K <= g_small_nk) by the element kernel, others by 64 x 64 tiles
  const double big_macs = ldexp(1.0, g_split_log2);
  std::vector<GemmDesc> big, tiny, tiled;
  tiny.reserve(probs.size());
  for (const auto &p : probs) {
    if (precision == 1 && (double)p.M * p.N * p.K >= big_macs && p.M >= g_split_m) big.push_back(p);
    else if (p.N <= g_small_nk && p.K <= g_small_nk) tiny.push_back(p);
    else tiled.push_back(p);
  }
  if (!big.empty()) {
    int *err = pool<int>("gemm_err", 1);
    if (g_gemm_path == 1) launch_gemm_fused(big, err, st);
    else launch_gemm_split(big, err, st);
  }
  if (!tiny.empty()) {
    std::vector<long long> eoff(tiny.size() + 1);
    eoff[0] = 0;
    for (size_t i = 0; i < tiny.size(); ++i) eoff[i + 1] = eoff[i] + (long long)tiny[i].M * tiny[i].N;
    GemmDesc *d = pool<GemmDesc>("gemm_small_probs", tiny.size());
    long long *de = pool<long long>("gemm_small_eoff", eoff.size());
    stage_h2d(d, tiny.data(), tiny.size() * sizeof(GemmDesc), st);
    stage_h2d(de, eoff.data(), eoff.size() * sizeof(long long), st);
    if (eoff.back() > 0)
      k_gemm_small<<<(unsigned)((eoff.back() + 255) / 256), 256, 0, st>>>((int)tiny.size(), d, de);
  }
  if (tiled.empty()) return;
  int tiles = 0;
  for (auto &p : tiled) { p.tile0 = tiles; tiles += gemm_tiles(p.M, p.N); }
  GemmDesc *d = pool<GemmDesc>("gemm_f64_probs", tiled.size());
  stage_h2d(d, tiled.data(), tiled.size() * sizeof(GemmDesc), st);
  launch_gemm_f64((int)tiled.size(), tiles, d, st);
}

}  // namespace hss
