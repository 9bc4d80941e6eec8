// band_sbr.cu -- symmetric band -> tridiagonal reduction on the GPU
// (Householder bulge chasing) and the back-transformation of eigenvectors.
//
// The reference reduces a band matrix to tridiagonal form with LAPACK DSBTRD
// (Givens rotations) where it does not run its own band divide and conquer:
// eigenvalues only (SRC/mdsbedc.f90:311-318, DSBTRD + DSTERF) and, through
// DSBEVD, bandwidths above 16 (SRC/mdsbedc.f90:274-276).  Here the same
// reduction is done with Householder reflectors of length b (the bandwidth),
// the bulge-chasing order of successive band reduction:
//
//   sweep s (s = 0 .. n-3), step j (p = s+1+j b, q = min(p+b-1, n-1)):
//     the reflector H = I - tau v v^T on rows p..q annihilates A(p+1..q, c),
//     c = s at step 0 and c = p-b (the first column of the bulge the previous
//     step created) after; it is applied from the left to A(p..q, c..p-1),
//     from both sides to the diagonal block A(p..q, p..q) and from the right
//     to A(q+1..q+b, p..q), which leaves the next bulge there.
//
// A step touches rows and columns p-b .. q+b only, so sweep s+1 can follow
// sweep s a fixed number of steps behind: with S steps per CTA ("super-step")
// and sweep s at super-step u = t - lag s in wavefront t, the regions of the
// sweeps active in one wavefront are disjoint for lag > 1 + 2/S, and every
// region is visited in the sequential order.  One launch per wavefront, one
// CTA per active sweep; the band lives in HBM/L2 in lower storage with 2b
// diagonals (the bulges reach 2b-1 below the diagonal).
//
// Eigenvectors: Z = Q Z_T with Q the product of all reflectors in creation
// order; the reflectors of one sweep act on disjoint row ranges, so the
// back-transformation applies one sweep per launch (last sweep first), every
// reflector of the sweep and every column chunk of Z in parallel.
#include <vector>

#include "hss_common.cuh"
#include "hss_kernels.h"

namespace hss {

__host__ __device__ inline int sbr_nsteps(int n, int b, int s) {
  return (b < 2 || s > n - 3) ? 0 : 1 + (n - 3 - s) / b;
}

// A(i, k), 0 <= i - k < 2b, of the working band (column k's entries contiguous)
__device__ __forceinline__ double &lbat(double *LB, int ldb, int i, int k) {
  return LB[(long long)k * ldb + (i - k)];
}

// LB <- the lower triangle of the band given in upper storage (AB(kd+i-j, j)
// = A(i, j), i <= j), the bulge diagonals b+1 .. 2b-1 zeroed.
__global__ void k_sbr_load(int n, int kd, int b, const double *__restrict__ AB, long long ldab,
                           double *__restrict__ LB, int ldb) {
  const long long total = (long long)n * ldb;
  for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < total;
       x += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(x / ldb), dist = (int)(x % ldb), i = k + dist;
    double a = 0.0;
    if (dist <= b && dist <= kd && i < n) a = AB[(long long)i * ldab + (kd + k - i)];
    LB[x] = a;
  }
}

__device__ __forceinline__ double sbr_block_sum(double x, double *red) {
  x = warp_sum(x);
  const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[w] = x;
  __syncthreads();
  double s = 0.0;
  for (int i = 0; i < nw; ++i) s += red[i];
  return s;
}

// One wavefront: CTA x runs super-step t - lag s of sweep s = s_lo + x.
// R / rtau (may be null): reflector v (b entries) and tau of step j of sweep s
// at index roff[s] + j.
__global__ void __launch_bounds__(256)
k_sbr_wave(int n, int b, int S, int lag, int t, int s_lo, double *__restrict__ LB, int ldb,
           double *__restrict__ R, const long long *__restrict__ roff, double *__restrict__ rtau) {
  extern __shared__ double sm[];
  double *v = sm, *y = sm + b, *red = sm + 2 * b, *scal = red + 32;
  const int s = s_lo + blockIdx.x;
  const int ns = sbr_nsteps(n, b, s);
  const int u = t - lag * s;
  if (u < 0) return;
  const int j0 = u * S, j1 = min(ns, j0 + S);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  for (int j = j0; j < j1; ++j) {
    const int p = s + 1 + j * b, col = j == 0 ? s : p - b;
    const int q = min(p + b - 1, n - 1), L = q - p + 1;
    const int r = min(q + b, n - 1);
    // (1) the reflector that maps A(p..q, col) to beta e_1 (LAPACK DLARFG's form)
    double sq = 0.0;
    for (int i = threadIdx.x; i < L; i += blockDim.x) {
      const double x = lbat(LB, ldb, p + i, col);
      v[i] = x;
      if (i > 0) sq += x * x;
    }
    const double sig = sbr_block_sum(sq, red);
    if (threadIdx.x == 0) {
      const double alpha = v[0];
      double tau = 0.0, beta = alpha, scale = 0.0;
      if (sig != 0.0) {
        const double mu = sqrt(alpha * alpha + sig);
        beta = alpha >= 0.0 ? -mu : mu;
        tau = (beta - alpha) / beta;
        scale = 1.0 / (alpha - beta);
      }
      scal[0] = tau;
      scal[1] = beta;
      scal[2] = scale;
    }
    __syncthreads();
    const double tau = scal[0], beta = scal[1], scale = scal[2];
    for (int i = threadIdx.x; i < L; i += blockDim.x) {
      const double vi = i == 0 ? 1.0 : v[i] * scale;
      lbat(LB, ldb, p + i, col) = i == 0 ? beta : 0.0;
      if (R) R[(roff[s] + j) * (long long)b + i] = vi;
    }
    if (R && threadIdx.x == 0) rtau[roff[s] + j] = tau;
    __syncthreads();
    for (int i = threadIdx.x; i < L; i += blockDim.x)
      if (i > 0) v[i] *= scale;
    if (threadIdx.x == 0) v[0] = 1.0;
    __syncthreads();
    if (tau == 0.0) continue;  // x was already beta e_1: H = I
    // (2) from the left on the rest of the bulge block, columns col+1 .. p-1
    for (int k = col + 1 + warp; k < p; k += nwarp) {
      double dot = 0.0;
      for (int i = lane; i < L; i += 32) dot += v[i] * lbat(LB, ldb, p + i, k);
      dot = warp_sum(dot) * tau;
      for (int i = lane; i < L; i += 32) lbat(LB, ldb, p + i, k) -= dot * v[i];
    }
    // (3a) y = tau D v for the diagonal block (symmetric, lower stored)
    for (int i = warp; i < L; i += nwarp) {
      double acc = 0.0;
      for (int m = lane; m < L; m += 32)
        acc += (m <= i ? lbat(LB, ldb, p + i, p + m) : lbat(LB, ldb, p + m, p + i)) * v[m];
      acc = warp_sum(acc);
      if (lane == 0) y[i] = tau * acc;
    }
    // (4) from the right on the rows below, A(q+1 .. r, p .. q): the next bulge
    for (int i2 = q + 1 + warp; i2 <= r; i2 += nwarp) {
      double dot = 0.0;
      for (int m = lane; m < L; m += 32) dot += lbat(LB, ldb, i2, p + m) * v[m];
      dot = warp_sum(dot) * tau;
      for (int m = lane; m < L; m += 32) lbat(LB, ldb, i2, p + m) -= dot * v[m];
    }
    __syncthreads();
    double vy = 0.0;
    for (int i = threadIdx.x; i < L; i += blockDim.x) vy += v[i] * y[i];
    const double cc = 0.5 * tau * sbr_block_sum(vy, red);
    for (int i = threadIdx.x; i < L; i += blockDim.x) y[i] -= cc * v[i];  // y <- w
    __syncthreads();
    // (3b) D <- D - v w^T - w v^T on the lower triangle
    const int npair = L * (L + 1) / 2;
    for (int x = threadIdx.x; x < npair; x += blockDim.x) {
      // x -> (i, m), i >= m, row-major over the lower triangle
      int i = (int)((sqrt(8.0 * x + 1.0) - 1.0) * 0.5);
      while ((i + 1) * (i + 2) / 2 <= x) ++i;
      while (i * (i + 1) / 2 > x) --i;
      const int m = x - i * (i + 1) / 2;
      lbat(LB, ldb, p + i, p + m) -= v[i] * y[m] + y[i] * v[m];
    }
    __syncthreads();
  }
}

// d(i) = A(i, i), e(i) = A(i+1, i) of the reduced band.
__global__ void k_sbr_tri(int n, const double *__restrict__ LB, int ldb, double *__restrict__ d,
                          double *__restrict__ e) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    d[i] = LB[(long long)i * ldb];
    if (i + 1 < n) e[i] = LB[(long long)i * ldb + 1];
  }
}

// Z(p.., c) <- H_{s,j} Z(p.., c) for every step j of sweep s (blockIdx.x) and
// the columns of chunk blockIdx.y (64 columns, a warp per column).
__global__ void __launch_bounds__(256)
k_sbr_apply(int n, int b, int s, const double *__restrict__ R, const long long *__restrict__ roff,
            const double *__restrict__ rtau, double *__restrict__ Z, long long ldz) {
  extern __shared__ double v[];
  const int j = blockIdx.x;
  const int p = s + 1 + j * b, q = min(p + b - 1, n - 1), L = q - p + 1;
  const long long idx = roff[s] + j;
  const double tau = rtau[idx];
  if (tau == 0.0) return;
  for (int i = threadIdx.x; i < L; i += blockDim.x) v[i] = R[idx * b + i];
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int c1 = min(n, (int)(blockIdx.y + 1) * 64);
  for (int c = blockIdx.y * 64 + warp; c < c1; c += blockDim.x >> 5) {
    double *zc = Z + (long long)c * ldz + p;
    double dot = 0.0;
    for (int i = lane; i < L; i += 32) dot += v[i] * zc[i];
    dot = warp_sum(dot) * tau;
    for (int i = lane; i < L; i += 32) zc[i] -= dot * v[i];
  }
}

// ------------------------------------------------------------- host side --
int sbr_lag(int S) { return S >= 3 ? 2 : S == 2 ? 3 : 4; }

long long sbr_reflectors(int n, int b, std::vector<long long> *roff) {
  long long tot = 0;
  if (roff) roff->assign(std::max(n, 1), 0);
  for (int s = 0; s < n; ++s) {
    if (roff) (*roff)[s] = tot;
    tot += sbr_nsteps(n, b, s);
  }
  return tot;
}

void launch_sbr_load(int n, int kd, int b, const double *AB, long long ldab, double *LB, int ldb,
                     cudaStream_t st) {
  const long long total = (long long)n * ldb;
  const int grid = (int)std::min<long long>((total + 255) / 256, 152LL * 16);
  k_sbr_load<<<grid, 256, 0, st>>>(n, kd, b, AB, ldab, LB, ldb);
}

int launch_sbr_reduce(int n, int b, double *LB, int ldb, double *R, const long long *droff,
                      double *rtau, cudaStream_t st) {
  if (b < 2 || n < 3) return 0;
  const int S = std::max(1, 48 / b), lag = sbr_lag(S);
  const size_t smem = sizeof(double) * (2 * (size_t)b + 40);
  if (smem > 48 * 1024)
    (void)cudaFuncSetAttribute(k_sbr_wave, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  std::vector<int> nsup(n);
  for (int s = 0; s < n; ++s) nsup[s] = (sbr_nsteps(n, b, s) + S - 1) / S;
  int launches = 0, s_lo = 0;
  const int s_last = n - 3;
  for (int t = 0; s_lo <= s_last; ++t) {
    while (s_lo <= s_last && t - lag * s_lo >= nsup[s_lo]) ++s_lo;
    if (s_lo > s_last) break;
    const int s_hi = std::min(s_last, t / lag);
    if (s_hi < s_lo) continue;
    k_sbr_wave<<<s_hi - s_lo + 1, 256, smem, st>>>(n, b, S, lag, t, s_lo, LB, ldb, R, droff, rtau);
    ++launches;
  }
  return launches;
}

void launch_sbr_tri(int n, const double *LB, int ldb, double *d, double *e, cudaStream_t st) {
  k_sbr_tri<<<std::max(1, std::min((n + 255) / 256, 1024)), 256, 0, st>>>(n, LB, ldb, d, e);
}

int launch_sbr_back(int n, int b, const double *R, const long long *droff, const double *rtau,
                    double *Z, long long ldz, cudaStream_t st) {
  int launches = 0;
  const size_t smem = sizeof(double) * (size_t)b;
  if (smem > 48 * 1024)
    (void)cudaFuncSetAttribute(k_sbr_apply, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  for (int s = n - 3; s >= 0; --s) {
    const int ns = sbr_nsteps(n, b, s);
    if (ns == 0) continue;
    k_sbr_apply<<<dim3(ns, (n + 63) / 64), 256, smem, st>>>(n, b, s, R, droff, rtau, Z, ldz);
    ++launches;
  }
  return launches;
}

}  // namespace hss
