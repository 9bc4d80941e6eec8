// hsschol.cu -- HSS Cholesky factorisation of a dense SPD matrix and its solves
// on sm_103a (HssCholSolver, SRC/HssCholSolver.f90:1-139, with mat2hsscholsvd /
// mat2hsscholsvdr, solvecholsvd and cg of SRC/mat2hsssvd.f90).
//
// The method (Li, Gu, Wu, Xia, SIMAX 33, 2012): at a node with diagonal block
// D = L L^T and block column T (the node's variables against every other
// current variable), the scaled block column T L^{-T} is compressed: its right
// singular vectors V = [V1 V2] split at the singular values above tol (rank rk,
// at most ncol).  With Q = [V2 V1] and the QL factorisation L Q = Qt Lt, the
// node's variables in the basis Qt decouple: the first ir = m - rk of them touch
// nothing outside the node once T L^{-T} V2 is dropped, so they are eliminated
// by Lt11, and the remaining rk carry the Schur complement Lt22 Lt22^T and the
// block column T W with W = L^{-T} V1 Lt22^T.  Parents stack their children's
// remaining variables; the root is factored by a plain Cholesky.  The
// factorisation is SPD by construction (every Schur complement is Lt22 Lt22^T).
//
// The reference visits the nodes in post order, one at a time, packing the
// partially compressed matrix in a stack (mat2hsssvd.f90:117-264).  Here all
// nodes of one tree height are compressed at once on an explicit reduced matrix
// Ah in HBM (each active node owns a contiguous range, in leaf order): a batched
// Cholesky of the diagonal blocks, the scaled block columns Ah(:, I) L^{-T} as a
// grouped GEMM (the node's own rows zeroed), their right singular vectors by the
// TSQR / pivoted-QR / Jacobi kernels of the dense HSS construction (or, for the
// randomised variant, of the ps x m sketches Omega X), the per-node QL step, and
// the congruence Ah' = W^T Ah W (W block diagonal; W_i = I for nodes that keep
// their variables) as two grouped GEMMs around a transpose -- its diagonal
// blocks are exactly Lt22 Lt22^T.  Nodes of one height see each other's
// variables uncompressed, so the kept subspaces differ from the sequential
// order's by the truncation tolerance; with no truncation both are exact.
//
// Solves run level by level in the same order: forward, each compressed node
// applies Qt^T, eliminates its first ir entries with Lt11 and hands Lt21's
// update of the remaining rk to the next level; the root is solved with its
// Cholesky factor; backward reverses it (solvecholsvd, mat2hsssvd.f90:553-671).
// The preconditioned CG of the reference (cg, :674-726) runs on the device with
// a dense FP64 matrix-vector product.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "hss_common.cuh"
#include "hss_gemm.h"
#include "hss_hss.h"
#include "hss_plan.h"
#include "hss_pool.h"
#include "hss_chol.h"

namespace hss {

#define CCK(x)                                                                              \
  do {                                                                                      \
    cudaError_t e_ = (x);                                                                   \
    if (e_ != cudaSuccess) throw HssError{std::string(#x) + ": " + cudaGetErrorString(e_)}; \
  } while (0)

constexpr int CHT = 256;  // threads per node CTA
constexpr size_t CH_SLOT = (size_t)CH_MAXM * CH_MAXM;

// ------------------------------------------------------------- kernels ----

// Cholesky D = L L^T of each node's diagonal block (one CTA per node, the block
// in shared memory); L (lower, m x m) and It = L^{-T} (upper) to the node's
// scratch slot.  status |= 1 when a pivot is not positive.
__global__ void __launch_bounds__(CHT)
k_ch_chol(const ChNode *__restrict__ nd, const double *__restrict__ Ah, long long lda,
          double *__restrict__ Lb, double *__restrict__ Ib, int *__restrict__ status) {
  extern __shared__ double S[];  // column j at S + j * (m + 1)
  __shared__ int bad;
  const ChNode q = nd[blockIdx.x];
  const int m = q.m, ld = m + 1, tid = threadIdx.x;
  const double *D = Ah + (long long)q.o * lda + q.o;
  for (int e = tid; e < m * m; e += CHT) {
    const int j = e / m, i = e - j * m;
    S[j * ld + i] = D[(long long)j * lda + i];
  }
  if (tid == 0) bad = 0;
  __syncthreads();
  for (int j = 0; j < m; ++j) {
    if (tid == 0) {
      const double d = S[j * ld + j];
      if (!(d > 0.0)) { bad = 1; S[j * ld + j] = 1.0; }
      else S[j * ld + j] = sqrt(d);
    }
    __syncthreads();
    if (bad) break;
    const double piv = S[j * ld + j];
    for (int i = j + 1 + tid; i < m; i += CHT) S[j * ld + i] /= piv;
    __syncthreads();
    const int t = m - j - 1;
    for (int e = tid; e < t * t; e += CHT) {
      const int kk = e / t, ii = e - kk * t;
      if (ii >= kk) S[(j + 1 + kk) * ld + j + 1 + ii] -= S[j * ld + j + 1 + ii] * S[j * ld + j + 1 + kk];
    }
    __syncthreads();
  }
  if (bad) {
    if (tid == 0) atomicOr(status, 1);
    return;
  }
  double *L = Lb + (size_t)q.slot * CH_SLOT, *It = Ib + (size_t)q.slot * CH_SLOT;
  for (int e = tid; e < m * m; e += CHT) {
    const int j = e / m, i = e - j * m;
    L[(long long)j * m + i] = i >= j ? S[j * ld + i] : 0.0;
  }
  // It(c, i) = L^{-1}(i, c): column c of L^{-1} by forward substitution
  for (int c = tid; c < m; c += CHT) {
    for (int i = 0; i < c; ++i) It[c + (long long)i * m] = 0.0;
    for (int i = c; i < m; ++i) {
      double s = (i == c) ? 1.0 : 0.0;
      for (int l = c; l < i; ++l) s -= S[l * ld + i] * It[c + (long long)l * m];
      It[c + (long long)i * m] = s / S[i * ld + i];
    }
  }
}

// Rows of the node's own range in its scaled block column X(:, I) set to zero.
__global__ void k_ch_zero_own(const ChNode *__restrict__ nd, double *__restrict__ X, long long ld) {
  const ChNode q = nd[blockIdx.x];
  for (int e = threadIdx.x; e < q.m * q.m; e += blockDim.x) {
    const int j = e / q.m, i = e - j * q.m;
    X[(long long)(q.o + j) * ld + q.o + i] = 0.0;
  }
}

// The QL step of one compressed node (one CTA; m <= 128).  In: L, It = L^{-T}
// (scratch slot), V1 = the first rk right singular vectors (P, ld m).  Out: Qt
// and Lt (m x m each, the factor store), W = It V1 Lt22^T (m x rk, scratch).
//   1. Householder QR of V1 (m x rk); the columns rk .. m-1 of its orthogonal
//      factor span the complement V2.  Q = [V2 V1].
//   2. M = L Q in shared memory; QL factorisation M = Qt Lt by Householder
//      reflectors from the last column up (DGEQL2's order), Qt formed
//      explicitly.
__global__ void __launch_bounds__(CHT)
k_ch_node(const ChNode *__restrict__ nd, const double *__restrict__ Lb,
          const double *__restrict__ Ib, const double *__restrict__ Pb, double *__restrict__ Gb,
          double *__restrict__ fac, double *__restrict__ Wb) {
  extern __shared__ double S[];  // M, column j at S + j * (m + 1)
  __shared__ double tau[CH_MAXM], sc[CH_MAXM], red[CHT / 32];
  __shared__ double s_beta;
  const ChNode q = nd[blockIdx.x];
  const int m = q.m, rk = q.rk, ir = q.ir, ld = m + 1, tid = threadIdx.x;
  const int lane = tid & 31, wid = tid >> 5;
  const size_t so = (size_t)q.slot * CH_SLOT;
  const double *L = Lb + so, *It = Ib + so, *P = Pb + so;
  double *G = Gb + 4 * so;          // Householder QR of V1 (m x rk)
  double *Q = G + CH_SLOT;          // [V2 V1]
  double *Vq = Q + CH_SLOT;         // QL reflectors (column c: rows 0..c-1)
  double *Y = Vq + CH_SLOT;         // It V1
  double *Qt = fac + q.f, *Lt = Qt + (size_t)m * m;
  double *W = Wb + so;
  for (int e = tid; e < m * rk; e += CHT) G[e] = P[e];
  __syncthreads();
  // ---- 1. QR of V1: reflector k = [1; G(k+1:m, k) * sc[k]]
  for (int k = 0; k < rk; ++k) {
    double a = 0.0;
    for (int i = k + 1 + tid; i < m; i += CHT) { const double x = G[k * m + i]; a = fma(x, x, a); }
    a = warp_sum(a);
    if (lane == 0) red[wid] = a;
    __syncthreads();
    if (tid == 0) {
      double s = 0.0;
      for (int w = 0; w < CHT / 32; ++w) s += red[w];
      const double alpha = G[k * m + k];
      double beta = alpha, t = 0.0, scl = 0.0;
      if (s > 0.0) {
        beta = -copysign(sqrt(fma(alpha, alpha, s)), alpha);
        t = (beta - alpha) / beta;
        scl = 1.0 / (alpha - beta);
      }
      tau[k] = t; sc[k] = scl; s_beta = beta;
    }
    __syncthreads();
    const double t = tau[k], scl = sc[k];
    for (int j = k + 1 + tid; j < rk; j += CHT) {  // columns to the right
      double w = G[j * m + k];
      for (int i = k + 1; i < m; ++i) w = fma(G[k * m + i] * scl, G[j * m + i], w);
      w *= t;
      G[j * m + k] -= w;
      for (int i = k + 1; i < m; ++i) G[j * m + i] = fma(-w * scl, G[k * m + i], G[j * m + i]);
    }
    __syncthreads();
    for (int i = k + 1 + tid; i < m; i += CHT) G[k * m + i] *= scl;
    if (tid == 0) G[k * m + k] = s_beta;
    __syncthreads();
  }
  // ---- complement: Q(:, c) = H_0 ... H_{rk-1} e_{rk + c}, c < ir; Q(:, ir + t) = V1(:, t)
  for (int c = tid; c < ir; c += CHT) {
    double *x = Q + (long long)c * m;
    for (int i = 0; i < m; ++i) x[i] = (i == rk + c) ? 1.0 : 0.0;
    for (int k = rk - 1; k >= 0; --k) {
      double w = x[k];
      for (int i = k + 1; i < m; ++i) w = fma(G[k * m + i], x[i], w);
      w *= tau[k];
      x[k] -= w;
      for (int i = k + 1; i < m; ++i) x[i] = fma(-w, G[k * m + i], x[i]);
    }
  }
  for (int e = tid; e < m * rk; e += CHT) Q[(long long)ir * m + e] = P[e];
  __syncthreads();
  // ---- 2. M = L Q
  for (int e = tid; e < m * m; e += CHT) {
    const int j = e / m, i = e - j * m;
    double s = 0.0;
    for (int l = 0; l <= i; ++l) s = fma(L[(long long)l * m + i], Q[(long long)j * m + l], s);
    S[j * ld + i] = s;
  }
  __syncthreads();
  // QL: column c, reflector v = [S(0:c-1, c) * sc; 1] acting on rows 0..c
  for (int c = m - 1; c >= 0; --c) {
    double a = 0.0;
    for (int i = tid; i < c; i += CHT) { const double x = S[c * ld + i]; a = fma(x, x, a); }
    a = warp_sum(a);
    if (lane == 0) red[wid] = a;
    __syncthreads();
    if (tid == 0) {
      double s = 0.0;
      for (int w = 0; w < CHT / 32; ++w) s += red[w];
      const double alpha = S[c * ld + c];
      double beta = alpha, t = 0.0, scl = 0.0;
      if (s > 0.0) {
        beta = -copysign(sqrt(fma(alpha, alpha, s)), alpha);
        t = (beta - alpha) / beta;
        scl = 1.0 / (alpha - beta);
      }
      tau[c] = t; sc[c] = scl; s_beta = beta;
    }
    __syncthreads();
    const double t = tau[c], scl = sc[c];
    for (int j = tid; j < c; j += CHT) {  // columns to the left, rows 0..c
      double w = S[j * ld + c];
      for (int i = 0; i < c; ++i) w = fma(S[c * ld + i] * scl, S[j * ld + i], w);
      w *= t;
      S[j * ld + c] -= w;
      for (int i = 0; i < c; ++i) S[j * ld + i] = fma(-w * scl, S[c * ld + i], S[j * ld + i]);
    }
    __syncthreads();
    for (int i = tid; i < c; i += CHT) {
      Vq[(long long)c * m + i] = S[c * ld + i] * scl;
      S[c * ld + i] = 0.0;
    }
    if (tid == 0) S[c * ld + c] = s_beta;
    __syncthreads();
  }
  // Lt = S (lower triangular now)
  for (int e = tid; e < m * m; e += CHT) {
    const int j = e / m, i = e - j * m;
    Lt[e] = i >= j ? S[j * ld + i] : 0.0;
  }
  // Qt = H_{m-1} ... H_0 (H_0 applied first), column j on thread j
  for (int j = tid; j < m; j += CHT) {
    double *x = Qt + (long long)j * m;
    for (int i = 0; i < m; ++i) x[i] = (i == j) ? 1.0 : 0.0;
    for (int c = 0; c < m; ++c) {
      if (tau[c] == 0.0) continue;
      double w = x[c];
      for (int i = 0; i < c; ++i) w = fma(Vq[(long long)c * m + i], x[i], w);
      w *= tau[c];
      x[c] -= w;
      for (int i = 0; i < c; ++i) x[i] = fma(-w, Vq[(long long)c * m + i], x[i]);
    }
  }
  // Y = It V1 (It upper triangular)
  for (int e = tid; e < m * rk; e += CHT) {
    const int t = e / m, i = e - t * m;
    double s = 0.0;
    for (int l = i; l < m; ++l) s = fma(It[(long long)l * m + i], P[(long long)t * m + l], s);
    Y[(long long)t * m + i] = s;
  }
  __syncthreads();
  // W = Y Lt22^T: W(i, j) = sum_{t <= j} Y(i, t) Lt(ir + j, ir + t)
  for (int e = tid; e < m * rk; e += CHT) {
    const int j = e / m, i = e - j * m;
    double s = 0.0;
    for (int t = 0; t <= j; ++t) s = fma(Y[(long long)t * m + i], S[(ir + t) * ld + ir + j], s);
    W[(long long)j * m + i] = s;
  }
}

// Columns [o, o + m) of A (rows x ., lda) copied to columns [o2, o2 + m) of B
// for the nodes that keep their variables (ir = 0).
__global__ void k_ch_copy_cols(const ChNode *__restrict__ nd, int nn, int rows,
                               const double *__restrict__ A, long long lda, double *__restrict__ B,
                               long long ldb) {
  const ChNode q = nd[blockIdx.y];
  if (q.ir != 0) return;
  const long long tot = (long long)rows * q.m;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < tot;
       e += (long long)gridDim.x * blockDim.x) {
    const long long j = e / rows, i = e - j * rows;
    B[(q.o2 + j) * ldb + i] = A[(q.o + j) * lda + i];
  }
}

// ---- solves: Y (level vectors, ld) for each right-hand side column
// forward: u = Qt^T y(I); u1 = Lt11^{-1} u1 (kept in y(I) for the backward
// pass); y2(I') = u2 - Lt21 u1.  Nodes that keep their variables copy.
__global__ void __launch_bounds__(CHT)
k_ch_fwd(const ChNode *__restrict__ nd, const double *__restrict__ fac, double *__restrict__ Y,
         long long ldy, double *__restrict__ Y2, long long ldy2, int nrhs) {
  __shared__ double u[CH_MAXM];
  const ChNode q = nd[blockIdx.x];
  const int m = q.m, ir = q.ir, tid = threadIdx.x, lane = tid & 31;
  for (int r = 0; r < nrhs; ++r) {
    double *y = Y + (long long)r * ldy + q.o;
    double *y2 = Y2 + (long long)r * ldy2 + q.o2;
    if (ir == 0) {
      for (int i = tid; i < m; i += CHT) y2[i] = y[i];
      continue;
    }
    const double *Qt = fac + q.f, *Lt = Qt + (size_t)m * m;
    for (int i = tid; i < m; i += CHT) {
      double s = 0.0;
      for (int l = 0; l < m; ++l) s = fma(Qt[(long long)i * m + l], y[l], s);
      u[i] = s;
    }
    __syncthreads();
    if (tid < 32) {
      for (int i = 0; i < ir; ++i) {
        double s = 0.0;
        for (int l = lane; l < i; l += 32) s = fma(Lt[(long long)l * m + i], u[l], s);
        s = warp_sum(s);
        if (lane == 0) u[i] = (u[i] - s) / Lt[(long long)i * m + i];
        __syncwarp();
      }
    }
    __syncthreads();
    for (int i = ir + tid; i < m; i += CHT) {
      double s = u[i];
      for (int l = 0; l < ir; ++l) s = fma(-Lt[(long long)l * m + i], u[l], s);
      y2[i - ir] = s;
    }
    for (int i = tid; i < ir; i += CHT) y[i] = u[i];
    __syncthreads();
  }
}

// backward: u2 = x2(I'); u1 = Lt11^{-T} (u1 - Lt21^T u2); x(I) = Qt [u1; u2].
__global__ void __launch_bounds__(CHT)
k_ch_bwd(const ChNode *__restrict__ nd, const double *__restrict__ fac, double *__restrict__ Y,
         long long ldy, const double *__restrict__ Y2, long long ldy2, int nrhs) {
  __shared__ double u[CH_MAXM];
  const ChNode q = nd[blockIdx.x];
  const int m = q.m, ir = q.ir, tid = threadIdx.x, lane = tid & 31;
  for (int r = 0; r < nrhs; ++r) {
    double *y = Y + (long long)r * ldy + q.o;
    const double *y2 = Y2 + (long long)r * ldy2 + q.o2;
    if (ir == 0) {
      for (int i = tid; i < m; i += CHT) y[i] = y2[i];
      continue;
    }
    const double *Qt = fac + q.f, *Lt = Qt + (size_t)m * m;
    for (int i = ir + tid; i < m; i += CHT) u[i] = y2[i - ir];
    __syncthreads();
    for (int l = tid; l < ir; l += CHT) {
      double s = y[l];
      for (int i = ir; i < m; ++i) s = fma(-Lt[(long long)l * m + i], u[i], s);
      u[l] = s;
    }
    __syncthreads();
    if (tid < 32) {
      for (int l = ir - 1; l >= 0; --l) {
        double s = 0.0;
        for (int i = l + 1 + lane; i < ir; i += 32) s = fma(Lt[(long long)l * m + i], u[i], s);
        s = warp_sum(s);
        if (lane == 0) u[l] = (u[l] - s) / Lt[(long long)l * m + l];
        __syncwarp();
      }
    }
    __syncthreads();
    for (int i = tid; i < m; i += CHT) {
      double s = 0.0;
      for (int l = 0; l < m; ++l) s = fma(Qt[(long long)l * m + i], u[l], s);
      y[i] = s;
    }
    __syncthreads();
  }
}

// L L^T x = y for the root (n x n lower L, one CTA), each column in place.
__global__ void __launch_bounds__(CHT)
k_ch_root(int n, const double *__restrict__ L, double *__restrict__ Y, long long ldy, int nrhs) {
  const int tid = threadIdx.x, lane = tid & 31;
  if (tid >= 32) return;
  for (int r = 0; r < nrhs; ++r) {
    double *y = Y + (long long)r * ldy;
    for (int i = 0; i < n; ++i) {
      double s = 0.0;
      for (int l = lane; l < i; l += 32) s = fma(L[(long long)l * n + i], y[l], s);
      s = warp_sum(s);
      if (lane == 0) y[i] = (y[i] - s) / L[(long long)i * n + i];
      __syncwarp();
    }
    for (int i = n - 1; i >= 0; --i) {
      double s = 0.0;
      for (int l = i + 1 + lane; l < n; l += 32) s = fma(L[(long long)i * n + l], y[l], s);
      s = warp_sum(s);
      if (lane == 0) y[i] = (y[i] - s) / L[(long long)i * n + i];
      __syncwarp();
    }
  }
}

// y = A x for column-major A (n x n, lda): partial sums over column chunks
// (grid.y), then a fixed-order reduction -- deterministic.
constexpr int GV_CHUNK = 256;
__global__ void k_gemv_part(int n, const double *__restrict__ A, long long lda,
                            const double *__restrict__ x, double *__restrict__ part) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int c0 = blockIdx.y * GV_CHUNK, c1 = min(n, c0 + GV_CHUNK);
  if (i >= n) return;
  double s = 0.0;
  for (int j = c0; j < c1; ++j) s = fma(A[(long long)j * lda + i], __ldg(x + j), s);
  part[(long long)blockIdx.y * n + i] = s;
}
__global__ void k_gemv_sum(int n, int nch, const double *__restrict__ part, double *__restrict__ y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0.0;
  for (int c = 0; c < nch; ++c) s += part[(long long)c * n + i];
  y[i] = s;
}
// out[k] = a_k . b_k for up to three pairs (partials per block, then one block)
__global__ void k_dots(int n, const double *__restrict__ a0, const double *__restrict__ b0,
                       const double *__restrict__ a1, const double *__restrict__ b1,
                       double *__restrict__ part) {
  __shared__ double red[2][CHT / 32];
  double s0 = 0.0, s1 = 0.0;
  for (int i = blockIdx.x * CHT + threadIdx.x; i < n; i += gridDim.x * CHT) {
    s0 = fma(a0[i], b0[i], s0);
    if (a1) s1 = fma(a1[i], b1[i], s1);
  }
  s0 = warp_sum(s0);
  s1 = warp_sum(s1);
  if ((threadIdx.x & 31) == 0) { red[0][threadIdx.x >> 5] = s0; red[1][threadIdx.x >> 5] = s1; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t0 = 0.0, t1 = 0.0;
    for (int w = 0; w < CHT / 32; ++w) { t0 += red[0][w]; t1 += red[1][w]; }
    part[2 * blockIdx.x] = t0;
    part[2 * blockIdx.x + 1] = t1;
  }
}
__global__ void k_dots_sum(int nb, const double *__restrict__ part, double *__restrict__ out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double t0 = 0.0, t1 = 0.0;
    for (int b = 0; b < nb; ++b) { t0 += part[2 * b]; t1 += part[2 * b + 1]; }
    out[0] = t0;
    out[1] = t1;
  }
}
// x += nu p; r -= nu z
__global__ void k_cg_update(int n, double nu, const double *__restrict__ p,
                            const double *__restrict__ z, double *__restrict__ x,
                            double *__restrict__ r) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  x[i] = fma(nu, p[i], x[i]);
  r[i] = fma(-nu, z[i], r[i]);
}
// p = y + mu p
__global__ void k_cg_dir(int n, double mu, const double *__restrict__ y, double *__restrict__ p) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = fma(mu, p[i], y[i]);
}
// uniform [0, 1) sketch entries from a counter hash (splitmix64), seeded
__global__ void k_ch_omega(long long count, unsigned long long seed, double *__restrict__ O) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  unsigned long long z = seed + 0x9E3779B97F4A7C15ull * (unsigned long long)(i + 1);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  O[i] = (double)(z >> 11) * 0x1.0p-53;
}

// ---------------------------------------------------------------- host ----

template <class T>
static T *dev_alloc(CholFactor &F, size_t count) {
  void *p = nullptr;
  CCK(cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T)));
  F.allocs.push_back(p);
  F.fac_bytes += (long long)(std::max<size_t>(count, 1) * sizeof(T));
  return (T *)p;
}

static void set_smem(const void *fn, size_t bytes) {
  CCK(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
}

constexpr size_t CH_SMEM = (size_t)CH_MAXM * (CH_MAXM + 1) * sizeof(double);

// Factor A (n x n, lda; read only), leaves of ni rows (npart's tree), singular
// values above tol kept, at most ncol per node.  ps = 0: the scaled block
// columns are compressed by their exact right singular vectors (RS = 'S');
// ps > 0: by those of a ps-row uniform [0, 1) sketch (RS = 'R', as the
// reference's random_number Omega).  Returns 0 or a status: 1 not positive
// definite, 2 a node of more than 128 rows.
int hss_chol_factor_core(int n, const double *A, long long lda, int ni, double tol, int ncol,
                         int ps, unsigned long long seed, CholFactor &F, cudaStream_t st) {
  F.n = n;
  const HostTree t = make_tree(n, ni);
  const int ltr = t.ltr;
  if (t.mmax > CH_MAXM) return 2;
  std::vector<int> height(ltr + 1, 0);
  for (int i = 1; i <= ltr; ++i)
    if (!t.leaf(i)) height[i] = 1 + std::max(height[t.c1[i]], height[t.c2[i]]);
  const int H = height[ltr];
  static bool attr = false;
  if (!attr) {
    set_smem((const void *)k_ch_chol, CH_SMEM);
    set_smem((const void *)k_ch_node, CH_SMEM);
    attr = true;
  }
  const size_t nn = (size_t)n * n;
  double *cur = pool<double>("hc_A0", nn), *nxt = pool<double>("hc_A1", nn);
  double *X = pool<double>("hc_X", nn), *Xt = pool<double>("hc_Xt", nn);
  const int nslot = t.lm;  // a level factors at most one node per leaf
  double *Lb = pool<double>("hc_L", nslot * CH_SLOT), *Ib = pool<double>("hc_I", nslot * CH_SLOT);
  double *Pb = pool<double>("hc_P", nslot * CH_SLOT), *PTb = pool<double>("hc_PT", nslot * CH_SLOT);
  double *Gb = pool<double>("hc_G", 4 * nslot * CH_SLOT), *Wb = pool<double>("hc_W", nslot * CH_SLOT);
  int *status = pool<int>("hc_status", 2);
  double *Om = nullptr, *Ys = nullptr;
  if (ps > 0) {
    Om = pool<double>("hc_omega", (size_t)ps * n);
    Ys = pool<double>("hc_sketch", (size_t)nslot * ps * CH_MAXM);
    const long long cnt = (long long)ps * n;
    k_ch_omega<<<(unsigned)((cnt + 255) / 256), 256, 0, st>>>(cnt, seed, Om);
  }
  CCK(cudaMemsetAsync(status, 0, 2 * sizeof(int), st));
  CCK(cudaMemcpy2DAsync(cur, sizeof(double) * n, A, sizeof(double) * lda, sizeof(double) * n, n,
                        cudaMemcpyDeviceToDevice, st));
  std::vector<int> ids, sizes;  // the active nodes, left to right
  for (int i = 1, it = 0; i <= ltr; ++i)
    if (t.leaf(i)) { ids.push_back(i); sizes.push_back(t.m[it++]); }
  int Nc = n;
  for (int h = 0; h <= H; ++h) {
    // the parents of this height take over their (adjacent) children's ranges
    for (int p = 1; p <= ltr; ++p) {
      if (t.leaf(p) || height[p] != h) continue;
      const int a = (int)(std::find(ids.begin(), ids.end(), t.c1[p]) - ids.begin());
      if (a + 1 >= (int)ids.size() || ids[a + 1] != t.c2[p])
        throw HssError{"hsschol: children not adjacent"};
      ids[a] = p;
      sizes[a] += sizes[a + 1];
      ids.erase(ids.begin() + a + 1);
      sizes.erase(sizes.begin() + a + 1);
    }
    if (h == H) break;
    const int na = (int)ids.size();
    std::vector<ChNode> nodes(na);
    std::vector<ChNode> cand;
    for (int k = 0, o = 0; k < na; ++k) {
      nodes[k] = ChNode{o, sizes[k], 0, sizes[k], 0, -1, 0};
      // mat2hsssvd.f90:136, :210: only blocks of 20 or more rows with 20 or
      // more other variables are compressed
      if (height[ids[k]] == h && sizes[k] >= 20 && Nc - sizes[k] >= 20) {
        if (sizes[k] > CH_MAXM) return 2;
        nodes[k].slot = (int)cand.size();
        cand.push_back(nodes[k]);
      }
      o += sizes[k];
    }
    std::vector<int> rk(cand.size(), 0);
    if (!cand.empty()) {
      ChNode *dc = pool<ChNode>("hc_cand", cand.size());
      stage_h2d(dc, cand.data(), cand.size() * sizeof(ChNode), st);
      k_ch_chol<<<(unsigned)cand.size(), CHT, CH_SMEM, st>>>(dc, cur, Nc, Lb, Ib, status);
      std::vector<GemmDesc> g;  // X(:, I) = Ah(:, I) L^{-T}
      for (auto &q : cand)
        g.push_back(GemmDesc{cur + (long long)q.o * Nc, Ib + (size_t)q.slot * CH_SLOT,
                             X + (long long)q.o * Nc, Nc, q.m, Nc, Nc, q.m, q.m, 0, 0});
      launch_gemm(g, 0, st);
      k_ch_zero_own<<<(unsigned)cand.size(), 256, 0, st>>>(dc, X, Nc);
      std::vector<const double *> xs;
      std::vector<int> rows, cols;
      std::vector<long long> lds;
      std::vector<double *> P, PT;
      if (ps > 0) {  // sketches Omega(:, 0:Nc) X(:, I), ps x m
        std::vector<GemmDesc> gs;
        for (auto &q : cand)
          gs.push_back(GemmDesc{Om, X + (long long)q.o * Nc, Ys + (size_t)q.slot * ps * CH_MAXM, ps,
                                Nc, ps, ps, q.m, Nc, 0, 0});
        launch_gemm(gs, 0, st);
      }
      for (auto &q : cand) {
        if (ps > 0) {
          xs.push_back(Ys + (size_t)q.slot * ps * CH_MAXM);
          rows.push_back(ps);
          lds.push_back(ps);
        } else {
          xs.push_back(X + (long long)q.o * Nc);
          rows.push_back(Nc);
          lds.push_back(Nc);
        }
        cols.push_back(q.m);
        P.push_back(Pb + (size_t)q.slot * CH_SLOT);
        PT.push_back(PTb + (size_t)q.slot * CH_SLOT);
      }
      int hs[2] = {0, 0};
      CCK(cudaMemcpyAsync(hs, status, sizeof hs, cudaMemcpyDeviceToHost, st));
      rk = tall_right_bases(xs, rows, cols, lds, P, PT, tol, st);  // synchronises
      if (hs[0]) return 1;
    }
    // ranks (at most ncol), the next level's ranges, the factor offsets
    ChLevel L;
    L.Nc = Nc;
    long long ftot = 0;
    std::vector<ChNode> comp;
    for (int k = 0, o2 = 0; k < na; ++k) {
      ChNode &q = nodes[k];
      const int r = q.slot >= 0 ? std::max(0, std::min(rk[q.slot], ncol)) : q.m;
      if (q.slot >= 0 && r < q.m) {
        q.rk = r;
        q.ir = q.m - r;
        q.f = ftot;
        ftot += 2LL * q.m * q.m;
        F.max_rank = std::max(F.max_rank, r);
      } else {
        q.rk = q.m;
        q.ir = 0;
      }
      q.o2 = o2;
      o2 += q.rk;
      sizes[k] = q.rk;
    }
    for (const ChNode &q : nodes)
      if (q.ir > 0) comp.push_back(q);
    const int Nc2 = nodes.empty() ? 0 : nodes.back().o2 + nodes.back().rk;
    L.Nc2 = Nc2;
    L.fac = dev_alloc<double>(F, (size_t)ftot);
    L.d_nodes = dev_alloc<ChNode>(F, nodes.size());
    CCK(cudaMemcpyAsync(L.d_nodes, nodes.data(), nodes.size() * sizeof(ChNode),
                        cudaMemcpyHostToDevice, st));
    if (!comp.empty()) {
      ChNode *dq = pool<ChNode>("hc_comp", comp.size());
      stage_h2d(dq, comp.data(), comp.size() * sizeof(ChNode), st);
      k_ch_node<<<(unsigned)comp.size(), CHT, CH_SMEM, st>>>(dq, Lb, Ib, Pb, Gb, L.fac, Wb);
    }
    // congruence Ah' = W^T Ah W: X2 = Ah W, Xt = X2^T, Ah' = Xt W
    {
      std::vector<GemmDesc> g1, g2;
      for (auto &q : comp) {
        if (q.rk == 0) continue;  // every variable of the node eliminated
        const double *Wq = Wb + (size_t)q.slot * CH_SLOT;
        g1.push_back(GemmDesc{cur + (long long)q.o * Nc, Wq, X + (long long)q.o2 * Nc, Nc, q.m, Nc,
                              Nc, q.rk, q.m, 0, 0});
        g2.push_back(GemmDesc{Xt + (long long)q.o * Nc2, Wq, nxt + (long long)q.o2 * Nc2, Nc2, q.m,
                              Nc2, Nc2, q.rk, q.m, 0, 0});
      }
      const unsigned gx = (unsigned)std::min<long long>(((long long)Nc * CH_MAXM + 255) / 256, 512);
      if (Nc2 > 0) {
        launch_gemm(g1, 0, st);
        k_ch_copy_cols<<<dim3(gx, (unsigned)na), 256, 0, st>>>(L.d_nodes, na, Nc, cur, Nc, X, Nc);
        transpose(Nc, Nc2, X, Nc, Xt, Nc2, st);
        launch_gemm(g2, 0, st);
        k_ch_copy_cols<<<dim3(gx, (unsigned)na), 256, 0, st>>>(L.d_nodes, na, Nc2, Xt, Nc2, nxt,
                                                                Nc2);
      }
    }
    L.nodes = nodes;
    F.lv.push_back(L);
    std::swap(cur, nxt);
    Nc = Nc2;
  }
  // the root: a plain Cholesky of what is left (mat2hsssvd.f90:266-278)
  F.Nroot = Nc;
  if (Nc > CH_MAXM) return 2;
  F.root = dev_alloc<double>(F, (size_t)Nc * Nc);
  if (Nc > 0) {
    std::vector<ChNode> r1{ChNode{0, Nc, 0, Nc, 0, 0, 0}};
    ChNode *dr = pool<ChNode>("hc_cand", 1);
    stage_h2d(dr, r1.data(), sizeof(ChNode), st);
    CCK(cudaMemsetAsync(status, 0, sizeof(int), st));
    k_ch_chol<<<1, CHT, CH_SMEM, st>>>(dr, cur, Nc, Lb, Ib, status);
    CCK(cudaMemcpyAsync(F.root, Lb, sizeof(double) * Nc * Nc, cudaMemcpyDeviceToDevice, st));
    int hs = 0;
    CCK(cudaMemcpyAsync(&hs, status, sizeof hs, cudaMemcpyDeviceToHost, st));
    CCK(cudaStreamSynchronize(st));
    if (hs) return 1;
  }
  CCK(cudaGetLastError());
  return 0;
}

// B (n x nrhs, ldb) <- A_hss^{-1} B with the factor (solvecholsvd).
void hss_chol_solve_core(const CholFactor &F, double *B, long long ldb, int nrhs, cudaStream_t st) {
  const int n = F.n, nl = (int)F.lv.size();
  std::vector<long long> off(nl + 2, 0);
  std::vector<int> dim(nl + 1);
  for (int h = 0; h < nl; ++h) dim[h] = F.lv[h].Nc;
  dim[nl] = F.Nroot;
  for (int h = 0; h <= nl; ++h) off[h + 1] = off[h] + (long long)dim[h] * nrhs;
  double *Y = pool<double>("hc_Y", (size_t)std::max<long long>(off[nl + 1], 1));
  CCK(cudaMemcpy2DAsync(Y, sizeof(double) * n, B, sizeof(double) * ldb, sizeof(double) * n, nrhs,
                        cudaMemcpyDeviceToDevice, st));
  for (int h = 0; h < nl; ++h)
    k_ch_fwd<<<(unsigned)F.lv[h].nodes.size(), CHT, 0, st>>>(F.lv[h].d_nodes, F.lv[h].fac,
                                                             Y + off[h], dim[h], Y + off[h + 1],
                                                             dim[h + 1], nrhs);
  if (F.Nroot > 0) k_ch_root<<<1, 32, 0, st>>>(F.Nroot, F.root, Y + off[nl], F.Nroot, nrhs);
  for (int h = nl - 1; h >= 0; --h)
    k_ch_bwd<<<(unsigned)F.lv[h].nodes.size(), CHT, 0, st>>>(F.lv[h].d_nodes, F.lv[h].fac,
                                                             Y + off[h], dim[h], Y + off[h + 1],
                                                             dim[h + 1], nrhs);
  CCK(cudaMemcpy2DAsync(B, sizeof(double) * ldb, Y, sizeof(double) * n, sizeof(double) * n, nrhs,
                        cudaMemcpyDeviceToDevice, st));
}

static void gemv(int n, const double *A, long long lda, const double *x, double *y, double *part,
                 cudaStream_t st) {
  const int nch = (n + GV_CHUNK - 1) / GV_CHUNK;
  k_gemv_part<<<dim3((n + 127) / 128, nch), 128, 0, st>>>(n, A, lda, x, part);
  k_gemv_sum<<<(n + 255) / 256, 256, 0, st>>>(n, nch, part, y);
}

// two dot products (the second optional) read back to the host
static void dots(int n, const double *a0, const double *b0, const double *a1, const double *b1,
                 double *out, double *part, double *dout, cudaStream_t st) {
  const int nb = std::min(256, (n + CHT - 1) / CHT);
  k_dots<<<nb, CHT, 0, st>>>(n, a0, b0, a1, b1, part);
  k_dots_sum<<<1, 32, 0, st>>>(nb, part, dout);
  CCK(cudaMemcpyAsync(out, dout, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
  CCK(cudaStreamSynchronize(st));
}

// Preconditioned CG (cg, mat2hsssvd.f90:674-726) on the device: x <- the
// solution of A x = b (A n x n, lda), preconditioner the HSS Cholesky solve
// when F is given.  Stops when |r| / |b| < tau or after maxit + 1 steps, as the
// reference's loop.  Returns the steps; *relres the last relative residual.
int hss_chol_pcg_core(const CholFactor *F, int n, const double *A, long long lda, const double *b,
                      double *x, double tau, int maxit, double *relres, cudaStream_t st) {
  double *v = pool<double>("hc_cg", (size_t)5 * n);
  double *r = v, *p = v + n, *y = v + 2 * n, *z = v + 3 * n;
  const int nch = (n + GV_CHUNK - 1) / GV_CHUNK;
  double *part = pool<double>("hc_cg_part", (size_t)std::max(nch * n, 512));
  double *dout = pool<double>("hc_cg_dot", 2);
  CCK(cudaMemcpyAsync(r, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
  CCK(cudaMemcpyAsync(p, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
  CCK(cudaMemsetAsync(x, 0, sizeof(double) * n, st));
  double h[2];
  dots(n, b, b, nullptr, nullptr, h, part, dout, st);
  const double tb = sqrt(h[0]);
  if (F) hss_chol_solve_core(*F, p, n, 1, st);
  CCK(cudaMemcpyAsync(y, p, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
  double res = tb > 0.0 ? 1.0 : 0.0;
  int it = 0;
  dots(n, y, r, nullptr, nullptr, h, part, dout, st);
  double dt = h[0];
  const unsigned g = (unsigned)((n + 255) / 256);
  while (res >= tau && it <= maxit) {
    ++it;
    gemv(n, A, lda, p, z, part, st);
    dots(n, p, z, nullptr, nullptr, h, part, dout, st);
    const double nu = dt / h[0];
    k_cg_update<<<g, 256, 0, st>>>(n, nu, p, z, x, r);
    CCK(cudaMemcpyAsync(y, r, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
    if (F) hss_chol_solve_core(*F, y, n, 1, st);
    dots(n, y, r, r, r, h, part, dout, st);
    const double mu = h[0] / dt;
    dt = h[0];
    k_cg_dir<<<g, 256, 0, st>>>(n, mu, y, p);
    res = sqrt(h[1]) / tb;
  }
  CCK(cudaStreamSynchronize(st));
  *relres = res;
  return it;
}

}  // namespace hss
