// mat2hss.cu -- dense matrix -> HSS by truncated SVD on sm_103a (mat2hssvd,
// SRC/ConstructHssd.f90:371-693) and the products of DHSSMM / DHSSMML
// (SRC/DHSSMM.f90:1-125, SRC/DHSSMML.f90:2-122).
//
// The reference visits the HSS tree in post order, one node at a time: the
// node's block column and block row (every current row / column outside the
// node; parts owned by nodes visited earlier are already compressed) are
// factored by DGEQRF + DGESVD and replaced by their projections on the
// singular vectors whose singular values exceed tol (count(svs > tol), an
// absolute threshold).  Here every node of one tree depth is compressed at
// once, on a reduced matrix Ah (rows x cols, column-major) that starts as the
// input and in which each node owns a contiguous row range and column range
// (leaf order; a parent's ranges are its two children's compressed ones):
//
//   row phase     node i: the block row Ah(I_i, ~J_i) (r_i x N) is factored
//                 through its transpose, R = qr(Ah(I_i, ~J_i)^T) (k_tall_qr:
//                 Householder on row tiles in shared memory; R factors of row
//                 ranges stacked and factored again), then a pivoted QR of R
//                 and one-sided Jacobi on its leading rows (k_node_basis): the
//                 block row's left singular vectors, those above tol form U_i.
//                 Ah(I_i, :) <- U_i^T Ah(I_i, :) by the grouped GEMM.
//   column phase  the same on the block column Ah(~I_j, J_j) (R = qr of the
//                 block column; the Jacobi columns are its right singular
//                 vectors): V_j, then Ah(:, J_j) <- Ah(:, J_j) V_j.
//   B generators  B_i = Ah(I_i, J_sibling(i)) after both phases.
// One host synchronisation per phase reads the ranks (the next shapes).
//
// Both factorisation kernels are FP64-pipe bound (about 2 FP64 instructions
// per clock per SM on this part), so scalar work that every lane would repeat
// (square roots and divides of a reflector or a rotation) is done by one lane
// and shared.
//
// The generators land in the layout of the Cauchy-like construction, so the
// same level-batched multiply applies: Ug(i) = U_i (rows x k), Vg(i) = V_i^T
// (k' x cols), Bg(i) = B_i (k_i x k'_sibling), leaf D_i = A(I_i, I_i).
#include <algorithm>
#include <climits>
#include <cstring>
#include <vector>

#include "hss_common.cuh"
#include "hss_gemm.h"
#include "hss_hss.h"
#include "hss_plan.h"
#include "hss_pool.h"

namespace hss {

#define MCK(x)                                                                              \
  do {                                                                                      \
    cudaError_t e_ = (x);                                                                   \
    if (e_ != cudaSuccess) throw HssError{std::string(#x) + ": " + cudaGetErrorString(e_)}; \
  } while (0)

constexpr int QR_MAXC = 128;    // largest node dimension (rows of U, rows of V)
constexpr int QT = 256;         // threads per CTA
constexpr int QR_TILE = 25000;  // doubles in the shared QR tile (195 KB)
constexpr int JAC_SWEEPS = 40;  // one-sided Jacobi sweep limit

// Rows [t0, t1) of the "tall" matrix of one node: element (t, c) lives at
// base[phys(t) * st + c * sc] with phys(t) = t below s0 and t + skip from s0
// on (the node's own block is skipped).
struct TallDesc {
  const double *base;
  long long st, sc;
  int ntot, ncol;
  int s0, skip;
};
struct QrJob {
  int desc, t0, t1;
  double *out;  // R (ncol x ncol, upper triangular), leading dim ldo
  int ldo;
};
struct BasisJob {
  const double *R;  // r x r upper triangular, leading dim r
  int r;
  double *P;   // orthonormal basis, r x k, leading dim r
  double *PT;  // its transpose, k x r, leading dim k
  int *rank;
};
struct CopyDesc {
  const double *src;
  long long lds;
  double *dst;
  long long ldd;
  int rows, cols;
};

__host__ __device__ inline int qr_chunk(int r) {
  const int nc = QR_TILE / r - r - 1;
  return nc > 256 ? 256 : nc;
}

__device__ __forceinline__ unsigned group_mask(int gs) {
  if (gs >= 32) return HSS_FULL;
  return ((1u << gs) - 1u) << ((threadIdx.x & 31) & ~(gs - 1));
}
__device__ __forceinline__ double group_sum(double v, int gs, unsigned mask) {
  for (int o = gs >> 1; o > 0; o >>= 1) v += __shfl_xor_sync(mask, v, o);
  return v;
}
// largest power of two g <= 32 with g * groups <= QT
__device__ __forceinline__ int group_size(int groups) {
  int gs = 32;
  while (gs > 1 && gs * groups > QT) gs >>= 1;
  return gs;
}

struct HousePar {
  double beta, tau, scale;
};
__device__ __forceinline__ HousePar house_par(double alpha, double sg) {
  HousePar h{alpha, 0.0, 0.0};
  if (sg > 0.0) {
    h.beta = -copysign(sqrt(fma(alpha, alpha, sg)), alpha);
    h.tau = (h.beta - alpha) / h.beta;
    h.scale = 1.0 / (alpha - h.beta);
  }
  return h;
}

// Householder QR of the tile [R; C]: rows 0..r-1 hold the upper triangular R
// so far, rows r..r+na-1 a chunk of the tall matrix; on return rows 0..r-1
// hold the R factor of both.  Column k's reflector has nonzeros only in row k
// and the chunk rows (R is triangular), v_k = 1, v_chunk = C(:, k) * scale.
// Column j > k is updated by a group of gs lanes; the group of column k + 1
// also forms that column's sum of squares and, on one lane, the next
// reflector (double-buffered in hp), so one barrier per column.
__device__ void house_tile(double *S, int LD, int r, int na, HousePar *hp, double *red) {
  const int tid = threadIdx.x;
  {
    double q = 0.0;
    for (int i = tid; i < na; i += QT) { const double x = S[r + i]; q = fma(x, x, q); }
    q = warp_sum(q);
    if ((tid & 31) == 0) red[tid >> 5] = q;
    __syncthreads();
    if (tid == 0) {
      double s = 0.0;
      for (int w = 0; w < QT / 32; ++w) s += red[w];
      hp[0] = house_par(S[0], s);
    }
    __syncthreads();
  }
  for (int k = 0; k < r; ++k) {
    const HousePar h = hp[k & 1];
    const int left = r - k - 1;
    if (left > 0) {
      const int gs = group_size(left);
      const int grp = tid / gs, ln = tid - grp * gs;
      if (grp < left) {
        const unsigned mask = group_mask(gs);
        double *Sj = S + (k + 1 + grp) * LD;
        const double *Sk = S + k * LD;
        if (h.tau != 0.0) {
          double dd = 0.0;
          for (int i = r + ln; i < r + na; i += gs) dd = fma(Sk[i], Sj[i], dd);
          dd = group_sum(dd, gs, mask);
          const double tw = h.tau * fma(h.scale, dd, Sj[k]), tws = tw * h.scale;
          for (int i = r + ln; i < r + na; i += gs) Sj[i] = fma(-tws, Sk[i], Sj[i]);
          if (ln == 0) Sj[k] -= tw;
        }
        if (grp == 0) {
          double q = 0.0;
          for (int i = r + ln; i < r + na; i += gs) q = fma(Sj[i], Sj[i], q);
          q = group_sum(q, gs, mask);
          // entry (k+1, k+1) is not written during step k
          if (ln == 0) hp[(k + 1) & 1] = house_par(Sj[k + 1], q);
        }
      }
    }
    __syncthreads();
    if (tid == 0) S[k * LD + k] = h.beta;  // nobody reads (k, k) after step k
  }
  __syncthreads();
}

// R factor of rows [t0, t1) of a tall matrix (ncol <= QR_MAXC), one CTA per
// job, tiles of qr_chunk(ncol) rows.
__global__ void __launch_bounds__(QT)
k_tall_qr(const TallDesc *__restrict__ descs, const QrJob *__restrict__ jobs) {
  extern __shared__ double S[];
  __shared__ HousePar hp[2];
  __shared__ double red[QT / 32];
  const QrJob jb = jobs[blockIdx.x];
  const TallDesc d = descs[jb.desc];
  const int r = d.ncol, nc = qr_chunk(r), LD = r + nc + 1;
  const int tid = threadIdx.x;
  for (int e = tid; e < LD * r; e += QT) S[e] = 0.0;
  __syncthreads();
  for (int t = jb.t0; t < jb.t1; t += nc) {
    const int na = min(nc, jb.t1 - t);
    if (d.sc == 1) {  // a tall row is contiguous: lanes along c
      for (int e = tid; e < na * r; e += QT) {
        const int tt = e / r, c = e - tt * r, v = t + tt;
        const long long ph = v < d.s0 ? v : (long long)v + d.skip;
        S[c * LD + r + tt] = d.base[ph * d.st + c];
      }
    } else {  // a tall column is contiguous: lanes along t
      for (int e = tid; e < na * r; e += QT) {
        const int c = e / na, tt = e - c * na, v = t + tt;
        const long long ph = v < d.s0 ? v : (long long)v + d.skip;
        S[c * LD + r + tt] = d.base[ph * d.st + (long long)c * d.sc];
      }
    }
    __syncthreads();
    house_tile(S, LD, r, na, hp, red);
  }
  for (int e = tid; e < r * r; e += QT) {
    const int c = e / r, i = e - c * r;
    jb.out[(long long)c * jb.ldo + i] = i <= c ? S[c * LD + i] : 0.0;
  }
}

// Basis of one node from its R factor: the left singular vectors of R^T with
// singular value > tol, in decreasing order (the left singular vectors of a
// block row whose transpose has R as QR factor, or the right singular vectors
// of a block column with R as QR factor).
//   A. Householder QR with column pivoting of R, R Pi = Q2 R2, in shared memory
//      (squared trailing column norms downdated, recomputed when they lose
//      three digits); it stops at the first step k0 where the trailing block's
//      Frobenius norm is below tol / 100, so R2's rows from k0 on are dropped:
//      they move the kept subspace by less than that.
//   B. One-sided Jacobi (Hestenes) on the k0 leading rows of R2 as vectors of
//      length r (R^T = Pi R2^T Q2^T, so the left singular vectors of R^T are Pi
//      times those of R2^T, i.e. of the rows): round-robin pairs, one group of
//      lanes per pair, squared norms cached (refreshed each sweep, a' = a - t c,
//      b' = b + t c), one lane forms each rotation, rows below tol / 100 left
//      out.  Pivoting makes the rows graded (Drmac & Veselic, "New fast and
//      accurate Jacobi SVD algorithm", SIAM J. Matrix Anal. Appl. 29, 2008),
//      so few sweeps are needed, on k0 ~ rank rows instead of r.
//   C. Normalised rows with norm > tol, un-permuted, sorted by decreasing norm.
// status |= 1 if the sweep limit is reached.
__global__ void __launch_bounds__(QT)
k_node_basis(const BasisJob *__restrict__ jobs, double tol, int *status) {
  extern __shared__ double M[];  // column j at M + j * LDM
  __shared__ double cn[QR_MAXC], cref[QR_MAXC], nrm[QR_MAXC];
  __shared__ int prm[QR_MAXC], pos[QR_MAXC];
  __shared__ HousePar s_h;
  __shared__ int s_piv, s_k;
  const BasisJob jb = jobs[blockIdx.x];
  const int r = jb.r, LDM = r + 1, tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  for (int e = tid; e < r * r; e += QT) {
    const int c = e / r, i = e - c * r;
    M[c * LDM + i] = i <= c ? jb.R[i + (long long)c * r] : 0.0;
  }
  __syncthreads();
  {
    const int gs = group_size(r), grp = tid / gs, ln = tid - grp * gs;
    const unsigned mask = group_mask(gs);
    for (int c = grp; c < r; c += QT / gs) {
      double a = 0.0;
      for (int i = ln; i <= c; i += gs) { const double u = M[c * LDM + i]; a = fma(u, u, a); }
      a = group_sum(a, gs, mask);
      if (ln == 0) { cn[c] = a; cref[c] = a; prm[c] = c; }
    }
  }
  __syncthreads();
  // ---- A: pivoted QR, stopped when the trailing block is negligible
  const double stop2 = tol > 0.0 ? 1e-4 * tol * tol : 0.0;
  int k0 = r;
  for (int k = 0; k < r; ++k) {
    if (wid == 0) {
      ArgMax am{-1.0, r};
      for (int j = k + lane; j < r; j += 32) am = argmax_merge(am, ArgMax{cn[j], j});
      am = warp_argmax(am);
      if (lane == 0) s_piv = ((double)(r - k) * am.v <= stop2) ? -1 : am.i;
    }
    __syncthreads();
    const int p = s_piv;
    if (p < 0) { k0 = k; break; }
    if (p != k) {
      for (int i = tid; i < r; i += QT) {
        const double t = M[k * LDM + i];
        M[k * LDM + i] = M[p * LDM + i];
        M[p * LDM + i] = t;
      }
      if (tid == 0) {
        double t = cn[k]; cn[k] = cn[p]; cn[p] = t;
        t = cref[k]; cref[k] = cref[p]; cref[p] = t;
        const int q = prm[k]; prm[k] = prm[p]; prm[p] = q;
      }
      __syncthreads();
    }
    if (wid == 0) {
      double q = 0.0;
      for (int i = k + 1 + lane; i < r; i += 32) { const double u = M[k * LDM + i]; q = fma(u, u, q); }
      q = warp_sum(q);
      if (lane == 0) s_h = house_par(M[k * LDM + k], q);
    }
    __syncthreads();
    const HousePar h = s_h;
    const int left = r - k - 1;
    if (left > 0) {
      const int gs = group_size(left), grp = tid / gs, ln = tid - grp * gs;
      if (grp < left) {
        const unsigned mask = group_mask(gs);
        const int j = k + 1 + grp;
        double *Mj = M + j * LDM;
        const double *Mk = M + k * LDM;
        double rk = Mj[k];
        if (h.tau != 0.0) {
          double dd = 0.0;
          for (int i = k + 1 + ln; i < r; i += gs) dd = fma(Mk[i], Mj[i], dd);
          dd = group_sum(dd, gs, mask);
          const double tw = h.tau * fma(h.scale, dd, rk), tws = tw * h.scale;
          for (int i = k + 1 + ln; i < r; i += gs) Mj[i] = fma(-tws, Mk[i], Mj[i]);
          rk -= tw;
        }
        // trailing norm of column j without row k
        double c2 = fma(-rk, rk, cn[j]);
        double cr = cref[j];
        if (c2 < 1e-3 * cr) {  // cancellation: recompute
          double a = 0.0;
          for (int i = k + 1 + ln; i < r; i += gs) { const double u = Mj[i]; a = fma(u, u, a); }
          c2 = group_sum(a, gs, mask);
          cr = c2;
        }
        __syncwarp(mask);
        if (ln == 0) { Mj[k] = rk; cn[j] = c2; cref[j] = cr; }
      }
    }
    if (tid == 0) M[k * LDM + k] = h.beta;
    __syncthreads();
  }
  // rows 0..k0-1 of R2 (upper trapezoidal): clear the reflectors stored below
  // the diagonal inside them
  for (int e = tid; e < k0 * k0; e += QT) {
    const int j = e / k0, i = e - j * k0;
    if (i > j) M[j * LDM + i] = 0.0;
  }
  __syncthreads();
  // ---- B: one-sided Jacobi on the k0 rows
  const int rp = k0 + (k0 & 1), np = rp / 2;
  const int gs = group_size(np > 0 ? np : 1);
  const int grp = tid / gs, ln = tid - grp * gs;
  const unsigned mask = group_mask(gs);
  const int ng = QT / gs;
  const int lead = (tid & 31) & ~(gs - 1);
  const double jtol = HSS_EPS * (r > 16 ? r : 16);
  const double frz2 = stop2;
  int conv = k0 < 2;
  for (int sweep = 0; sweep < JAC_SWEEPS && !conv; ++sweep) {
    for (int t = grp; t < k0; t += ng) {
      double a = 0.0;
      for (int j = ln; j < r; j += gs) { const double u = M[j * LDM + t]; a = fma(u, u, a); }
      a = group_sum(a, gs, mask);
      if (ln == 0) nrm[t] = a;
    }
    __syncthreads();
    int rot = 0;
    for (int s = 0; s < rp - 1; ++s) {
      if (grp < np) {
        int p, q;
        if (grp == 0) { p = 0; q = 1 + s % (rp - 1); }
        else { p = 1 + (s + grp) % (rp - 1); q = 1 + (s - grp + rp - 1) % (rp - 1); }
        if (p < k0 && q < k0) {
          const double a = nrm[p], b = nrm[q];
          if (a > 0.0 && b > 0.0 && a >= frz2 && b >= frz2) {
            double c = 0.0;
            for (int j = ln; j < r; j += gs) c = fma(M[j * LDM + p], M[j * LDM + q], c);
            c = group_sum(c, gs, mask);
            double cs = 1.0, sn = 0.0;
            int go = 0;
            if (ln == 0 && c != 0.0 && fabs(c) > jtol * sqrt(a * b)) {
              const double zeta = (b - a) / (2.0 * c);
              const double t = fabs(zeta) > 1e150
                                   ? 0.5 / zeta
                                   : copysign(1.0, zeta) / (fabs(zeta) + sqrt(fma(zeta, zeta, 1.0)));
              cs = 1.0 / sqrt(fma(t, t, 1.0));
              sn = cs * t;
              nrm[p] = fma(-t, c, a);
              nrm[q] = fma(t, c, b);
              go = 1;
            }
            go = __shfl_sync(mask, go, lead);
            if (go) {
              cs = __shfl_sync(mask, cs, lead);
              sn = __shfl_sync(mask, sn, lead);
              for (int j = ln; j < r; j += gs) {
                const double u = M[j * LDM + p], v = M[j * LDM + q];
                M[j * LDM + p] = fma(cs, u, -sn * v);
                M[j * LDM + q] = fma(sn, u, cs * v);
              }
              rot = 1;
            }
          }
        }
      }
      __syncthreads();
    }
    conv = !__syncthreads_or(rot);
  }
  if (!conv && tid == 0) atomicOr(status, 1);
  __syncthreads();
  // ---- C: norms, order, rank, outputs
  for (int t = grp; t < k0; t += ng) {
    double a = 0.0;
    for (int j = ln; j < r; j += gs) { const double u = M[j * LDM + t]; a = fma(u, u, a); }
    a = group_sum(a, gs, mask);
    if (ln == 0) nrm[t] = sqrt(a);
  }
  __syncthreads();
  for (int t = tid; t < k0; t += QT) {
    const double v = nrm[t];
    int p = 0;
    for (int t2 = 0; t2 < k0; ++t2) {
      const double w = nrm[t2];
      p += (w > v) || (w == v && t2 < t);
    }
    pos[t] = p;
  }
  if (tid == 0) {
    int k = 0;
    for (int t = 0; t < k0; ++t) k += nrm[t] > tol;
    s_k = k;
    *jb.rank = k;
  }
  __syncthreads();
  const int k = s_k;
  for (int e = tid; e < k0 * r; e += QT) {
    const int t = e / r, j = e - t * r;
    const int pt = pos[t];
    if (pt < k) {
      const double val = M[j * LDM + t] / nrm[t];
      const int row = prm[j];
      jb.P[row + (long long)pt * r] = val;
      jb.PT[pt + (long long)row * k] = val;
    }
  }
}

__global__ void k_copy_blocks(const CopyDesc *__restrict__ ds, int nd) {
  for (int q = blockIdx.y; q < nd; q += gridDim.y) {
    const CopyDesc c = ds[q];
    const long long tot = (long long)c.rows * c.cols;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < tot;
         e += (long long)gridDim.x * blockDim.x) {
      const long long j = e / c.rows, i = e - j * c.rows;
      c.dst[i + j * c.ldd] = c.src[i + j * c.lds];
    }
  }
}

template <class T>
static T *upload(const char *name, const std::vector<T> &v, cudaStream_t st) {
  T *d = pool<T>(name, std::max<size_t>(v.size(), 1));
  if (!v.empty()) stage_h2d(d, v.data(), v.size() * sizeof(T), st);
  return d;
}

static int copy_blocks(const std::vector<CopyDesc> &cds, cudaStream_t st) {
  std::vector<CopyDesc> v;
  long long mx = 0;
  for (const auto &c : cds)
    if (c.rows > 0 && c.cols > 0) { v.push_back(c); mx = std::max(mx, (long long)c.rows * c.cols); }
  if (v.empty()) return 0;
  CopyDesc *d = upload("m2h_copy", v, st);
  dim3 g((unsigned)std::min<long long>((mx + 255) / 256, 1024), (unsigned)std::min<size_t>(v.size(), 65535));
  k_copy_blocks<<<g, 256, 0, st>>>(d, (int)v.size());
  return 1;
}

static int sm_count() {
  static int n = 0;
  if (n == 0) {
    int dev = 0;
    MCK(cudaGetDevice(&dev));
    MCK(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev));
    if (n <= 0) n = 1;
  }
  return n;
}

// Bases of a set of tall matrices: R = qr(desc), then the normalised Jacobi
// columns of R^T with norm > tol into P[i] (ncol x k, ld ncol) and PT[i]
// (k x ncol, ld k).  Returns the ranks (one host synchronisation).
static std::vector<int> tall_bases(const std::vector<TallDesc> &ds, const std::vector<double *> &P,
                                   const std::vector<double *> &PT, double tol, int &launches,
                                   cudaStream_t st) {
  const int nd = (int)ds.size();
  std::vector<int> rk(nd, 0);
  if (nd == 0) return rk;
  static bool attr = false;
  if (!attr) {
    MCK(cudaFuncSetAttribute(k_tall_qr, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             QR_TILE * (int)sizeof(double)));
    MCK(cudaFuncSetAttribute(k_node_basis, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             QR_MAXC * (QR_MAXC + 1) * (int)sizeof(double)));
    attr = true;
  }
  // rows per first-pass job: enough jobs for two CTAs per SM, and at least
  // four times the column count
  long long tot = 0;
  for (const auto &d : ds) tot += d.ntot;
  const long long per0 = std::max<long long>(1, tot / (2LL * sm_count()));
  double *Rfin = pool<double>("m2h_Rfin", (size_t)nd * QR_MAXC * QR_MAXC);
  std::vector<QrJob> j1, j2;
  std::vector<TallDesc> d2;
  std::vector<long long> soff(nd, -1);
  std::vector<int> njob(nd, 0);
  long long stot = 0;
  for (int i = 0; i < nd; ++i) {
    const int r = ds[i].ncol;
    const long long per = std::max<long long>(per0, 4LL * r);
    njob[i] = (int)std::min<long long>(64, (ds[i].ntot + per - 1) / per);
    if (njob[i] > 1) { soff[i] = stot; stot += (long long)njob[i] * r * r; }
  }
  double *stk = pool<double>("m2h_Rstack", (size_t)std::max<long long>(stot, 1));
  for (int i = 0; i < nd; ++i) {
    const int r = ds[i].ncol, nj = njob[i];
    double *fin = Rfin + (size_t)i * QR_MAXC * QR_MAXC;
    if (nj == 1) {
      j1.push_back({i, 0, ds[i].ntot, fin, r});
      continue;
    }
    double *sb = stk + soff[i];
    const int ld = nj * r;
    for (int q = 0; q < nj; ++q) {
      const int a = (int)((long long)ds[i].ntot * q / nj), b = (int)((long long)ds[i].ntot * (q + 1) / nj);
      j1.push_back({i, a, b, sb + (size_t)q * r, ld});
    }
    d2.push_back({sb, 1, (long long)ld, ld, r, INT_MAX, 0});
    j2.push_back({(int)d2.size() - 1, 0, ld, fin, r});
  }
  TallDesc *dd = upload("m2h_desc", ds, st);
  QrJob *dj = upload("m2h_job1", j1, st);
  k_tall_qr<<<(unsigned)j1.size(), QT, QR_TILE * sizeof(double), st>>>(dd, dj);
  ++launches;
  if (!j2.empty()) {
    TallDesc *dd2 = upload("m2h_desc2", d2, st);
    QrJob *dj2 = upload("m2h_job2", j2, st);
    k_tall_qr<<<(unsigned)j2.size(), QT, QR_TILE * sizeof(double), st>>>(dd2, dj2);
    ++launches;
  }
  int *drk = pool<int>("m2h_rank", nd + 1);
  MCK(cudaMemsetAsync(drk, 0, sizeof(int) * (nd + 1), st));
  std::vector<BasisJob> bj(nd);
  int rmax = 1;
  for (int i = 0; i < nd; ++i) {
    bj[i] = {Rfin + (size_t)i * QR_MAXC * QR_MAXC, ds[i].ncol, P[i], PT[i], drk + i};
    rmax = std::max(rmax, ds[i].ncol);
  }
  BasisJob *db = upload("m2h_bjob", bj, st);
  k_node_basis<<<nd, QT, (size_t)rmax * (rmax + 1) * sizeof(double), st>>>(db, tol, drk + nd);
  ++launches;
  std::vector<int> h(nd + 1);
  MCK(cudaMemcpyAsync(h.data(), drk, sizeof(int) * (nd + 1), cudaMemcpyDeviceToHost, st));
  MCK(cudaStreamSynchronize(st));
  if (h[nd]) throw HssError{"mat2hss: one-sided Jacobi SVD did not converge"};
  for (int i = 0; i < nd; ++i) rk[i] = h[i];
  return rk;
}

// Right singular vectors with singular value above tol of column-major tall
// matrices X[i] (rows[i] x ncol[i], leading dimension ld[i], ncol <= 128), in
// decreasing order, into P[i] (ncol x k, ld ncol) and PT[i] (k x ncol, ld k);
// returns the ranks k (one host synchronisation).
std::vector<int> tall_right_bases(const std::vector<const double *> &X,
                                  const std::vector<int> &rows, const std::vector<int> &ncol,
                                  const std::vector<long long> &ld, const std::vector<double *> &P,
                                  const std::vector<double *> &PT, double tol, cudaStream_t st) {
  std::vector<TallDesc> ds;
  for (size_t i = 0; i < X.size(); ++i) {
    if (ncol[i] > QR_MAXC) throw HssError{"tall_right_bases: more than 128 columns"};
    ds.push_back(TallDesc{X[i], 1, ld[i], rows[i], ncol[i], INT_MAX, 0});
  }
  int launches = 0;
  return tall_bases(ds, P, PT, tol, launches, st);
}

struct Front {
  int node, ra, rb, ca, cb;
};

// Generators of the HSS approximation of the n x n matrix A (leading dim lda)
// in pl, for hss_multiply (Y = X A).  pl.ok = false when a node dimension
// exceeds QR_MAXC; the caller then multiplies by A itself.
int mat2hss_construct(HssPlan &pl, const double *A, long long lda, int n, int ni, double tol,
                      int precision, cudaStream_t st) {
  int launches = 0;
  pl.t = make_tree(n, ni);
  const HostTree &t = pl.t;
  const int ltr = t.ltr;
  HssDev &h = pl.h;
  std::memset(&h, 0, sizeof h);
  pl.Ur.assign(ltr + 1, 0); pl.Uc.assign(ltr + 1, 0); pl.Vr.assign(ltr + 1, 0);
  pl.Vc.assign(ltr + 1, 0); pl.Br.assign(ltr + 1, 0); pl.Bc.assign(ltr + 1, 0);
  pl.Dm.assign(ltr + 1, 0);
  pl.doff.clear();
  pl.max_rank = 0;
  pl.ok = true;
  if (t.mmax > QR_MAXC) { pl.ok = false; return 0; }
  // leaf diagonal blocks D_i = A(I_i, I_i)
  std::vector<CopyDesc> cd;
  long long dtot = 0;
  for (int i = 1, li = 0; i <= ltr; ++i)
    if (t.leaf(i)) { pl.doff.push_back(dtot); dtot += (long long)t.m[li] * t.m[li]; ++li; }
  h.Dg = pool<double>("m2h_Dg", (size_t)dtot);
  for (int i = 1, li = 0; i <= ltr; ++i)
    if (t.leaf(i)) {
      const int m = t.m[li], a = t.leafstart[i];
      pl.Dm[i] = m;
      cd.push_back({A + a + (long long)a * lda, lda, h.Dg + pl.doff[li], m, m, m});
      ++li;
    }
  launches += copy_blocks(cd, st);
  if (t.lm == 1) return launches;
  h.ucap = h.vcap = h.bcap = (long long)QR_MAXC * QR_MAXC;
  h.Ug = pool<double>("m2h_Ug", (size_t)(ltr + 1) * h.ucap);
  h.Vg = pool<double>("m2h_Vg", (size_t)(ltr + 1) * h.vcap);
  h.Bg = pool<double>("m2h_Bg", (size_t)(ltr + 1) * h.bcap);
  double *Ws = pool<double>("m2h_W", (size_t)(ltr + 1) * QR_MAXC * QR_MAXC);  // U^T / V operands
  double *A1 = pool<double>("m2h_A1", (size_t)n * n), *A2 = pool<double>("m2h_A2", (size_t)n * n);
  auto Ug = [&](int nd) { return h.Ug + (size_t)nd * h.ucap; };
  auto Vg = [&](int nd) { return h.Vg + (size_t)nd * h.vcap; };
  auto Bg = [&](int nd) { return h.Bg + (size_t)nd * h.bcap; };
  auto Wn = [&](int nd) { return Ws + (size_t)nd * QR_MAXC * QR_MAXC; };
  std::vector<Front> fr;
  for (int i = 1; i <= ltr; ++i)
    if (t.leaf(i)) {
      const int a = t.leafstart[i], b = a + pl.Dm[i];
      fr.push_back({i, a, b, a, b});
    }
  const double *Ah = A;
  long long ldh = lda;
  int Rc = n;
  for (int LL = t.lvl; LL >= 1; --LL) {
    const int nf = (int)fr.size();
    std::vector<char> act(nf);
    for (int x = 0; x < nf; ++x) act[x] = t.depth[fr[x].node] == LL;
    for (int x = 0; x < nf; ++x)
      if (act[x] && (fr[x].rb - fr[x].ra > QR_MAXC || fr[x].cb - fr[x].ca > QR_MAXC)) {
        pl.ok = false;
        return launches;
      }
    // ---- row phase: U_i from the block rows Ah(I_i, ~J_i)
    std::vector<TallDesc> ds;
    std::vector<double *> P, PT;
    std::vector<int> who;
    for (int x = 0; x < nf; ++x) {
      if (!act[x]) continue;
      const Front &f = fr[x];
      const int r = f.rb - f.ra, ntot = Rc - (f.cb - f.ca);
      if (r == 0 || ntot == 0) continue;
      ds.push_back({Ah + f.ra, ldh, 1, ntot, r, f.ca, f.cb - f.ca});
      P.push_back(Ug(f.node));
      PT.push_back(Wn(f.node));
      who.push_back(x);
    }
    std::vector<int> rk = tall_bases(ds, P, PT, tol, launches, st);
    std::vector<int> kr(nf, 0);
    for (size_t q = 0; q < who.size(); ++q) kr[who[q]] = rk[q];
    int Rr1 = 0;
    std::vector<int> ra1(nf);
    for (int x = 0; x < nf; ++x) {
      const Front &f = fr[x];
      ra1[x] = Rr1;
      if (act[x]) {
        pl.Ur[f.node] = f.rb - f.ra;
        pl.Uc[f.node] = kr[x];
        pl.max_rank = std::max(pl.max_rank, kr[x]);
        Rr1 += kr[x];
      } else {
        Rr1 += f.rb - f.ra;
      }
    }
    std::vector<GemmDesc> gm;
    cd.clear();
    for (int x = 0; x < nf; ++x) {
      const Front &f = fr[x];
      if (act[x]) {
        if (kr[x] > 0)
          gm.push_back({Wn(f.node), Ah + f.ra, A1 + ra1[x], kr[x], (int)ldh, Rr1, kr[x], Rc,
                        f.rb - f.ra, 0, 0});
      } else {
        cd.push_back({Ah + f.ra, ldh, A1 + ra1[x], Rr1, f.rb - f.ra, Rc});
      }
    }
    if (Rr1 > 0) {
      launch_gemm(gm, precision, st);
      launches += gm.empty() ? 0 : 1;
      launches += copy_blocks(cd, st);
    }
    // ---- column phase: V_j from the block columns A1(~I_j, J_j)
    ds.clear(); P.clear(); PT.clear(); who.clear();
    for (int x = 0; x < nf; ++x) {
      if (!act[x]) continue;
      const Front &f = fr[x];
      const int c = f.cb - f.ca, ntot = Rr1 - kr[x];
      if (c == 0 || ntot == 0) continue;
      ds.push_back({A1 + (long long)f.ca * Rr1, 1, (long long)Rr1, ntot, c, ra1[x], kr[x]});
      P.push_back(Wn(f.node));
      PT.push_back(Vg(f.node));
      who.push_back(x);
    }
    rk = tall_bases(ds, P, PT, tol, launches, st);
    std::vector<int> kc(nf, 0);
    for (size_t q = 0; q < who.size(); ++q) kc[who[q]] = rk[q];
    int Rc1 = 0;
    std::vector<int> ca1(nf);
    for (int x = 0; x < nf; ++x) {
      const Front &f = fr[x];
      ca1[x] = Rc1;
      if (act[x]) {
        pl.Vr[f.node] = kc[x];
        pl.Vc[f.node] = f.cb - f.ca;
        pl.max_rank = std::max(pl.max_rank, kc[x]);
        Rc1 += kc[x];
      } else {
        Rc1 += f.cb - f.ca;
      }
    }
    gm.clear();
    cd.clear();
    for (int x = 0; x < nf; ++x) {
      const Front &f = fr[x];
      if (act[x]) {
        if (kc[x] > 0 && Rr1 > 0)
          gm.push_back({A1 + (long long)f.ca * Rr1, Wn(f.node), A2 + (long long)ca1[x] * Rr1, Rr1,
                        f.cb - f.ca, Rr1, Rr1, kc[x], f.cb - f.ca, 0, 0});
      } else {
        cd.push_back({A1 + (long long)f.ca * Rr1, Rr1, A2 + (long long)ca1[x] * Rr1, Rr1, Rr1,
                      f.cb - f.ca});
      }
    }
    launch_gemm(gm, precision, st);
    launches += gm.empty() ? 0 : 1;
    launches += copy_blocks(cd, st);
    // ---- new ranges, B generators between siblings of this depth
    for (int x = 0; x < nf; ++x) {
      Front &f = fr[x];
      const int r = act[x] ? kr[x] : f.rb - f.ra, c = act[x] ? kc[x] : f.cb - f.ca;
      f.ra = ra1[x]; f.rb = ra1[x] + r; f.ca = ca1[x]; f.cb = ca1[x] + c;
    }
    cd.clear();
    for (int x = 0; x < nf; ++x) {
      if (!act[x]) continue;
      const int sb = t.sibling(fr[x].node);
      int y = -1;
      for (int z = 0; z < nf; ++z)
        if (fr[z].node == sb) y = z;
      if (y < 0) throw HssError{"mat2hss: sibling missing from the frontier"};
      const int kb = fr[x].rb - fr[x].ra, kcb = fr[y].cb - fr[y].ca;
      pl.Br[fr[x].node] = kb;
      pl.Bc[fr[x].node] = kcb;
      cd.push_back({A2 + fr[x].ra + (long long)fr[y].ca * Rr1, Rr1, Bg(fr[x].node),
                    std::max(kb, 1), kb, kcb});
    }
    launches += copy_blocks(cd, st);
    // ---- siblings of this depth become their parent
    std::vector<Front> nx;
    for (int x = 0; x < nf; ++x) {
      if (act[x] && x + 1 < nf && act[x + 1] && t.parent[fr[x].node] == t.parent[fr[x + 1].node]) {
        nx.push_back({t.parent[fr[x].node], fr[x].ra, fr[x + 1].rb, fr[x].ca, fr[x + 1].cb});
        ++x;
      } else {
        nx.push_back(fr[x]);
      }
    }
    fr.swap(nx);
    Ah = A2;
    ldh = Rr1;
    Rc = Rc1;
  }
  return launches;
}

// DHSSMM / DHSSMML on device arrays.  side 0: B (n x k, ldb) <- A_hss B, as
// (B^T A_hss^T)^T with the HSS form of A^T; side 1: B (k x n, ldb) <- B A_hss.
// times[0] / times[1]: construction / multiplication (ms).
int hss_dhssmm_core(int n, const double *A, long long lda, double *B, long long ldb, int k,
                    double tol, int ni, int side, int precision, int *rank, float *times,
                    cudaStream_t st) {
  int launches = 0;
  cudaEvent_t e0, e1, e2;
  MCK(cudaEventCreate(&e0)); MCK(cudaEventCreate(&e1)); MCK(cudaEventCreate(&e2));
  MCK(cudaEventRecord(e0, st));
  const double *M = A;
  long long ldm = lda;
  if (side == 0) {
    double *At = pool<double>("m2h_At", (size_t)n * n);
    transpose(n, n, A, lda, At, n, st);
    ++launches;
    M = At;
    ldm = n;
  }
  HssPlan pl;
  launches += mat2hss_construct(pl, M, ldm, n, ni, tol, precision, st);
  MCK(cudaEventRecord(e1, st));
  double *X = pool<double>("m2h_X", (size_t)k * n), *Y = pool<double>("m2h_Y", (size_t)k * n);
  const double *Xs;
  long long ldx;
  if (side == 0) {
    transpose(n, k, B, ldb, X, k, st);
    ++launches;
    Xs = X;
    ldx = k;
  } else {
    Xs = B;
    ldx = ldb;
  }
  if (pl.ok) {
    launches += hss_multiply(pl, Xs, ldx, k, Y, k, precision, st);
    *rank = pl.max_rank;
  } else {
    std::vector<GemmDesc> g{{Xs, M, Y, (int)ldx, (int)ldm, k, k, n, n, 0, 0}};
    launch_gemm(g, precision, st);
    ++launches;
    *rank = n;
  }
  if (side == 0) {
    transpose(k, n, Y, k, B, ldb, st);
  } else {
    MCK(cudaMemcpy2DAsync(B, ldb * sizeof(double), Y, k * sizeof(double), k * sizeof(double), n,
                          cudaMemcpyDeviceToDevice, st));
  }
  ++launches;
  MCK(cudaEventRecord(e2, st));
  MCK(cudaEventSynchronize(e2));
  if (times) {
    MCK(cudaEventElapsedTime(&times[0], e0, e1));
    MCK(cudaEventElapsedTime(&times[1], e1, e2));
  }
  cudaEventDestroy(e0); cudaEventDestroy(e1); cudaEventDestroy(e2);
  return launches;
}

}  // namespace hss
