// bsvd.cu -- SVD of an upper banded matrix by structured banded divide and
// conquer (MDBDSVD, SRC/mdbdsvd.f90:1; S.-G. Li's SBDC).
//
// The n x n upper banded matrix B (semibandwidth sb, LAPACK upper band storage:
// B(i, j) = AB(sb + i - j, j), 0 <= j - i <= sb, 0-based) is cut by the tree of
// MDBDSVDT (SRC/mdbdsvdt.f90): a node of rows [s, s + N) keeps nl rows on the
// left, sb center rows c = s + nl .. s + nl + sb - 1, and nr = N - nl - sb rows
// on the right.  Its left child holds rows [s, s + nl) and columns
// [s, s + nl + sb) (nl x (nl + sb)); its right child rows and columns from
// s + nl + sb, with sb extra columns unless it ends the matrix.  Leaves are
// dense SVDs (DGESVD at mdbdsvd.f90:168, :214).
//
// Storage is the bidiagonal SVD's (svd.cu): slot p holds U(:, p), V(:, p) and
// sigma_p = Dp[p]; a node's triples sit in the slots of its rows and its null
// vectors in V slots past them, i.e. the left child's null vectors are V slots
// c .. c + sb - 1, the center rows' slots.
//
// A merge (MDBDSVD1, SRC/mdbdsvd1.f90) appends the sb center rows one at a
// time.  Before the append of row c_k = s + nl + k, with coefficients
// z = V^T b (b = row c_k of B), the null vectors of the node (V slots
// c_k .. s + nl + sb - 1 and the right child's extra columns) are folded by one
// Householder reflection so that z vanishes on all but slot c_k (the role of
// MDBDSVD2's QR of the inserted rows and DTZRZF of the extra columns,
// mdbdsvd2.f90:269-275, :546-571).  Row c_k then forms, with the node's current
// singular values, the broken arrow [z_pole z^T; 0 diag(sigma)] whose pole
// d = 0 has left vector e_{c_k}: exactly the merge of the bidiagonal divide and
// conquer, which the deflation below (MDBDSVD2 / MDBDSVD22's tests) and the
// bidiagonal kernels (secular equation, Loewner z, vector blocks, products or
// HSS, ascending order) then run.
#include "hss_block.cuh"
#include "hss_common.cuh"
#include "hss_kernels.h"
#include "hss_svdprep.cuh"

namespace hss {

constexpr int BSVD_ROWS_MAX = 64;   // leaf rows (one CTA's shared-memory Jacobi)
constexpr int BSVD_COLS_MAX = 96;   // leaf columns (rows + sb)
constexpr int BSVD_SWEEPS = 40;

// Sum over the warp, valid in lane 0 only (the rotation's scalars are formed
// there): a halving tree, each step's adds on the lanes that need them.
__device__ __forceinline__ double warp_sum0(double v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double t = __shfl_down_sync(HSS_FULL, v, o);
    if (lane < o) v += t;
  }
  return v;
}

__device__ __forceinline__ double bsvd_at(const double *__restrict__ AB, long long ldab, int sb,
                                          int i, int j) {
  const int d = j - i;
  return (d < 0 || d > sb) ? 0.0 : AB[(long long)j * ldab + (sb - d)];
}

// ------------------------------------------------------------- leaves -----
// One CTA per leaf: the r x c block B(a + i, a + q) by one-sided Jacobi on its
// columns (Hestenes 1958): B J has mutually orthogonal columns, so with
// sigma_q = |(B J)_q| the r largest give U_q = (B J)_q / sigma_q and V = J is
// the full c x c orthogonal factor, its last c - r columns the null vectors.
// Pairs follow the round-robin tournament ordering (c/2 disjoint rotations
// per round, one warp each).  U is reorthogonalised (classical Gram-Schmidt
// twice, descending sigma), and completed from unit vectors where a column
// vanished (rank-deficient blocks).  Results ascending in slots a .. a + r - 1
// (U, V, Dp, perm), null vectors in V slots a + r .. a + c - 1.
__global__ void __launch_bounds__(256)
k_bsvd_leaf(int nleaf, const int *__restrict__ la, const int *__restrict__ lr,
            const int *__restrict__ lc, int sb, const double *__restrict__ AB, long long ldab,
            double *__restrict__ U, long long ldu, double *__restrict__ V, long long ldv,
            double *__restrict__ Dp, int *__restrict__ perm, int *__restrict__ status) {
  extern __shared__ double sm[];
  double *Bs = sm;                                     // column q at Bs + q * RP
  double *Vs = Bs + BSVD_COLS_MAX * BSVD_ROWS_MAX;     // column q at Vs + q * CP
  double *Us = Vs + BSVD_COLS_MAX * BSVD_COLS_MAX;     // column t (by rank) at Us + t * RP
  double *sg = Us + BSVD_ROWS_MAX * BSVD_ROWS_MAX;     // sigma per column
  double *cf = sg + BSVD_COLS_MAX;                     // projection coefficients
  __shared__ int rank_of[BSVD_COLS_MAX], col_of[BSVD_COLS_MAX];
  __shared__ int s_rot, s_ok;
  constexpr int RP = BSVD_ROWS_MAX, CP = BSVD_COLS_MAX;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = blockDim.x >> 5;
  const int L = blockIdx.x;
  if (L >= nleaf) return;
  const int a = la[L], r = lr[L], c = lc[L];
  for (int t = tid; t < c * r; t += blockDim.x) {
    const int q = t / r, i = t % r;
    Bs[q * RP + i] = bsvd_at(AB, ldab, sb, a + i, a + q);
  }
  for (int t = tid; t < c * c; t += blockDim.x) {
    const int q = t / c, i = t % c;
    Vs[q * CP + i] = (i == q) ? 1.0 : 0.0;
  }
  __shared__ double s_red[8];
  {  // |B|_F^2 of the block
    double p2 = 0.0;
    for (int t = tid; t < c * r; t += blockDim.x) {
      const double x = Bs[(t / r) * RP + t % r];
      p2 += x * x;
    }
    p2 = warp_sum(p2);
    if (lane == 0) s_red[wid] = p2;
  }
  __syncthreads();
  double nb2 = 0.0;
  for (int i = 0; i < nw; ++i) nb2 += s_red[i];
  const int cc = c + (c & 1);  // tournament over an even count (index c = bye)
  const double tolr = 4.0 * c * HSS_EPS;
  // columns below 4 c eps |B|_F are rounding residue (a wide block has c - r
  // of them); their mutual angles are noise, so they are never rotated
  const double tolr2 = tolr * tolr, small2 = tolr2 * nb2;
  bool conv = c < 2;
  for (int sweep = 0; sweep < BSVD_SWEEPS && !conv; ++sweep) {
    if (tid == 0) s_rot = 0;
    __syncthreads();
    for (int round = 0; round < cc - 1; ++round) {
      for (int pi = wid; pi < cc / 2; pi += nw) {
        const int i0 = pi, i1 = cc - 1 - pi;
        const int p = i0 == 0 ? 0 : ((i0 - 1 + round) % (cc - 1)) + 1;
        const int q = ((i1 - 1 + round) % (cc - 1)) + 1;
        if (p >= c || q >= c) continue;
        double al = 0.0, be = 0.0, ga = 0.0;
        for (int i = lane; i < r; i += 32) {
          const double x = Bs[p * RP + i], y = Bs[q * RP + i];
          al += x * x; be += y * y; ga += x * y;
        }
        al = warp_sum0(al); be = warp_sum0(be); ga = warp_sum0(ga);
        // the test and the rotation on lane 0 only, cs and sn broadcast
        double cs = 1.0, sn = 0.0;
        int go = 0;
        if (lane == 0 && al > small2 && be > small2 && ga * ga > tolr2 * (al * be)) {
          // the angle in FP32 (any t gives an exactly orthogonal rotation once
          // cs and sn are formed in FP64; an angle good to 1e-7 still removes
          // all but 1e-7 of ga).  With both norms above small2 and ga above the
          // test, |ze| < 1 / (2 tolr^2) fits FP32; beyond 1e18 (where ze^2
          // would overflow) t = 1 / (2 |ze|).
          const float zf = (float)qdiv(be - al, 2.0 * ga), az = fabsf(zf);
          const float w1 = fmaf(zf, zf, 1.f);
          const float tf = az > 1e18f ? __fdividef(0.5f, az) : __fdividef(1.f, az + w1 * rsqrtf(w1));
          const double t = (double)copysignf(tf, zf);
          // cs = 1 / sqrt(1 + t^2), 1 + t^2 in [1, 2]: FP32 estimate (rel.
          // 1e-7) and two Newton steps y (3/2 - x y^2 / 2) in FP64
          const double hx = 0.5 * fma(t, t, 1.0);
          cs = (double)rsqrtf((float)(2.0 * hx));
          cs *= fma(-hx, cs * cs, 1.5);
          cs *= fma(-hx, cs * cs, 1.5);
          sn = cs * t;
          go = 1;
        }
        if (!__shfl_sync(HSS_FULL, go, 0)) continue;
        cs = __shfl_sync(HSS_FULL, cs, 0);
        sn = __shfl_sync(HSS_FULL, sn, 0);
        for (int i = lane; i < r; i += 32) {
          const double x = Bs[p * RP + i], y = Bs[q * RP + i];
          Bs[p * RP + i] = cs * x - sn * y;
          Bs[q * RP + i] = sn * x + cs * y;
        }
        for (int i = lane; i < c; i += 32) {
          const double x = Vs[p * CP + i], y = Vs[q * CP + i];
          Vs[p * CP + i] = cs * x - sn * y;
          Vs[q * CP + i] = sn * x + cs * y;
        }
        if (lane == 0) s_rot = 1;
      }
      __syncthreads();
    }
    conv = s_rot == 0;
    __syncthreads();
  }
  if (!conv && tid == 0) atomicMax(status, HSS_LEAF_NOCONV);
  // column norms, ranks by descending norm (ties by index)
  for (int q = wid; q < c; q += nw) {
    double s2 = 0.0;
    for (int i = lane; i < r; i += 32) s2 += Bs[q * RP + i] * Bs[q * RP + i];
    s2 = warp_sum(s2);
    if (lane == 0) sg[q] = sqrt(s2);
  }
  __syncthreads();
  for (int q = tid; q < c; q += blockDim.x) {
    int rk = 0;
    const double v = sg[q];
    for (int q2 = 0; q2 < c; ++q2) rk += (sg[q2] > v) || (sg[q2] == v && q2 < q);
    rank_of[q] = rk;
    col_of[rk] = q;
  }
  __syncthreads();
  // U columns by rank (the r largest), then Gram-Schmidt twice in rank order
  for (int t = tid; t < r * r; t += blockDim.x) {
    const int k = t / r, i = t % r;
    const int q = col_of[k];
    Us[k * RP + i] = sg[q] > 0.0 ? Bs[q * RP + i] / sg[q] : 0.0;
  }
  __syncthreads();
  for (int k = 0; k < r; ++k) {
    for (int cand = -1; cand < r; ++cand) {
      if (cand >= 0) {  // completion: start from e_cand
        for (int i = tid; i < r; i += blockDim.x) Us[k * RP + i] = (i == cand) ? 1.0 : 0.0;
        __syncthreads();
      }
      for (int pass = 0; pass < 2; ++pass) {
        for (int k2 = wid; k2 < k; k2 += nw) {
          double dt = 0.0;
          for (int i = lane; i < r; i += 32) dt += Us[k2 * RP + i] * Us[k * RP + i];
          dt = warp_sum(dt);
          if (lane == 0) cf[k2] = dt;
        }
        __syncthreads();
        for (int i = tid; i < r; i += blockDim.x) {
          double x = Us[k * RP + i];
          for (int k2 = 0; k2 < k; ++k2) x -= cf[k2] * Us[k2 * RP + i];
          Us[k * RP + i] = x;
        }
        __syncthreads();
      }
      if (wid == 0) {
        double s2 = 0.0;
        for (int i = lane; i < r; i += 32) s2 += Us[k * RP + i] * Us[k * RP + i];
        s2 = warp_sum(s2);
        // the column itself must keep half its length; a completion e_cand
        // some of it (with k < r vectors fixed, some e_cand keeps >= 1/r of
        // its squared length, so 1/(2r) always admits one)
        const double need = cand < 0 ? 0.25 : 0.5 / r;
        if (lane == 0) { s_ok = s2 > need; cf[RP] = s2 > 0.0 ? 1.0 / sqrt(s2) : 0.0; }
      }
      __syncthreads();
      if (s_ok) {
        const double inv = cf[RP];
        for (int i = tid; i < r; i += blockDim.x) Us[k * RP + i] *= inv;
        __syncthreads();
        break;
      }
      __syncthreads();
    }
  }
  // ascending slots: rank k < r goes to slot a + r - 1 - k; null vectors (rank
  // >= r) to V slots a + rank
  for (int t = tid; t < r * r; t += blockDim.x) {
    const int k = t / r, i = t % r;
    U[(long long)(a + r - 1 - k) * ldu + a + i] = Us[k * RP + i];
  }
  for (int t = tid; t < c * c; t += blockDim.x) {
    const int q = t / c, i = t % c;
    const int k = rank_of[q];
    const int slot = k < r ? a + r - 1 - k : a + k;
    V[(long long)slot * ldv + a + i] = Vs[q * CP + i];
  }
  for (int k = tid; k < r; k += blockDim.x) {
    Dp[a + r - 1 - k] = sg[col_of[k]];
    perm[a + r - 1 - k] = a + r - 1 - k;
  }
}

// ------------------------------------------------------ row coefficients ---
// z(p) = sum_q B(c_k, c_k + q) V(c_k + q, p) for every V slot p of the merge's
// window [s, s + M): one thread per slot (poff: prefix of the windows, P + 1).
__global__ void k_bsvd_z(int P, const int *__restrict__ poff, const int *__restrict__ ms,
                         const int *__restrict__ mrow, int sb, int n, const double *__restrict__ AB,
                         long long ldab, const double *__restrict__ V, long long ldv,
                         double *__restrict__ z) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= poff[P]) return;
  const int m = find_merge(poff, P, t);
  const int s = ms[m], ck = mrow[m];
  const int M = poff[m + 1] - poff[m];
  const long long p = s + (t - poff[m]);
  const int qmax = min(sb, min(n, s + M) - 1 - ck);
  double acc = 0.0;
  for (int q = 0; q <= qmax; ++q)
    acc += AB[(long long)(ck + q) * ldab + (sb - q)] * V[p * ldv + ck + q];
  z[p] = acc;
}

// ---------------------------------------------------- null-vector fold ----
// One CTA per merge: the null V slots (c_k .. s + nl + sb - 1, then
// s + N .. s + M - 1) times the Householder reflection H = I - beta v v^T
// with H x = zeta e_1 for x = z on those slots; z(c_k) <- zeta.  Also the
// largest |B(c_k, :)| for the merge's scale (amax[m]).
template <int MT>
__global__ void __launch_bounds__(MT)
k_bsvd_fold(int P, const int *__restrict__ ms, const int *__restrict__ mN,
            const int *__restrict__ mM, const int *__restrict__ mnl, const int *__restrict__ mrow,
            int sb, int n, const double *__restrict__ AB, long long ldab, double *__restrict__ V,
            long long ldv, double *__restrict__ z, double *__restrict__ amax) {
  __shared__ double hv[2 * 32 + 2];
  __shared__ int hslot[2 * 32 + 2];
  __shared__ double s_beta;
  const int m = blockIdx.x;
  if (m >= P) return;
  const int s = ms[m], N = mN[m], M = mM[m], nl = mnl[m], ck = mrow[m];
  const int nleft = s + nl + sb - ck, nn = nleft + (M - N);
  const int tid = threadIdx.x;
  if (tid == 0) {
    double x2 = 0.0, am = 0.0;
    for (int q = 0; q <= sb && ck + q < n; ++q) am = fmax(am, fabs(AB[(long long)(ck + q) * ldab + (sb - q)]));
    for (int c = 0; c < nn; ++c) {
      const int slot = c < nleft ? ck + c : s + N + (c - nleft);
      hslot[c] = slot;
      hv[c] = z[slot];
      x2 += hv[c] * hv[c];
    }
    amax[m] = am;
    const double xn = sqrt(x2);
    if (xn == 0.0 || nn == 1) {
      s_beta = 0.0;  // nothing to fold
    } else {
      const double x0 = hv[0];
      const double zeta = x0 >= 0.0 ? -xn : xn;
      hv[0] = x0 - zeta;
      s_beta = 1.0 / (xn * (xn + fabs(x0)));  // 2 / v^T v
      z[ck] = zeta;
      for (int c = 1; c < nn; ++c) z[hslot[c]] = 0.0;
    }
  }
  __syncthreads();
  const double beta = s_beta;
  if (beta == 0.0) return;
  for (int i = tid; i < M; i += MT) {
    const long long row = s + i;
    double wv = 0.0;
    for (int c = 0; c < nn; ++c) wv += V[(long long)hslot[c] * ldv + row] * hv[c];
    wv *= beta;
    for (int c = 0; c < nn; ++c) V[(long long)hslot[c] * ldv + row] -= wv * hv[c];
  }
}

// ------------------------------------------------------------ deflation ---
// One CTA per merge (MDBDSVD2 / MDBDSVD22): position 0 is the pole of row c_k
// (d = 0, z = z(c_k), U(:, c_k) = e_{c_k}); positions 1 .. cnt - 1 the node's
// current singular values in ascending order, merged from the list
// perm[s .. s + na) and, for the first append, the right child's list
// perm[sb0 .. sb0 + nb).  Scale max(|sigma|, |B(c_k, :)|); tolerance
// 8 eps max(sigma_max, |z|_max) (mdbdsvd2.f90:329-331, mdbdsvd22.f90:198-200).
template <int MT>
__global__ void __launch_bounds__(MT)
k_bsvd_prepare(int P, const int *__restrict__ ms, const int *__restrict__ mrow,
               const int *__restrict__ mna, const int *__restrict__ mb0, const int *__restrict__ mnb,
               const double *__restrict__ amax, const double *__restrict__ zslot,
               double *__restrict__ U, long long ldu, const double *__restrict__ Dp,
               const int *__restrict__ perm, LevelScratch w, int *__restrict__ out,
               double *__restrict__ onrm) {
  const int m = blockIdx.x;
  if (m >= P) return;
  const int s = ms[m], ck = mrow[m], na = mna[m], b0 = mb0[m], nb = mnb[m];
  const int N = na + nb + 1;
  const int tid = threadIdx.x;
  if (tid == 0) U[(long long)ck * ldu + ck] = 1.0;  // the appended row's left vector
  double dm = amax[m];
  for (int i = tid; i < na + nb; i += MT) {
    const int slot = i < na ? perm[s + i] : perm[b0 + (i - na)];
    const double v = Dp[slot];
    w.zs[s + i] = v;
    dm = fmax(dm, fabs(v));
  }
  const double nrm0 = block_max<MT>(dm);
  const double nrm = nrm0 > 0.0 ? nrm0 : 1.0;
  __syncthreads();
  const double *hv = w.zs + s;
  for (int i = tid; i < na; i += MT) {
    const double a = hv[i];
    int lo = 0, hi = nb;
    while (lo < hi) { const int md = (lo + hi) >> 1; if (hv[na + md] < a) lo = md + 1; else hi = md; }
    w.srt[s + 1 + i + lo] = perm[s + i];
    w.ds[s + 1 + i + lo] = a / nrm;
  }
  for (int j = tid; j < nb; j += MT) {
    const double b = hv[na + j];
    int lo = 0, hi = na;
    while (lo < hi) { const int md = (lo + hi) >> 1; if (hv[md] <= b) lo = md + 1; else hi = md; }
    w.srt[s + 1 + j + lo] = perm[b0 + j];
    w.ds[s + 1 + j + lo] = b / nrm;
  }
  __syncthreads();
  const double inv = 1.0 / nrm;
  double zm = 0.0;
  for (int i = tid + 1; i < N; i += MT) {
    const double zv = zslot[w.srt[s + i]] * inv;
    w.zs[s + i] = zv;
    w.typ[s + i] = 1;
    zm = fmax(zm, fabs(zv));
  }
  const double z0 = zslot[ck] * inv;
  if (tid == 0) { w.srt[s] = ck; w.ds[s] = 0.0; w.typ[s] = 0; }
  zm = block_max<MT>(fmax(zm, fabs(z0)));
  const double dmaxn = N > 1 ? w.ds[s + N - 1] : 0.0;
  const double tol = 8.0 * HSS_EPS * fmax(dmaxn, zm);
  const int ng = svd_prep_chain<MT>(s, N, tol, w);
  if (tid == 0) w.zs[s] = fabs(z0) <= tol ? tol : z0;
  __syncthreads();
  svd_prep_compact<MT>(s, N, tol, ng, Dp, w, out + 5 * m);
  if (tid == 0) onrm[m] = nrm;
}

// ---------------------------------------------------------------- launch --
size_t bsvd_leaf_smem() {
  return sizeof(double) * ((size_t)BSVD_COLS_MAX * BSVD_ROWS_MAX + (size_t)BSVD_COLS_MAX * BSVD_COLS_MAX +
                           (size_t)BSVD_ROWS_MAX * BSVD_ROWS_MAX + BSVD_COLS_MAX + BSVD_ROWS_MAX + 1);
}
int bsvd_rows_max() { return BSVD_ROWS_MAX; }
int bsvd_cols_max() { return BSVD_COLS_MAX; }

void launch_bsvd_leaf(int nleaf, const int *la, const int *lr, const int *lc, int sb,
                      const double *AB, long long ldab, double *U, long long ldu, double *V,
                      long long ldv, double *Dp, int *perm, int *status, cudaStream_t st) {
  if (nleaf <= 0) return;
  const size_t smem = bsvd_leaf_smem();
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_bsvd_leaf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    attr = true;
  }
  k_bsvd_leaf<<<nleaf, 256, smem, st>>>(nleaf, la, lr, lc, sb, AB, ldab, U, ldu, V, ldv, Dp, perm,
                                        status);
}

void launch_bsvd_z(int P, int total, const int *poff, const int *ms, const int *mrow, int sb, int n,
                   const double *AB, long long ldab, const double *V, long long ldv, double *z,
                   cudaStream_t st) {
  if (P > 0 && total > 0)
    k_bsvd_z<<<(total + 255) / 256, 256, 0, st>>>(P, poff, ms, mrow, sb, n, AB, ldab, V, ldv, z);
}

void launch_bsvd_fold(int P, int maxm, const int *ms, const int *mN, const int *mM, const int *mnl,
                      const int *mrow, int sb, int n, const double *AB, long long ldab, double *V,
                      long long ldv, double *z, double *amax, cudaStream_t st) {
  if (P <= 0) return;
  if (maxm <= 1024)
    k_bsvd_fold<128><<<P, 128, 0, st>>>(P, ms, mN, mM, mnl, mrow, sb, n, AB, ldab, V, ldv, z, amax);
  else
    k_bsvd_fold<512><<<P, 512, 0, st>>>(P, ms, mN, mM, mnl, mrow, sb, n, AB, ldab, V, ldv, z, amax);
}

void launch_bsvd_prepare(int P, int maxn, const int *ms, const int *mrow, const int *mna,
                         const int *mb0, const int *mnb, const double *amax, const double *zslot,
                         double *U, long long ldu, const double *Dp, const int *perm,
                         const LevelScratch &w, int *out, double *onrm, cudaStream_t st) {
  if (P <= 0) return;
#define BSVDP_CASE(T)                                                                         \
  case T:                                                                                    \
    k_bsvd_prepare<T><<<P, T, 0, st>>>(P, ms, mrow, mna, mb0, mnb, amax, zslot, U, ldu, Dp, \
                                       perm, w, out, onrm);                                  \
    break;
  switch (maxn <= 64 ? 64 : maxn <= 256 ? 128 : maxn <= 2048 ? 256 : 512) {
    BSVDP_CASE(64)
    BSVDP_CASE(128)
    BSVDP_CASE(256)
    default:
    BSVDP_CASE(512)
  }
#undef BSVDP_CASE
}

}  // namespace hss
