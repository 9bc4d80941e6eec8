// svd.cu -- bidiagonal SVD divide and conquer (MDBDSDC, SRC/mdbdsdc.f90:1;
// MDLASD0-3/8, SRC/mdlasd1.f90, SRC/mdlasd2.f90, SRC/mdlasd8.f90).
//
// Storage ("physical slots", as the eigensolver): U (n x n) and V (m x m,
// V = VT^T, right singular vectors as columns) never move their columns.  Slot
// p holds U(:, p), V(:, p) and sigma_p = Dp[p]; a node covering rows
// [s, s + N) has its N triples in slots s .. s + N - 1 and, when it has an extra
// column (sqre = 1), its null vector in V slot s + N.  The center row c = s + nl
// of a merge starts as U(:, c) = e_c, paired with V slot c = the left child's
// null vector (the d_1 = 0 entry of DLASD2).
//
// A merge is the SVD of the K x K "broken arrow" M = e_1 z^T + diag(d),
// d_1 = 0 (after deflation).  Since M^T M = diag(d^2) + z z^T, its right
// singular vectors are the Cauchy-like columns z_i / (d_i^2 - sigma_j^2) and
// U = M V Sigma^-1 gives u_1j = -1, u_ij = d_i z_i / (d_i^2 - sigma_j^2) up to
// column norms (DLASD3).  The secular equation, the Loewner rebuild of z and
// the column norms therefore run through the eigensolver's kernels in their
// squared mode; this file holds the leaf SVDs, the deflation (MDLASD2) and the
// construction of the two K x K vector blocks.
#include "hss_block.cuh"
#include "hss_common.cuh"
#include "hss_kernels.h"
#include "hss_svdprep.cuh"

namespace hss {

constexpr int SVD_LEAF_MAX = 32;

// ------------------------------------------------------------- leaves -----
// One thread per leaf: the r x (r + sqre) upper bidiagonal rows a .. a + r - 1
// (diag d[a + i], superdiag e[a + i]; with sqre the extra entry e[a + r - 1] sits
// in column a + r) by the Golub-Kahan implicit-shift QR SVD (Golub & Kahan
// 1965; Golub & Van Loan, Alg. 8.6.2), U and V accumulated as products of
// rotations (the role of DLASDQ at SRC/mdlasd0.f90).  The extra column is first
// chased out by column rotations, leaving its null vector in V(:, r).  Results
// sorted ascending into slots a .. a + r - 1 (U, V, Dp, perm) and V slot a + r.
__global__ void __launch_bounds__(32)
k_svd_leaf(int nleaf, const int *__restrict__ lstart, const int *__restrict__ lsize,
           const int *__restrict__ lsqre, int rmax, const double *__restrict__ d,
           const double *__restrict__ e, double *__restrict__ U, long long ldu,
           double *__restrict__ V, long long ldv, double *__restrict__ Dp, int *__restrict__ perm,
           int *__restrict__ status) {
  extern __shared__ double lsm[];
  const int lane = threadIdx.x, LW = blockDim.x;
  const int leaf = blockIdx.x * LW + lane;
  const int cmax = rmax + 1;
  double *Ds = lsm, *Es = lsm + rmax * LW, *Us = lsm + 2 * rmax * LW,
         *Vs = lsm + (2 * rmax + rmax * rmax) * LW;
#define DD(i) Ds[(i) * LW + lane]
#define EE(i) Es[(i) * LW + lane]
#define UU(r_, c_) Us[((r_) * rmax + (c_)) * LW + lane]
#define VV(r_, c_) Vs[((r_) * cmax + (c_)) * LW + lane]
  if (leaf >= nleaf) return;
  const int a = lstart[leaf], r = lsize[leaf], sq = lsqre[leaf], c = r + sq;
  for (int i = 0; i < r; ++i) {
    DD(i) = d[a + i];
    EE(i) = (i < r - 1 + sq) ? e[a + i] : 0.0;
    for (int j = 0; j < r; ++j) UU(i, j) = (i == j) ? 1.0 : 0.0;
  }
  for (int i = 0; i < c; ++i)
    for (int j = 0; j < c; ++j) VV(i, j) = (i == j) ? 1.0 : 0.0;
  if (sq) {  // chase the extra column's entry up and out: column r becomes zero
    double f = EE(r - 1);
    EE(r - 1) = 0.0;
    for (int i = r - 1; i >= 0; --i) {
      const double t = hypot(DD(i), f);
      const double cs = t == 0.0 ? 1.0 : DD(i) / t, sn = t == 0.0 ? 0.0 : f / t;
      DD(i) = t;
      for (int q = 0; q < c; ++q) {
        const double vi = VV(q, i), vr = VV(q, r);
        VV(q, i) = cs * vi + sn * vr;
        VV(q, r) = -sn * vi + cs * vr;
      }
      if (i > 0) { f = -sn * EE(i - 1); EE(i - 1) = cs * EE(i - 1); }
    }
  }
  int iter = 0, bad = 0;
  while (true) {
    for (int i = 0; i + 1 < r; ++i)
      if (fabs(EE(i)) <= HSS_EPS * (fabs(DD(i)) + fabs(DD(i + 1)))) EE(i) = 0.0;
    int hi = r - 1;
    while (hi > 0 && EE(hi - 1) == 0.0) --hi;
    if (hi == 0) break;
    int lo = hi - 1;
    while (lo > 0 && EE(lo - 1) != 0.0) --lo;
    if (++iter > 30 * r * r) { bad = 1; break; }
    int zi = -1;
    for (int i = lo; i < hi; ++i)
      if (DD(i) == 0.0) { zi = i; break; }
    if (zi < 0 && DD(hi) == 0.0) {  // zero at the bottom: chase E(hi-1) out by columns
      double f = EE(hi - 1);
      EE(hi - 1) = 0.0;
      for (int k = hi - 1; k >= lo; --k) {
        const double t = hypot(DD(k), f);
        const double cs = DD(k) / t, sn = f / t;
        DD(k) = t;
        for (int q = 0; q < c; ++q) {
          const double vk = VV(q, k), vh = VV(q, hi);
          VV(q, k) = cs * vk + sn * vh;
          VV(q, hi) = -sn * vk + cs * vh;
        }
        if (k > lo) { f = -sn * EE(k - 1); EE(k - 1) = cs * EE(k - 1); }
      }
      continue;
    }
    if (zi >= 0) {  // zero inside: chase row zi's superdiagonal out by rows
      double f = EE(zi);
      EE(zi) = 0.0;
      for (int k = zi + 1; k <= hi; ++k) {
        const double t = hypot(DD(k), f);
        const double cs = DD(k) / t, sn = f / t;
        DD(k) = t;
        for (int q = 0; q < r; ++q) {
          const double uk = UU(q, k), ui = UU(q, zi);
          UU(q, k) = cs * uk + sn * ui;
          UU(q, zi) = -sn * uk + cs * ui;
        }
        if (k < hi) { f = -sn * EE(k); EE(k) = cs * EE(k); }
      }
      continue;
    }
    // Wilkinson shift from the trailing 2 x 2 of B^T B of the block
    const int mm = hi;
    const double t11 = DD(mm - 1) * DD(mm - 1) + (mm - 1 > lo ? EE(mm - 2) * EE(mm - 2) : 0.0);
    const double t12 = DD(mm - 1) * EE(mm - 1);
    const double t22 = DD(mm) * DD(mm) + EE(mm - 1) * EE(mm - 1);
    const double dd = 0.5 * (t11 - t22);
    double mu;
    if (dd == 0.0 && t12 == 0.0) mu = t22;
    else mu = t22 - t12 * t12 / (dd + copysign(hypot(dd, t12), dd != 0.0 ? dd : 1.0));
    double y = DD(lo) * DD(lo) - mu, z = DD(lo) * EE(lo), bulge = 0.0;
    for (int k = lo; k < hi; ++k) {
      double t = hypot(y, z);
      double cs = t == 0.0 ? 1.0 : y / t, sn = t == 0.0 ? 0.0 : z / t;
      if (k > lo) EE(k - 1) = t;
      {
        const double dk = DD(k), ek = EE(k);
        DD(k) = cs * dk + sn * ek;
        EE(k) = -sn * dk + cs * ek;
      }
      const double bl = sn * DD(k + 1);
      DD(k + 1) = cs * DD(k + 1);
      for (int q = 0; q < c; ++q) {
        const double vk = VV(q, k), vk1 = VV(q, k + 1);
        VV(q, k) = cs * vk + sn * vk1;
        VV(q, k + 1) = -sn * vk + cs * vk1;
      }
      y = DD(k);
      z = bl;
      t = hypot(y, z);
      cs = t == 0.0 ? 1.0 : y / t;
      sn = t == 0.0 ? 0.0 : z / t;
      DD(k) = t;
      {
        const double ek = EE(k), dk1 = DD(k + 1);
        EE(k) = cs * ek + sn * dk1;
        DD(k + 1) = -sn * ek + cs * dk1;
      }
      if (k + 1 < hi) { bulge = sn * EE(k + 1); EE(k + 1) = cs * EE(k + 1); }
      for (int q = 0; q < r; ++q) {
        const double uk = UU(q, k), uk1 = UU(q, k + 1);
        UU(q, k) = cs * uk + sn * uk1;
        UU(q, k + 1) = -sn * uk + cs * uk1;
      }
      if (k < hi - 1) { y = EE(k); z = bulge; }
    }
  }
  for (int i = 0; i < r; ++i)
    if (DD(i) < 0.0) {
      DD(i) = -DD(i);
      for (int q = 0; q < c; ++q) VV(q, i) = -VV(q, i);
    }
  for (int i = 0; i + 1 < r; ++i) {  // ascending, moving the columns along
    int k = i;
    double pmin = DD(i);
    for (int j = i + 1; j < r; ++j)
      if (DD(j) < pmin) { k = j; pmin = DD(j); }
    if (k != i) {
      DD(k) = DD(i);
      DD(i) = pmin;
      for (int q = 0; q < r; ++q) { const double t = UU(q, i); UU(q, i) = UU(q, k); UU(q, k) = t; }
      for (int q = 0; q < c; ++q) { const double t = VV(q, i); VV(q, i) = VV(q, k); VV(q, k) = t; }
    }
  }
  for (int j = 0; j < r; ++j) {
    for (int q = 0; q < r; ++q) U[(long long)(a + j) * ldu + a + q] = UU(q, j);
    Dp[a + j] = DD(j);
    perm[a + j] = a + j;
  }
  for (int j = 0; j < c; ++j)
    for (int q = 0; q < c; ++q) V[(long long)(a + j) * ldv + a + q] = VV(q, j);
  if (bad) atomicMax(status, HSS_LEAF_NOCONV);
#undef DD
#undef EE
#undef UU
#undef VV
}

// ------------------------------------------------------------ deflation ---
// One CTA per merge (MDLASD2, SRC/mdlasd2.f90).  Merge m: rows s .. s + N - 1
// with N = nl + 1 + nr, center c = s + nl, alpha = d[c], beta = e[c], extra
// column if sqre.  Outputs as the eigensolver's prepare: the non-deflated list
// (position 0 = the center, pole 0) in dl / zw / ndslot, the deflated slots in
// ascending order in dfval / dfslot, Givens pairs, out[5m] = {K, #rotations,
// #left-only, #right-only, #mixed}, and the scale onrm[m] of the merge
// (MDLASD1 divides by max(|alpha|, |beta|, |d_i|), SRC/mdlasd1.f90).
template <int MT>
__global__ void __launch_bounds__(MT)
k_svd_prepare(int P, const int *__restrict__ ms, const int *__restrict__ mnl,
              const int *__restrict__ mnr, const int *__restrict__ msq,
              const double *__restrict__ dB, const double *__restrict__ eB, double *__restrict__ U,
              long long ldu, double *__restrict__ V, long long ldv, const double *__restrict__ Dp,
              const int *__restrict__ perm, LevelScratch w, int *__restrict__ out,
              double *__restrict__ onrm) {
  const int m = blockIdx.x;
  if (m >= P) return;
  const int s = ms[m], nl = mnl[m], nr = mnr[m], sqre = msq[m];
  const int N = nl + 1 + nr, c = s + nl;
  const int tid = threadIdx.x;
  const double alpha = dB[c], beta = eB[c];
  if (tid == 0) U[(long long)c * ldu + c] = 1.0;  // the center row's left vector e_c
  // ---- scale (MDLASD1) and merge the children's ascending lists (DLAMRG) into
  //      positions 1 .. N-1; position 0 is the center
  double dm = fmax(fabs(alpha), fabs(beta));
  for (int i = tid; i < N - 1; i += MT) {
    const int slot = i < nl ? perm[s + i] : perm[c + 1 + (i - nl)];
    const double v = Dp[slot];
    w.zs[s + i] = v;
    dm = fmax(dm, fabs(v));
  }
  const double nrm0 = block_max<MT>(dm);
  const double nrm = nrm0 > 0.0 ? nrm0 : 1.0;
  __syncthreads();
  const double *hv = w.zs + s;
  for (int i = tid; i < nl; i += MT) {
    const double a = hv[i];
    int lo = 0, hi = nr;
    while (lo < hi) { const int md = (lo + hi) >> 1; if (hv[nl + md] < a) lo = md + 1; else hi = md; }
    w.srt[s + 1 + i + lo] = perm[s + i];
    w.ds[s + 1 + i + lo] = a / nrm;
  }
  for (int j = tid; j < nr; j += MT) {
    const double b = hv[nl + j];
    int lo = 0, hi = nl;
    while (lo < hi) { const int md = (lo + hi) >> 1; if (hv[md] <= b) lo = md + 1; else hi = md; }
    w.srt[s + 1 + j + lo] = perm[c + 1 + j];
    w.ds[s + 1 + j + lo] = b / nrm;
  }
  __syncthreads();
  // ---- z (mdlasd2.f90: alpha * VT(i, NL+1) for the left, beta * VT(i, NL+2)
  //      for the right) in merged order
  const double an = alpha / nrm, bn = beta / nrm;
  for (int i = tid + 1; i < N; i += MT) {
    const int slot = w.srt[s + i];
    const bool left = slot < c;
    w.zs[s + i] = left ? an * V[(long long)slot * ldv + c] : bn * V[(long long)slot * ldv + c + 1];
    w.typ[s + i] = left ? 1 : 2;
  }
  if (tid == 0) { w.srt[s] = c; w.ds[s] = 0.0; w.typ[s] = 0; }
  const double z1 = an * V[(long long)c * ldv + c];
  const double zM = sqre ? bn * V[(long long)(s + N) * ldv + c + 1] : 0.0;
  __syncthreads();
  const double dmaxn = N > 1 ? w.ds[s + N - 1] : 0.0;
  const double tol = 8.0 * HSS_EPS * fmax(dmaxn, fmax(fabs(an), fabs(bn)));
  // ---- small z deflates (mdlasd2.f90 loop 80/100); equal singular values
  //      within tol are rotated together
  const int ng = svd_prep_chain<MT>(s, N, tol, w);
  // ---- the center's z (with the right null vector rotated in when sqre)
  double zz1, cg1 = 1.0, sg1 = 0.0;
  if (sqre) {
    zz1 = hypot(z1, zM);
    if (zz1 <= tol) zz1 = tol;
    else { cg1 = z1 / zz1; sg1 = zM / zz1; }
    // V(:, c) <- cg V(:, c) + sg V(:, s+N);  V(:, s+N) <- -sg V(:, c) + cg V(:, s+N)
    for (int i = tid; i < N + 1; i += MT) {
      const long long rr = s + i;
      const double vc = V[(long long)c * ldv + rr], vn = V[(long long)(s + N) * ldv + rr];
      V[(long long)c * ldv + rr] = cg1 * vc + sg1 * vn;
      V[(long long)(s + N) * ldv + rr] = -sg1 * vc + cg1 * vn;
    }
  } else {
    zz1 = fabs(z1) <= tol ? tol : z1;
  }
  if (tid == 0) w.zs[s] = zz1;
  __syncthreads();
  // ---- compact: non-deflated (position 0 first) and the two deflated lists
  svd_prep_compact<MT>(s, N, tol, ng, Dp, w, out + 5 * m);
  if (tid == 0) onrm[m] = nrm;
}

// ------------------------------------------------------- vector blocks ----
// Warp per column j of merge m: V block v_ij = zhat_i / (d_i^2 - sigma_j^2),
// U block u_0j = -1, u_ij = d_i zhat_i / (d_i^2 - sigma_j^2), each column scaled
// to unit length (DLASD3).  Column-major K x K blocks at Vb / Ub + boff[m].
__global__ void k_svd_vectors(LevelView lv, const double *__restrict__ dl,
                              const double *__restrict__ difl, const double *__restrict__ difr,
                              const double *__restrict__ zhat, const long long *__restrict__ boff,
                              double *__restrict__ Ub, double *__restrict__ Vb) {
  const int lane = threadIdx.x & 31;
  const int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (r >= __ldg(lv.rootoff + lv.P)) return;
  const int m = find_merge(lv.rootoff, lv.P, r);
  const int j = r - __ldg(lv.rootoff + m);
  const int s = __ldg(lv.s + m);
  const int K = __ldg(lv.K + m);
  PoleDiff P{dl + s, difl + s, difr + s, true};
  double *vc = Vb + boff[m] + (long long)j * K, *uc = Ub + boff[m] + (long long)j * K;
  // each entry is formed once (FP64 issue slots are the scarce resource): the
  // unnormalised V column goes out first and is rescaled from L2 by the same
  // lanes; the divide through the one-ulp reciprocal
  double sv = 0.0, su = 0.0;
  for (int i = lane; i < K; i += HSS_WARP) {
    const double v = qdiv(__ldg(zhat + s + i), P.fd(i, j));
    vc[i] = v;
    sv += v * v;
    if (i > 0) { const double u = __ldg(dl + s + i) * v; su += u * u; }
  }
  sv = warp_sum(sv);
  su = warp_sum(su);
  const double av = 1.0 / sqrt(sv), au = 1.0 / sqrt(1.0 + su);
  for (int i = lane; i < K; i += HSS_WARP) {
    const double v = vc[i];
    vc[i] = v * av;
    uc[i] = i == 0 ? -au : __ldg(dl + s + i) * v * au;
  }
}

// One merge's column norms for the HSS path: alpha_j (V block), beta_j (U
// block, including the -1 of row 0) and the U generator ud_i = d_i zhat_i
// (arrays already offset to the merge; warp per column).
__global__ void k_svd_norms(int K, const double *__restrict__ dl, const double *__restrict__ difl,
                            const double *__restrict__ difr, const double *__restrict__ zhat,
                            double *__restrict__ alpha, double *__restrict__ beta,
                            double *__restrict__ ud) {
  const int lane = threadIdx.x & 31;
  const int j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (j >= K) return;
  PoleDiff P{dl, difl, difr, true};
  double sv = 0.0, su = 0.0;
  for (int i = lane; i < K; i += HSS_WARP) {
    const double v = __ldg(zhat + i) / P.fd(i, j);
    sv += v * v;
    if (i > 0) { const double u = __ldg(dl + i) * v; su += u * u; }
  }
  sv = warp_sum(sv);
  su = warp_sum(su);
  if (lane == 0) {
    alpha[j] = 1.0 / sqrt(sv);
    beta[j] = 1.0 / sqrt(1.0 + su);
    ud[j] = __ldg(dl + j) * __ldg(zhat + j);
  }
}

// T(:, j) -= beta_j X(:, 0): the row-0 entries -beta_j of the U block.
__global__ void k_svd_rank1(int nrows, int K, const double *__restrict__ X, long long ldx,
                            const double *__restrict__ beta, double *__restrict__ T,
                            long long ldt) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)nrows * K) return;
  const int i = (int)(idx % nrows), j = (int)(idx / nrows);
  T[(long long)j * ldt + i] -= beta[j] * X[i];
}

void launch_svd_norms(int K, const double *dl, const double *difl, const double *difr,
                      const double *zhat, double *alpha, double *beta, double *ud,
                      cudaStream_t st) {
  if (K > 0)
    k_svd_norms<<<(unsigned)(((long long)K * 32 + 255) / 256), 256, 0, st>>>(K, dl, difl, difr,
                                                                             zhat, alpha, beta, ud);
}
void launch_svd_rank1(int nrows, int K, const double *X, long long ldx, const double *beta,
                      double *T, long long ldt, cudaStream_t st) {
  const long long tot = (long long)nrows * K;
  if (tot > 0)
    k_svd_rank1<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(nrows, K, X, ldx, beta, T, ldt);
}

// sigma of every root back to the merge's scale (lam *= onrm[m]).
__global__ void k_svd_unscale(LevelView lv, const double *__restrict__ onrm,
                              double *__restrict__ lam) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= __ldg(lv.rootoff + lv.P)) return;
  const int m = find_merge(lv.rootoff, lv.P, r);
  lam[__ldg(lv.s + m) + r - __ldg(lv.rootoff + m)] *= onrm[m];
}

// VT(i, :) = V(:, perm(n-1-i))^T (descending singular values): 32 x 32 tiles
// through shared memory so both the reads of V and the writes of VT coalesce.
__global__ void k_svd_vt(int n, const int *__restrict__ perm, const double *__restrict__ V,
                         long long ldv, double *__restrict__ VT, long long ldvt) {
  __shared__ double tile[32][33];
  const int i0 = blockIdx.x * 32, j0 = blockIdx.y * 32;  // rows i of VT, columns j
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int i = i0 + k, j = j0 + threadIdx.x;
    if (i < n && j < n) tile[k][threadIdx.x] = V[(long long)perm[n - 1 - i] * ldv + j];
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int j = j0 + k, i = i0 + threadIdx.x;
    if (i < n && j < n) VT[(long long)j * ldvt + i] = tile[threadIdx.x][k];
  }
}

// U(:, i) = Uq(:, perm(n-1-i)), w(i) = Dp(perm(n-1-i)) (descending).
__global__ void k_svd_u(int n, const int *__restrict__ perm, const double *__restrict__ Dp,
                        const double *__restrict__ Uq, long long ldq, double *__restrict__ Uo,
                        long long ldu, double *__restrict__ w) {
  const int col = blockIdx.x;
  if (col >= n) return;
  const long long p = perm[n - 1 - col];
  for (int i = threadIdx.x; i < n; i += blockDim.x) Uo[(long long)col * ldu + i] = Uq[p * ldq + i];
  if (threadIdx.x == 0) w[col] = Dp[p];
}

__global__ void k_svd_w(int n, const int *__restrict__ perm, const double *__restrict__ Dp,
                        double *__restrict__ w) {
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col < n) w[col] = Dp[perm[n - 1 - col]];
}

// Rows of A rotated back to front (DLASR('L', 'V', 'B'), the lower-to-upper
// rotations of DBDSDC applied to U): for j = n-2 .. 0, with c = cs[j],
// s = sn[j]: (A_j, A_{j+1}) <- (s A_{j+1} + c A_j, c A_{j+1} - s A_j).  One
// thread per column.
__global__ void k_rows_rotate_back(int n, int ncols, const double *__restrict__ cs,
                                   const double *__restrict__ sn, double *__restrict__ A,
                                   long long lda) {
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= ncols) return;
  double *a = A + (long long)col * lda;
  for (int j = n - 2; j >= 0; --j) {
    const double c = cs[j], s = sn[j];
    const double t = a[j + 1];
    a[j + 1] = c * t - s * a[j];
    a[j] = s * t + c * a[j];
  }
}

// ---------------------------------------------------------------- launch --
void launch_rows_rotate_back(int n, int ncols, const double *cs, const double *sn, double *A,
                             long long lda, cudaStream_t st) {
  if (n > 1 && ncols > 0) k_rows_rotate_back<<<(ncols + 127) / 128, 128, 0, st>>>(n, ncols, cs, sn, A, lda);
}

void launch_svd_leaf(int nleaf, const int *lstart, const int *lsize, const int *lsqre, int rmax,
                     const double *d, const double *e, double *U, long long ldu, double *V,
                     long long ldv, double *Dp, int *perm, int *status, cudaStream_t st) {
  if (nleaf <= 0) return;
  rmax = std::max(1, std::min(rmax, SVD_LEAF_MAX));
  const size_t per = (size_t)(2 * rmax + rmax * rmax + (rmax + 1) * (rmax + 1)) * sizeof(double);
  int lw = 32;
  while (lw > 8 && (nleaf + lw - 1) / lw < 2 * 148) lw /= 2;
  while (lw > 1 && per * lw > 200 * 1024) lw /= 2;
  const size_t smem = per * lw;
  static size_t attr = 0;
  if (smem > 48 * 1024 && smem > attr) {
    cudaFuncSetAttribute(k_svd_leaf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    attr = smem;
  }
  k_svd_leaf<<<(nleaf + lw - 1) / lw, lw, smem, st>>>(nleaf, lstart, lsize, lsqre, rmax, d, e, U,
                                                       ldu, V, ldv, Dp, perm, status);
}

static int svd_threads(int maxn) {
  return maxn <= 64 ? 64 : maxn <= 256 ? 128 : maxn <= 2048 ? 256 : 512;
}

void launch_svd_prepare(int P, int maxn, const int *ms, const int *mnl, const int *mnr,
                        const int *msq, const double *d, const double *e, double *U,
                        long long ldu, double *V, long long ldv, const double *Dp, const int *perm,
                        const LevelScratch &w, int *out, double *onrm, cudaStream_t st) {
  if (P <= 0) return;
#define SVDP_CASE(T)                                                                        \
  case T:                                                                                  \
    k_svd_prepare<T><<<P, T, 0, st>>>(P, ms, mnl, mnr, msq, d, e, U, ldu, V, ldv, Dp, perm, \
                                      w, out, onrm);                                       \
    break;
  switch (svd_threads(maxn)) {
    SVDP_CASE(64)
    SVDP_CASE(128)
    SVDP_CASE(256)
    default:
    SVDP_CASE(512)
  }
#undef SVDP_CASE
}

void launch_svd_vectors(const LevelView &lv, int total, const double *dl, const double *difl,
                        const double *difr, const double *zhat, const long long *boff, double *Ub,
                        double *Vb, cudaStream_t st) {
  if (total <= 0) return;
  k_svd_vectors<<<(unsigned)(((long long)total * 32 + 255) / 256), 256, 0, st>>>(
      lv, dl, difl, difr, zhat, boff, Ub, Vb);
}
void launch_svd_unscale(const LevelView &lv, int total, const double *onrm, double *lam,
                        cudaStream_t st) {
  if (total > 0) k_svd_unscale<<<(total + 255) / 256, 256, 0, st>>>(lv, onrm, lam);
}

void launch_svd_outputs(int n, const int *perm, const double *Dp, const double *Uq,
                        long long ldq, const double *V, long long ldv, double *Uo, long long ldu,
                        double *VT, long long ldvt, double *w, bool vectors, cudaStream_t st) {
  if (n <= 0) return;
  if (vectors) {
    k_svd_u<<<n, 256, 0, st>>>(n, perm, Dp, Uq, ldq, Uo, ldu, w);
    dim3 g((n + 31) / 32, (n + 31) / 32);
    k_svd_vt<<<g, dim3(32, 8), 0, st>>>(n, perm, V, ldv, VT, ldvt);
  } else {
    k_svd_w<<<(n + 255) / 256, 256, 0, st>>>(n, perm, Dp, w);
  }
}

}  // namespace hss
