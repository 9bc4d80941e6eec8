// hss_svdprep.cuh -- the deflation steps shared by the SVD merge prepares
// (bidiagonal merges, MDLASD2 at SRC/mdlasd2.f90; banded row appends,
// MDBDSVD2 / MDBDSVD22 at SRC/mdbdsvd2.f90, SRC/mdbdsvd22.f90).  One CTA per
// merge.  Positions s .. s + N - 1 of the level scratch hold the merge in
// ascending order of the scaled singular values w.ds, with position 0 the pole
// d = 0 (the new row's left vector), its slot in w.srt, z in w.zs and a column
// type in w.typ (0: the pole, 1 / 2 / 3: left / right / mixed, 4 / 5: deflated
// by a small z / by a rotation).
#pragma once
#include "hss_block.cuh"
#include "hss_kernels.h"

namespace hss {

// Small z deflates (typ 4); the remaining candidates (positions >= 1) are
// listed in w.cand; equal singular values within tol rotate z_prev into z_j
// (one thread walks the chain, from a shared-memory copy when it fits).
// Returns the number of rotations (written to w.gvp/gvq/gvc/gvs).
template <int MT>
__device__ int svd_prep_chain(int s, int N, double tol, const LevelScratch &w) {
  const int tid = threadIdx.x;
  const int chunk = (N - 1 + MT - 1) / MT;
  const int b0 = min(N, 1 + tid * chunk), b1 = min(N, b0 + chunk);
  int cnt = 0;
  for (int i = b0; i < b1; ++i) {
    const bool big = fabs(w.zs[s + i]) > tol;
    cnt += big;
    if (!big) w.typ[s + i] = 4;
  }
  unsigned long long tot;
  int pos = (int)block_scan64<MT>((unsigned long long)cnt, &tot);
  const int nc = (int)tot;
  for (int i = b0; i < b1; ++i)
    if (w.typ[s + i] != 4) w.cand[s + pos++] = i;
  __syncthreads();
  constexpr int NCS = 1536;
  __shared__ double c_z[NCS], c_d[NCS];
  __shared__ unsigned char c_t[NCS];
  __shared__ int s_ng;
  const bool in_smem = nc <= NCS;
  if (in_smem) {
    for (int t = tid; t < nc; t += MT) {
      const int p = w.cand[s + t];
      c_z[t] = w.zs[s + p];
      c_d[t] = w.ds[s + p];
      c_t[t] = w.typ[s + p];
    }
    __syncthreads();
  }
  if (tid == 0) {
    int ng = 0;
    for (int t = 1; t < nc; ++t) {
      const int pt = t - 1;
      const int pp = w.cand[s + pt], np_ = w.cand[s + t];
      const double zp = in_smem ? c_z[pt] : w.zs[s + pp];
      const double zn = in_smem ? c_z[t] : w.zs[s + np_];
      const double dp = in_smem ? c_d[pt] : w.ds[s + pp];
      const double dn = in_smem ? c_d[t] : w.ds[s + np_];
      // the predecessor is the previous candidate: after a rotation the pole
      // rotated into becomes the new JPREV (mdlasd2.f90 loop 100)
      const unsigned char tp = in_smem ? c_t[pt] : w.typ[s + pp];
      if (fabs(dn - dp) <= tol) {
        const double tau = hypot(zn, zp);
        const double cg = zn / tau, sg = -zp / tau;
        const unsigned char tn = in_smem ? c_t[t] : w.typ[s + np_];
        const unsigned char tnn = (tn != tp) ? 3 : tn;
        if (in_smem) { c_z[t] = tau; c_z[pt] = 0.0; c_t[t] = tnn; c_t[pt] = 5; }
        else { w.zs[s + np_] = tau; w.zs[s + pp] = 0.0; w.typ[s + np_] = tnn; w.typ[s + pp] = 5; }
        w.gvp[s + ng] = w.srt[s + pp];
        w.gvq[s + ng] = w.srt[s + np_];
        w.gvc[s + ng] = cg;
        w.gvs[s + ng] = sg;
        ++ng;
      }
    }
    s_ng = ng;
  }
  __syncthreads();
  if (in_smem) {
    for (int t = tid; t < nc; t += MT) {
      const int p = w.cand[s + t];
      w.zs[s + p] = c_z[t];
      w.typ[s + p] = c_t[t];
    }
    __syncthreads();
  }
  const int ng = s_ng;
  __syncthreads();
  return ng;
}

// Compaction: the non-deflated positions (position 0 first) into dl / zw /
// ndslot, the two deflated lists (small z, rotated) merged into one ascending
// list dfval / dfslot (values from Dp, unscaled).  Writes out5[0..4] = {K, ng,
// #left, #right, #mixed}.  The pole's z must already be in w.zs[s].
template <int MT>
__device__ void svd_prep_compact(int s, int N, double tol, int ng, const double *__restrict__ Dp,
                                 const LevelScratch &w, int *__restrict__ out5) {
  const int tid = threadIdx.x;
  const int cb0 = min(N, tid * ((N + MT - 1) / MT)), cb1 = min(N, cb0 + (N + MT - 1) / MT);
  unsigned long long pk = 0;
  int n5 = 0;
  for (int i = cb0; i < cb1; ++i) {
    const int t = w.typ[s + i];
    if (t <= 3) pk += 1ull << (21 * (t <= 1 ? 0 : t == 2 ? 1 : 2));
    n5 += (t == 5);
  }
  unsigned long long ptot, t5;
  const unsigned long long pre = block_scan64<MT>(pk, &ptot);
  int r5 = (int)block_scan64<MT>((unsigned long long)n5, &t5);
  const int c1 = (int)(ptot & 0x1fffff), c2 = (int)((ptot >> 21) & 0x1fffff),
            c3 = (int)((ptot >> 42) & 0x1fffff);
  const int K = c1 + c2 + c3;
  const int nrot = (int)t5;
  int j = (int)(pre & 0x1fffff) + (int)((pre >> 21) & 0x1fffff) + (int)((pre >> 42) & 0x1fffff);
  for (int i = cb0; i < cb1; ++i) {
    const int t = w.typ[s + i];
    const int slot = w.srt[s + i];
    if (t <= 3) {
      w.dl[s + j] = w.ds[s + i];
      w.zw[s + j] = w.zs[s + i];
      w.ndslot[s + j] = slot;
      ++j;
    } else {
      const int a = i - j;  // deflated before position i
      const double v = Dp[slot];
      if (t == 5) { w.l2slot[s + r5] = slot; w.l2val[s + r5] = v; ++r5; }
      else { const int a1 = a - r5; w.l1slot[s + a1] = slot; w.l1val[s + a1] = v; }
    }
  }
  __syncthreads();
  // the first pole after the center stays at least tol/2 away from it
  if (tid == 0 && K >= 2 && fabs(w.dl[s + 1]) <= 0.5 * tol) w.dl[s + 1] = 0.5 * tol;
  const int n1l = (N - K) - nrot;
  for (int i = tid; i < n1l; i += MT) {  // both lists are ascending: merge them
    const double v = w.l1val[s + i];
    int lo = 0, hi = nrot;
    while (lo < hi) { const int md = (lo + hi) >> 1; if (w.l2val[s + md] < v) lo = md + 1; else hi = md; }
    w.dfval[s + i + lo] = v; w.dfslot[s + i + lo] = w.l1slot[s + i];
  }
  for (int i = tid; i < nrot; i += MT) {
    const double v = w.l2val[s + i];
    int lo = 0, hi = n1l;
    while (lo < hi) { const int md = (lo + hi) >> 1; if (w.l1val[s + md] <= v) lo = md + 1; else hi = md; }
    w.dfval[s + i + lo] = v; w.dfslot[s + i + lo] = w.l2slot[s + i];
  }
  if (tid == 0) { out5[0] = K; out5[1] = ng; out5[2] = c1; out5[3] = c2; out5[4] = c3; }
}

}  // namespace hss
