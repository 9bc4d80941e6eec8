// merge.cu -- per-level bookkeeping of the DC merges (MDLAED1/MDLAED2 of
// SRC/mdlaed1.f90:109-233 and SRC/mdlaed2.f90:149-528), batched one CTA per merge.
//
// Storage model ("physical slots").  The eigenvector matrix Q (n x n, column-
// major) is block diagonal at every level.  A column never moves: slot p keeps
// its storage, Dp[p] its eigenvalue, and perm[] lists the slots of each block
// in ascending eigenvalue order.  A merge rewrites only the K slots whose
// eigenvectors change (the non-deflated ones); deflated columns stay where
// they are, modified in place only by deflating Givens rotations.  This is the
// reference's INDXQ indirection (mdlaed0.f90:221, mdlaed2.f90:229-233) carried
// through to the end, so no level copies the whole n x n block.
#include <cooperative_groups.h>

#include "hss_block.cuh"
#include "hss_common.cuh"
#include "hss_kernels.h"

namespace hss {

// Q(row, slot) where the column is known to be zero outside the rows
// sup[slot] = [lo, hi) it has been written on (sup == nullptr: all rows valid).
__device__ __forceinline__ double qat(const double *__restrict__ Q, long long ldq,
                                      const int2 *__restrict__ sup, int slot, long long row) {
  if (sup) {
    const int2 r = sup[slot];
    if (row < r.x || row >= r.y) return 0.0;
  }
  return Q[(long long)slot * ldq + row];
}

// out[5*m + {0..4}] = K, #rotations, #type1, #type2, #type3 ; orho[m] = |2 rho|
template <int MT>
__global__ void __launch_bounds__(MT)
k_merge_prepare(int P, const int *__restrict__ ms, const int *__restrict__ mn,
                const int *__restrict__ mn1, const double *__restrict__ e,
                const double *__restrict__ Q, long long ldq, double *__restrict__ Dp,
                int *__restrict__ perm, LevelScratch w, int *__restrict__ out,
                double *__restrict__ orho, const double *__restrict__ zsrc,
                const double *__restrict__ rsrc, int flags, const int2 *__restrict__ sup) {
  const int m = blockIdx.x;
  if (m >= P) return;
  const int s = ms[m], n = mn[m], n1 = mn1[m], n2 = n - n1;
  const int tid = threadIdx.x;
  const double rho_in = rsrc ? rsrc[m] : e[s + n1 - 1];
  if (flags & PREP_FRONT) {
    // merged order and z already written by k_merge_front
  } else if (flags & PREP_SORTED) {
    // ---- the whole block is already ascending (a later rank-one update of a
    //      banded merge: mdsbed22.f90 takes INDXQ as it is)
    for (int i = tid; i < n; i += MT) {
      const int slot = perm[s + i];
      w.srt[s + i] = slot;
      w.ds[s + i] = Dp[slot];
    }
  } else {
    // ---- merge the two ascending halves (DLAMRG, ties to the first list) by
    //      merge path on contiguous copies of their eigenvalues (zs as scratch)
    for (int i = tid; i < n; i += MT) w.zs[s + i] = Dp[perm[s + i]];
    __syncthreads();
    const double *hv = w.zs + s;
    for (int i = tid; i < n1; i += MT) {
      const double a = hv[i];
      int lo = 0, hi = n2;  // count right values < a
      while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (hv[n1 + mid] < a) lo = mid + 1; else hi = mid;
      }
      w.srt[s + i + lo] = perm[s + i];
      w.ds[s + i + lo] = a;
    }
    for (int j = tid; j < n2; j += MT) {
      const double b = hv[n1 + j];
      int lo = 0, hi = n1;  // count left values <= b
      while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (hv[mid] <= b) lo = mid + 1; else hi = mid;
      }
      w.srt[s + j + lo] = perm[s + n1 + j];
      w.ds[s + j + lo] = b;
    }
  }
  __syncthreads();
  // ---- z = [last row of Q1, first row of Q2] / sqrt(2) (mdlaed1.f90:178-180,
  //      mdlaed2.f90:203-211) in merged order, or a given z per slot (Q^T w
  //      of a banded cut, scaled the same way at mdsbed22.f90)
  const double sc = 1.0 / sqrt(2.0);
  double dmax = 0.0, zmax = 0.0;
  for (int i = tid; i < n; i += MT) {
    double z;
    if (flags & PREP_FRONT) {
      z = w.zs[s + i];
    } else {
      const int slot = w.srt[s + i];
      const bool top = slot < s + n1;
      z = zsrc ? zsrc[slot] : qat(Q, ldq, sup, slot, top ? s + n1 - 1 : s + n1);
      if (!top && rho_in < 0.0) z = -z;
      z *= sc;
      w.zs[s + i] = z;
      w.typ[s + i] = (flags & PREP_DENSE) ? 2 : top ? 1 : 3;
    }
    dmax = fmax(dmax, fabs(w.ds[s + i]));
    zmax = fmax(zmax, fabs(z));
  }
  dmax = block_max<MT>(dmax);
  zmax = block_max<MT>(zmax);
  const double rho = fabs(2.0 * rho_in);
  const double tol = 8.0 * HSS_EPS * fmax(dmax, zmax);  // mdlaed2.f90:265-267
  if (rho * zmax <= tol) {  // nothing couples the halves
    for (int i = tid; i < n; i += MT) perm[s + i] = w.srt[s + i];
    if (tid == 0) {
      out[5 * m] = 0; out[5 * m + 1] = 0; out[5 * m + 2] = 0; out[5 * m + 3] = 0;
      out[5 * m + 4] = 0;
      orho[m] = rho;
    }
    return;
  }
  // ---- candidates: z large enough (deflation by small z, mdlaed2.f90:304-313)
  // Warp w scans the contiguous positions [w0, w1) in steps of 32 consecutive
  // positions (coalesced); ballots rank a position among its warp's, and a
  // scan over the warps' totals orders the warps, so every compaction keeps
  // the position order.
  constexpr int NW = MT / 32;
  const int lane = tid & 31, wid = tid >> 5;
  const int seg = (((n + NW - 1) / NW) + 31) & ~31;
  const int w0 = min(n, wid * seg), w1 = min(n, w0 + seg);
  const unsigned below = (1u << lane) - 1u;  // lanes ahead of this one
  // (position passes load four iterations ahead: the loads of one batch are
  // in flight together instead of one latency per 32 positions)
  constexpr int PB = 4;
  int cnt = 0;
  for (int i0 = w0; i0 < w1; i0 += 32 * PB) {
    double zv[PB];
#pragma unroll
    for (int b = 0; b < PB; ++b) {
      const int i = i0 + 32 * b + lane;
      zv[b] = i < w1 ? w.zs[s + i] : 0.0;
    }
#pragma unroll
    for (int b = 0; b < PB; ++b) {
      const int i = i0 + 32 * b + lane;
      const bool in = i < w1;
      const bool big = in && rho * fabs(zv[b]) > tol;
      if (in && !big) w.typ[s + i] = 4;  // deflated, small z
      cnt += __popc(__ballot_sync(HSS_FULL, big));
    }
  }
  unsigned long long tot;
  int pos = (int)block_scan64<MT>(lane == 0 ? (unsigned long long)cnt : 0ull, &tot);
  pos = __shfl_sync(HSS_FULL, pos, 0);
  const int nc = (int)tot;
  for (int i0 = w0; i0 < w1; i0 += 32 * PB) {
    double zv[PB];
#pragma unroll
    for (int b = 0; b < PB; ++b) {
      const int i = i0 + 32 * b + lane;
      zv[b] = i < w1 ? w.zs[s + i] : 0.0;
    }
#pragma unroll
    for (int b = 0; b < PB; ++b) {
      const int i = i0 + 32 * b + lane;
      const bool big = i < w1 && rho * fabs(zv[b]) > tol;  // the test of the pass above
      const unsigned m = __ballot_sync(HSS_FULL, big);
      if (big) w.cand[s + pos + __popc(m & below)] = i;
      pos += __popc(m);
    }
  }
  __syncthreads();
  // ---- close poles deflate by Givens rotations (mdlaed2.f90:314-371).  The
  //      chain always pairs candidate t-1 with candidate t, and a rotation
  //      changes only the values of its own pair, so the test of pair t on the
  //      original values holds unless pair t-1 rotated.  All pairs are tested
  //      in parallel first (the chain's quick test: clearly above the tolerance
  //      means no rotation); one thread then runs the exact DLAED2 test on the
  //      pairs that may rotate, in order, and after every rotation on the next
  //      pair too (its left value has changed) -- the rotations, their order
  //      and the values are those of the sequential chain.  The candidates' z,
  //      d and type sit in shared memory when they fit, else in global memory.
  constexpr int NCS = 1536;
  __shared__ double c_z[NCS], c_d[NCS];
  __shared__ unsigned char c_t[NCS];
  __shared__ int c_l[NCS], c_l2[NCS];
  __shared__ int s_ng, s_nl;
  const bool in_smem = nc <= NCS;
  if (in_smem) {
    for (int t = tid; t < nc; t += MT) {
      const int pos_t = w.cand[s + t];
      c_z[t] = w.zs[s + pos_t];
      c_d[t] = w.ds[s + pos_t];
      c_t[t] = w.typ[s + pos_t];
    }
    __syncthreads();
  }
  auto zr = [&](int t) -> double & { return in_smem ? c_z[t] : w.zs[s + w.cand[s + t]]; };
  auto dr = [&](int t) -> double & { return in_smem ? c_d[t] : w.ds[s + w.cand[s + t]]; };
  auto tr = [&](int t) -> unsigned char & {
    return in_smem ? c_t[t] : w.typ[s + w.cand[s + t]];
  };
  // pairs t = 1 .. nc-1 that may rotate, compacted in order (warp segments as above)
  int *lst = w.l1slot + s;  // free until the deflated lists are written below
  {
    const int np = max(nc - 1, 0);
    const int pseg = (((np + NW - 1) / NW) + 31) & ~31;
    const int p0 = min(np, wid * pseg), p1 = min(np, p0 + pseg);
    auto maybe = [&](int t) -> bool {  // t = 1 .. nc-1, original values
      const double zp = zr(t - 1), zn = zr(t);
      const double tt = dr(t) - dr(t - 1);
      return !(fabs(tt * zn * zp) > 1.000000000001 * tol * fma(zn, zn, zp * zp));
    };
    int cntp = 0;
    for (int a0 = p0; a0 < p1; a0 += 32) {
      const int a = a0 + lane;
      cntp += __popc(__ballot_sync(HSS_FULL, a < p1 && maybe(a + 1)));
    }
    unsigned long long ptot;
    int ppos = (int)block_scan64<MT>(lane == 0 ? (unsigned long long)cntp : 0ull, &ptot);
    ppos = __shfl_sync(HSS_FULL, ppos, 0);
    for (int a0 = p0; a0 < p1; a0 += 32) {
      const int a = a0 + lane;
      const bool mb = a < p1 && maybe(a + 1);
      const unsigned mk = __ballot_sync(HSS_FULL, mb);
      if (mb) {
        const int r = ppos + __popc(mk & below);
        if ((int)ptot <= NCS) c_l[r] = a + 1; else lst[r] = a + 1;
      }
      ppos += __popc(mk);
    }
    if (tid == 0) s_nl = (int)ptot;
    __syncthreads();
  }
  if (tid == 0) {
    const int nl = s_nl;
    const int *L = nl <= NCS ? c_l : lst;
    int ng = 0, done = 0;  // pairs up to `done` have been visited
    // the exact test of pair (t-1, t) on the current values; true if it rotated
    auto visit = [&](int t) -> bool {
      const int pj = t - 1, nj = t;
      const double zp = zr(pj), zn = zr(nj);
      const double tt = dr(nj) - dr(pj);
      if (fabs(tt * zn * zp) > 1.000000000001 * tol * fma(zn, zn, zp * zp)) return false;
      const double tau = hypot(zn, zp);
      const double c = zn / tau, sn = -zp / tau;
      if (!(fabs(tt * c * sn) <= tol)) return false;
      zr(nj) = tau;
      zr(pj) = 0.0;
      if (tr(nj) != tr(pj)) tr(nj) = 2;
      tr(pj) = 5;  // deflated by rotation: value changes, order fixed below
      w.gvp[s + ng] = w.srt[s + w.cand[s + pj]];
      w.gvq[s + ng] = w.srt[s + w.cand[s + nj]];
      w.gvc[s + ng] = c;
      w.gvs[s + ng] = sn;
      ++ng;
      const double dp = dr(pj), dn = dr(nj);
      dr(pj) = dp * c * c + dn * sn * sn;
      dr(nj) = dp * sn * sn + dn * c * c;
      return true;
    };
    for (int a = 0; a < nl; ++a) {
      int t = L[a];
      if (t <= done) continue;  // already visited after a rotation
      bool rot = visit(t);
      done = t;
      while (rot && t + 1 < nc) {
        ++t;
        rot = visit(t);
        done = t;
      }
    }
    s_ng = ng;
  }
  __syncthreads();
  if (in_smem) {  // scatter the chain's results back
    for (int t = tid; t < nc; t += MT) {
      const int pos_t = w.cand[s + t];
      w.zs[s + pos_t] = c_z[t];
      w.ds[s + pos_t] = c_d[t];
      w.typ[s + pos_t] = c_t[t];
    }
    __syncthreads();
  }
  // ---- compact non-deflated (poles, weights, slots, block-structure groups)
  //      and deflated (slots, values) lists; same warp segments and ranks
  unsigned long long pk = 0;  // types 1, 2, 3 counted in 21-bit fields
  int n5 = 0;
  for (int i0 = w0; i0 < w1; i0 += 32 * PB) {
    int tv[PB];
#pragma unroll
    for (int b = 0; b < PB; ++b) {
      const int i = i0 + 32 * b + lane;
      tv[b] = i < w1 ? w.typ[s + i] : 0;
    }
#pragma unroll
    for (int b = 0; b < PB; ++b) {
      const int t = tv[b];
      pk += (unsigned long long)__popc(__ballot_sync(HSS_FULL, t == 1)) +
            ((unsigned long long)__popc(__ballot_sync(HSS_FULL, t == 2)) << 21) +
            ((unsigned long long)__popc(__ballot_sync(HSS_FULL, t == 3)) << 42);
      n5 += __popc(__ballot_sync(HSS_FULL, t == 5));
    }
  }
  unsigned long long ptot, t5;
  unsigned long long pre = block_scan64<MT>(lane == 0 ? pk : 0ull, &ptot);
  int r5 = (int)block_scan64<MT>(lane == 0 ? (unsigned long long)n5 : 0ull, &t5);
  pre = __shfl_sync(HSS_FULL, pre, 0);
  r5 = __shfl_sync(HSS_FULL, r5, 0);
  const int c1 = (int)(ptot & 0x1fffff), c2 = (int)((ptot >> 21) & 0x1fffff),
            c3 = (int)((ptot >> 42) & 0x1fffff);
  const int K = c1 + c2 + c3;
  const int nrot = (int)t5;
  int r1 = (int)(pre & 0x1fffff), r2 = (int)((pre >> 21) & 0x1fffff),
      r3 = (int)((pre >> 42) & 0x1fffff);
  for (int i0 = w0; i0 < w1; i0 += 32 * PB) {
    int tb[PB], sb[PB];
    double db[PB], zb[PB];
#pragma unroll
    for (int b = 0; b < PB; ++b) {
      const int i = i0 + 32 * b + lane;
      const bool in = i < w1;
      tb[b] = in ? w.typ[s + i] : 0;
      db[b] = in ? w.ds[s + i] : 0.0;
      zb[b] = in ? w.zs[s + i] : 0.0;
      sb[b] = in ? w.srt[s + i] : 0;
    }
#pragma unroll
    for (int b = 0; b < PB; ++b) {
    const int i = i0 + 32 * b + lane;
    const bool in = i < w1;
    const int t = tb[b];
    const double dv = db[b], zv = zb[b];
    const int sv = sb[b];
    const unsigned m1 = __ballot_sync(HSS_FULL, t == 1), m2 = __ballot_sync(HSS_FULL, t == 2),
                   m3 = __ballot_sync(HSS_FULL, t == 3), m5 = __ballot_sync(HSS_FULL, t == 5);
    if (in) {
      // this position's rank among the non-deflated of each type and the rotated
      const int e1 = r1 + __popc(m1 & below), e2 = r2 + __popc(m2 & below),
                e3 = r3 + __popc(m3 & below), e5 = r5 + __popc(m5 & below);
      const int j = e1 + e2 + e3;  // non-deflated before position i
      if (t <= 3) {
        w.dl[s + j] = dv;
        w.zw[s + j] = zv;
        w.ndslot[s + j] = sv;
        w.grp[s + j] = (t == 1) ? e1 : (t == 2) ? c1 + e2 : c1 + c2 + e3;
      } else {
        const int a = i - j;  // deflated before position i
        Dp[sv] = dv;
        if (nrot == 0) {  // no rotated poles: the small-z list is the deflated list
          w.dfslot[s + a] = sv; w.dfval[s + a] = dv;
        } else if (t == 5) {
          w.l2slot[s + e5] = sv; w.l2val[s + e5] = dv;
        } else {
          const int a1 = a - e5;  // small-z deflated before position i
          w.l1slot[s + a1] = sv; w.l1val[s + a1] = dv;
        }
      }
    }
    r1 += __popc(m1); r2 += __popc(m2); r3 += __popc(m3); r5 += __popc(m5);
    }
  }
  __syncthreads();
  // The small-z list is ascending; rotated poles moved inside their gap
  // (mdlaed2.f90:340-356 inserts them in order), so sort those and merge.
  const int n1l = (n - K) - nrot;
  if (nrot > 0) {  // else the compaction wrote the deflated list directly
  // the (short) rotated list sorted in shared memory (the chain's arrays are
  // free now) and kept there for the searches of the long one
  const bool l2s = nrot <= NCS;
  const double *l2 = l2s ? c_z : w.l2val + s;
  if (l2s) {
    for (int i = tid; i < nrot; i += MT) { c_z[i] = w.l2val[s + i]; c_l[i] = w.l2slot[s + i]; }
    __syncthreads();
    if (nrot > 1) {
      block_sort_pairs(c_z, c_l, c_d, c_l2, nrot);
      for (int i = tid; i < nrot; i += MT) { w.l2val[s + i] = c_z[i]; w.l2slot[s + i] = c_l[i]; }
      __syncthreads();
    }
  } else if (nrot > 1) {
    block_sort_pairs(w.l2val + s, w.l2slot + s, w.ds + s, w.cand + s, nrot);
  }
  for (int i = tid; i < n1l; i += MT) {  // L1 element: count L2 < v
    const double v = w.l1val[s + i];
    int lo = 0, hi = nrot;
    while (lo < hi) { int md = (lo + hi) >> 1; if (l2[md] < v) lo = md + 1; else hi = md; }
    w.dfval[s + i + lo] = v; w.dfslot[s + i + lo] = w.l1slot[s + i];
  }
  for (int i = tid; i < nrot; i += MT) {  // L2 element: count L1 <= v
    const double v = w.l2val[s + i];
    int lo = 0, hi = n1l;
    while (lo < hi) { int md = (lo + hi) >> 1; if (w.l1val[s + md] <= v) lo = md + 1; else hi = md; }
    w.dfval[s + i + lo] = v; w.dfslot[s + i + lo] = w.l2slot[s + i];
  }
  }  // nrot > 0
  if (tid == 0) {
    out[5 * m] = K; out[5 * m + 1] = s_ng; out[5 * m + 2] = c1; out[5 * m + 3] = c2;
    out[5 * m + 4] = c3;
    orho[m] = rho;
  }
}

// ---- the same bookkeeping for merges of more than PCL_MIN_N positions, on a
// thread-block cluster of PCL_G CTAs per merge.  One CTA's position passes are
// bound by the memory-level parallelism of its SM (the loads of a 32768-position
// merge take ~140 us on one SM whatever its thread count), so every pass is
// split between the cluster's CTAs: each owns a contiguous range of positions
// (or of candidates), and its block-wide totals are combined with the other
// CTAs' through distributed shared memory, so every list keeps the position
// order of the one-CTA kernel.  The chain of Givens tests stays serial, on
// thread 0 of the first CTA (it visits only the pairs that may rotate), and
// the rotated list is sorted by that CTA; the results are those of
// k_merge_prepare.  Data another CTA wrote in this launch is read through L2
// (ld.global.cg); cluster barriers order the phases.  Requires PREP_FRONT (the
// merged order and z come from k_merge_front).
namespace cg = cooperative_groups;
constexpr int PCL_G = 8;
constexpr int PCL_T = 512;
constexpr int PCL_MIN_N = 8192;

// cluster-wide exclusive scan of each CTA's 64-bit total; two shared slots used
// alternately (a slot is rewritten only after the next cluster barrier)
__device__ __forceinline__ unsigned long long cl_scan(unsigned long long v,
                                                      unsigned long long *slot, int &ph,
                                                      unsigned long long *tot) {
  cg::cluster_group cl = cg::this_cluster();
  if (threadIdx.x == 0) slot[ph] = v;
  cl.sync();
  const unsigned r = cl.block_rank(), G = cl.num_blocks();
  unsigned long long base = 0, t = 0;
  for (unsigned q = 0; q < G; ++q) {
    const unsigned long long x = *cl.map_shared_rank(slot + ph, q);
    if (q < r) base += x;
    t += x;
  }
  ph ^= 1;
  *tot = t;
  return base;
}
// cluster-wide maxima of two values (one exchange)
__device__ __forceinline__ double2 cl_max2(double2 v, double2 *slot) {
  cg::cluster_group cl = cg::this_cluster();
  if (threadIdx.x == 0) *slot = v;
  cl.sync();
  double2 r = make_double2(0.0, 0.0);
  for (unsigned q = 0; q < cl.num_blocks(); ++q) {
    const double2 x = *cl.map_shared_rank(slot, q);
    r.x = fmax(r.x, x.x);
    r.y = fmax(r.y, x.y);
  }
  return r;
}

template <int MT>
__global__ void __launch_bounds__(MT)
k_merge_prepare_cl(int P, const int *__restrict__ ms, const int *__restrict__ mn,
                   const int *__restrict__ mn1, const double *__restrict__ e,
                   double *__restrict__ Dp, int *__restrict__ perm, LevelScratch w,
                   int *__restrict__ out, double *__restrict__ orho,
                   const double *__restrict__ rsrc) {
  cg::cluster_group cl = cg::this_cluster();
  const int G = (int)cl.num_blocks(), crank = (int)cl.block_rank();
  const int m = blockIdx.x / G;
  if (m >= P) return;  // whole clusters only (the grid is P * G)
  const int s = ms[m], n = mn[m], n1 = mn1[m];
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  constexpr int NW = MT / 32, PB = 4;
  const unsigned below = (1u << lane) - 1u;
  __shared__ unsigned long long s_sl[2];
  __shared__ double2 s_sd;
  __shared__ int s_ng;
  int ph = 0;
  const double rho_in = rsrc ? rsrc[m] : e[s + n1 - 1];
  // this CTA's positions, split into warp segments as in k_merge_prepare
  const int a0 = (int)((long long)n * crank / G), a1 = (int)((long long)n * (crank + 1) / G);
  const int seg = ((((a1 - a0) + NW - 1) / NW) + 31) & ~31;
  const int w0 = min(a1, a0 + wid * seg), w1 = min(a1, w0 + seg);
  // ---- maxima of |d| and |z| (mdlaed2.f90:265-267)
  double dmax = 0.0, zmax = 0.0;
  for (int i0 = w0; i0 < w1; i0 += 32 * PB) {
    double zv[PB], dv[PB];
#pragma unroll
    for (int b = 0; b < PB; ++b) {
      const int i = i0 + 32 * b + lane;
      zv[b] = i < w1 ? w.zs[s + i] : 0.0;
      dv[b] = i < w1 ? w.ds[s + i] : 0.0;
    }
#pragma unroll
    for (int b = 0; b < PB; ++b) { zmax = fmax(zmax, fabs(zv[b])); dmax = fmax(dmax, fabs(dv[b])); }
  }
  dmax = block_max<MT>(dmax);
  zmax = block_max<MT>(zmax);
  {
    const double2 mx = cl_max2(make_double2(dmax, zmax), &s_sd);
    dmax = mx.x;
    zmax = mx.y;
  }
  const double rho = fabs(2.0 * rho_in);
  const double tol = 8.0 * HSS_EPS * fmax(dmax, zmax);
  if (rho * zmax <= tol) {  // nothing couples the halves
    for (int i = a0 + tid; i < a1; i += MT) perm[s + i] = w.srt[s + i];
    if (crank == 0 && tid == 0) {
      out[5 * m] = 0; out[5 * m + 1] = 0; out[5 * m + 2] = 0; out[5 * m + 3] = 0;
      out[5 * m + 4] = 0;
      orho[m] = rho;
    }
    cl.sync();
    return;
  }
  // ---- candidates (deflation by small z, mdlaed2.f90:304-313), in position order
  int cnt = 0;
  for (int i0 = w0; i0 < w1; i0 += 32 * PB) {
    double zv[PB];
#pragma unroll
    for (int b = 0; b < PB; ++b) {
      const int i = i0 + 32 * b + lane;
      zv[b] = i < w1 ? w.zs[s + i] : 0.0;
    }
#pragma unroll
    for (int b = 0; b < PB; ++b) {
      const int i = i0 + 32 * b + lane;
      const bool in = i < w1;
      const bool big = in && rho * fabs(zv[b]) > tol;
      if (in && !big) w.typ[s + i] = 4;
      cnt += __popc(__ballot_sync(HSS_FULL, big));
    }
  }
  unsigned long long tot, ctot;
  int pos = (int)block_scan64<MT>(lane == 0 ? (unsigned long long)cnt : 0ull, &tot);
  pos = __shfl_sync(HSS_FULL, pos, 0) + (int)cl_scan(tot, s_sl, ph, &ctot);
  const int nc = (int)ctot;
  for (int i0 = w0; i0 < w1; i0 += 32 * PB) {
    double zv[PB];
#pragma unroll
    for (int b = 0; b < PB; ++b) {
      const int i = i0 + 32 * b + lane;
      zv[b] = i < w1 ? w.zs[s + i] : 0.0;
    }
#pragma unroll
    for (int b = 0; b < PB; ++b) {
      const int i = i0 + 32 * b + lane;
      const bool big = i < w1 && rho * fabs(zv[b]) > tol;
      const unsigned mk = __ballot_sync(HSS_FULL, big);
      if (big) w.cand[s + pos + __popc(mk & below)] = i;
      pos += __popc(mk);
    }
  }
  cl.sync();  // every candidate written
  // ---- pairs t = 1 .. nc-1 that may rotate (the chain's quick test on the
  //      original values), compacted in order into l1slot (free until the
  //      deflated lists are written)
  int *lst = w.l1slot + s;
  auto cz = [&](int t) { return w.zs[s + __ldcg(w.cand + s + t)]; };
  auto cd = [&](int t) { return w.ds[s + __ldcg(w.cand + s + t)]; };
  {
    const int np = max(nc - 1, 0);
    const int b0 = (int)((long long)np * crank / G), b1 = (int)((long long)np * (crank + 1) / G);
    const int pseg = ((((b1 - b0) + NW - 1) / NW) + 31) & ~31;
    const int p0 = min(b1, b0 + wid * pseg), p1 = min(b1, p0 + pseg);
    auto maybe = [&](int t) -> bool {
      const double zp = cz(t - 1), zn = cz(t);
      const double tt = cd(t) - cd(t - 1);
      return !(fabs(tt * zn * zp) > 1.000000000001 * tol * fma(zn, zn, zp * zp));
    };
    int cntp = 0;
    for (int q0 = p0; q0 < p1; q0 += 32) {
      const int a = q0 + lane;
      cntp += __popc(__ballot_sync(HSS_FULL, a < p1 && maybe(a + 1)));
    }
    unsigned long long ptot, pctot;
    int ppos = (int)block_scan64<MT>(lane == 0 ? (unsigned long long)cntp : 0ull, &ptot);
    ppos = __shfl_sync(HSS_FULL, ppos, 0) + (int)cl_scan(ptot, s_sl, ph, &pctot);
    for (int q0 = p0; q0 < p1; q0 += 32) {
      const int a = q0 + lane;
      const bool mb = a < p1 && maybe(a + 1);
      const unsigned mk = __ballot_sync(HSS_FULL, mb);
      if (mb) lst[ppos + __popc(mk & below)] = a + 1;
      ppos += __popc(mk);
    }
    if (tid == 0) s_ng = (int)pctot;  // the list's length, until the chain sets ng
  }
  cl.sync();  // the pair list complete
  // ---- the chain (mdlaed2.f90:314-371) on thread 0 of the first CTA
  if (crank == 0 && tid == 0) {
    const int nl = s_ng;
    auto zr = [&](int t) -> double & { return w.zs[s + __ldcg(w.cand + s + t)]; };
    auto dr = [&](int t) -> double & { return w.ds[s + __ldcg(w.cand + s + t)]; };
    auto tr = [&](int t) -> unsigned char & { return w.typ[s + __ldcg(w.cand + s + t)]; };
    int ng = 0, done = 0;
    auto visit = [&](int t) -> bool {
      const int pj = t - 1, nj = t;
      const double zp = zr(pj), zn = zr(nj);
      const double tt = dr(nj) - dr(pj);
      if (fabs(tt * zn * zp) > 1.000000000001 * tol * fma(zn, zn, zp * zp)) return false;
      const double tau = hypot(zn, zp);
      const double c = zn / tau, sn = -zp / tau;
      if (!(fabs(tt * c * sn) <= tol)) return false;
      zr(nj) = tau;
      zr(pj) = 0.0;
      if (tr(nj) != tr(pj)) tr(nj) = 2;
      tr(pj) = 5;
      w.gvp[s + ng] = w.srt[s + __ldcg(w.cand + s + pj)];
      w.gvq[s + ng] = w.srt[s + __ldcg(w.cand + s + nj)];
      w.gvc[s + ng] = c;
      w.gvs[s + ng] = sn;
      ++ng;
      const double dp = dr(pj), dn = dr(nj);
      dr(pj) = dp * c * c + dn * sn * sn;
      dr(nj) = dp * sn * sn + dn * c * c;
      return true;
    };
    for (int a = 0; a < nl; ++a) {
      int t = __ldcg(lst + a);
      if (t <= done) continue;
      bool rot = visit(t);
      done = t;
      while (rot && t + 1 < nc) {
        ++t;
        rot = visit(t);
        done = t;
      }
    }
    s_ng = ng;
    __threadfence();
  }
  cl.sync();  // the chain's values and types visible
  // ---- compact non-deflated and deflated lists (reads through L2: the chain
  //      may have changed any candidate)
  unsigned long long pk = 0;
  int n5 = 0;
  for (int i0 = w0; i0 < w1; i0 += 32 * PB) {
    int tv[PB];
#pragma unroll
    for (int b = 0; b < PB; ++b) {
      const int i = i0 + 32 * b + lane;
      tv[b] = i < w1 ? __ldcg(w.typ + s + i) : 0;
    }
#pragma unroll
    for (int b = 0; b < PB; ++b) {
      const int t = tv[b];
      pk += (unsigned long long)__popc(__ballot_sync(HSS_FULL, t == 1)) +
            ((unsigned long long)__popc(__ballot_sync(HSS_FULL, t == 2)) << 21) +
            ((unsigned long long)__popc(__ballot_sync(HSS_FULL, t == 3)) << 42);
      n5 += __popc(__ballot_sync(HSS_FULL, t == 5));
    }
  }
  unsigned long long ptot, t5, cptot, ct5;
  unsigned long long pre = block_scan64<MT>(lane == 0 ? pk : 0ull, &ptot);
  int r5 = (int)block_scan64<MT>(lane == 0 ? (unsigned long long)n5 : 0ull, &t5);
  pre = __shfl_sync(HSS_FULL, pre, 0) + cl_scan(ptot, s_sl, ph, &cptot);
  r5 = __shfl_sync(HSS_FULL, r5, 0) + (int)cl_scan(t5, s_sl, ph, &ct5);
  const int c1 = (int)(cptot & 0x1fffff), c2 = (int)((cptot >> 21) & 0x1fffff),
            c3 = (int)((cptot >> 42) & 0x1fffff);
  const int K = c1 + c2 + c3;
  const int nrot = (int)ct5;
  int r1 = (int)(pre & 0x1fffff), r2 = (int)((pre >> 21) & 0x1fffff),
      r3 = (int)((pre >> 42) & 0x1fffff);
  for (int i0 = w0; i0 < w1; i0 += 32 * PB) {
    int tb[PB], sb[PB];
    double db[PB], zb[PB];
#pragma unroll
    for (int b = 0; b < PB; ++b) {
      const int i = i0 + 32 * b + lane;
      const bool in = i < w1;
      tb[b] = in ? __ldcg(w.typ + s + i) : 0;
      db[b] = in ? __ldcg(w.ds + s + i) : 0.0;
      zb[b] = in ? __ldcg(w.zs + s + i) : 0.0;
      sb[b] = in ? w.srt[s + i] : 0;
    }
#pragma unroll
    for (int b = 0; b < PB; ++b) {
      const int i = i0 + 32 * b + lane;
      const bool in = i < w1;
      const int t = tb[b];
      const unsigned m1 = __ballot_sync(HSS_FULL, t == 1), m2 = __ballot_sync(HSS_FULL, t == 2),
                     m3 = __ballot_sync(HSS_FULL, t == 3), m5 = __ballot_sync(HSS_FULL, t == 5);
      if (in) {
        const int e1 = r1 + __popc(m1 & below), e2 = r2 + __popc(m2 & below),
                  e3 = r3 + __popc(m3 & below), e5 = r5 + __popc(m5 & below);
        const int j = e1 + e2 + e3;
        if (t <= 3) {
          w.dl[s + j] = db[b];
          w.zw[s + j] = zb[b];
          w.ndslot[s + j] = sb[b];
          w.grp[s + j] = (t == 1) ? e1 : (t == 2) ? c1 + e2 : c1 + c2 + e3;
        } else {
          const int a = i - j;
          Dp[sb[b]] = db[b];
          if (nrot == 0) {  // no rotated poles: the small-z list is the deflated list
            w.dfslot[s + a] = sb[b]; w.dfval[s + a] = db[b];
          } else if (t == 5) {
            w.l2slot[s + e5] = sb[b]; w.l2val[s + e5] = db[b];
          } else {
            const int a1d = a - e5;
            w.l1slot[s + a1d] = sb[b]; w.l1val[s + a1d] = db[b];
          }
        }
      }
      r1 += __popc(m1); r2 += __popc(m2); r3 += __popc(m3); r5 += __popc(m5);
    }
  }
  cl.sync();  // the lists complete (and no CTA leaves while another reads its slots)
  const int n1l = (n - K) - nrot;
  if (nrot > 0) {  // uniform: nrot is the cluster's count
  // ---- the rotated list sorted by the first CTA (usually short)
  if (crank == 0 && nrot > 1) {
    constexpr int NCS = 1536;
    __shared__ double c_v[NCS], c_tv[NCS];
    __shared__ int c_p[NCS], c_tp[NCS];
    if (nrot <= NCS) {
      for (int i = tid; i < nrot; i += MT) { c_v[i] = __ldcg(w.l2val + s + i); c_p[i] = __ldcg(w.l2slot + s + i); }
      __syncthreads();
      block_sort_pairs(c_v, c_p, c_tv, c_tp, nrot);
      for (int i = tid; i < nrot; i += MT) { w.l2val[s + i] = c_v[i]; w.l2slot[s + i] = c_p[i]; }
    } else {
      block_sort_pairs(w.l2val + s, w.l2slot + s, w.ds + s, w.cand + s, nrot);
    }
    __threadfence();
  }
  if (nrot > 1) cl.sync();  // the sorted rotated list visible
  // ---- merge the two deflated lists (mdlaed2.f90:340-356), split between CTAs
  {
    const int q0 = (int)((long long)n1l * crank / G), q1 = (int)((long long)n1l * (crank + 1) / G);
    for (int i = q0 + tid; i < q1; i += MT) {  // L1 element: count L2 < v
      const double v = __ldcg(w.l1val + s + i);
      int lo = 0, hi = nrot;
      while (lo < hi) { int md = (lo + hi) >> 1; if (__ldcg(w.l2val + s + md) < v) lo = md + 1; else hi = md; }
      w.dfval[s + i + lo] = v; w.dfslot[s + i + lo] = __ldcg(w.l1slot + s + i);
    }
    const int u0 = (int)((long long)nrot * crank / G), u1 = (int)((long long)nrot * (crank + 1) / G);
    for (int i = u0 + tid; i < u1; i += MT) {  // L2 element: count L1 <= v
      const double v = __ldcg(w.l2val + s + i);
      int lo = 0, hi = n1l;
      while (lo < hi) { int md = (lo + hi) >> 1; if (__ldcg(w.l1val + s + md) <= v) lo = md + 1; else hi = md; }
      w.dfval[s + i + lo] = v; w.dfslot[s + i + lo] = __ldcg(w.l2slot + s + i);
    }
  }
  }  // nrot > 0
  if (crank == 0 && tid == 0) {
    out[5 * m] = K; out[5 * m + 1] = s_ng; out[5 * m + 2] = c1; out[5 * m + 3] = c2;
    out[5 * m + 4] = c3;
    orho[m] = rho;
  }
}

// Apply each merge's Givens rotations, in order, to its slot pairs: one thread
// per row (rows of a block are independent; columns are read coalesced).
// Front half of the prepare for all merges of a level, one thread per
// position (positions of merge m: poff[m] .. poff[m+1]-1): the merged order of
// the two ascending halves (DLAMRG by merge path: each element counts the
// partner half's values below it) and z in merged order, as k_merge_prepare
// would compute them with one CTA per merge.
__global__ void k_merge_front(int P, const int *__restrict__ poff, const int *__restrict__ ms,
                              const int *__restrict__ mn, const int *__restrict__ mn1,
                              const double *__restrict__ e, const double *__restrict__ Q,
                              long long ldq, const double *__restrict__ Dp,
                              const int *__restrict__ perm, LevelScratch w,
                              const double *__restrict__ zsrc, const double *__restrict__ rsrc,
                              int flags, const int2 *__restrict__ sup) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= poff[P]) return;
  int lo = 0, hi = P;
  while (hi - lo > 1) { const int md = (lo + hi) >> 1; if (poff[md] <= t) lo = md; else hi = md; }
  const int m = lo, i = t - poff[m];
  const int s = ms[m], n1 = mn1[m], n2 = mn[m] - n1;
  const bool top = i < n1;
  const int slot = perm[s + i];  // left: perm[s+i]; right: perm[s+n1+(i-n1)]
  const double v = Dp[slot];
  int a = 0, b = top ? n2 : n1;
  const int base = top ? s + n1 : s;
  while (a < b) {  // top: count right values < v;  bottom: count left values <= v
    const int md = (a + b) >> 1;
    const double u = Dp[perm[base + md]];
    if (top ? (u < v) : (u <= v)) a = md + 1; else b = md;
  }
  const int pos = (top ? i : i - n1) + a;
  const double rho_in = rsrc ? rsrc[m] : e[s + n1 - 1];
  double z = zsrc ? zsrc[slot] : qat(Q, ldq, sup, slot, top ? s + n1 - 1 : s + n1);
  if (!top && rho_in < 0.0) z = -z;
  w.srt[s + pos] = slot;
  w.ds[s + pos] = v;
  w.zs[s + pos] = z * (1.0 / sqrt(2.0));
  w.typ[s + pos] = (flags & PREP_DENSE) ? 2 : top ? 1 : 3;
}

// Before the deflating rotations of merge m: every column they touch is made
// valid on all rows s .. s+n-1 of the merge (zeros written outside the rows it
// held data on) and its support widened, so the rotations read true values.
// One CTA per merge, rotations in order (a slot may take part in several).
__global__ void k_widen(int P, const int *__restrict__ ms, const int *__restrict__ mn,
                        const int *__restrict__ ng, const LevelScratch w, double *Q, long long ldq,
                        int2 *__restrict__ sup) {
  for (int m = blockIdx.x; m < P; m += gridDim.x) {
    const int s = ms[m], n = mn[m], g = ng[m];
    for (int t = 0; t < g; ++t)
      for (int side = 0; side < 2; ++side) {
        const int slot = side == 0 ? w.gvp[s + t] : w.gvq[s + t];
        __syncthreads();  // the previous update of sup is visible to all threads
        const int2 r = sup[slot];
        if (r.x == s && r.y == s + n) continue;  // uniform across the CTA
        double *col = Q + (long long)slot * ldq;
        for (int i = s + threadIdx.x; i < s + n; i += blockDim.x)
          if (i < r.x || i >= r.y) col[i] = 0.0;
        __syncthreads();
        if (threadIdx.x == 0) sup[slot] = make_int2(s, s + n);
      }
    __syncthreads();
  }
}

// Threads r >= n rotate rows p, q of column r - n of Zr (nz columns, leading
// dim zld) the same way: the remaining columns of a banded merge's
// Z = Q^T W follow the rotated eigenvectors (mdsbed22.f90 rotates Z(:, 2:)).
__global__ void k_givens(int P, const int *__restrict__ ms, const int *__restrict__ mn,
                         const int *__restrict__ ng, const LevelScratch w, double *Q,
                         long long ldq, double *Zr, int nz, long long zld) {
  for (int m = blockIdx.y; m < P; m += gridDim.y) {
    const int s = ms[m], n = mn[m], g = ng[m];
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n + nz || g == 0) continue;
    double *base;
    long long ld, row;
    if (r < n) { base = Q; ld = ldq; row = s + r; }
    else { base = Zr + (r - n) * zld; ld = 1; row = 0; }
    for (int t = 0; t < g; ++t) {
      const long long p = w.gvp[s + t], q = w.gvq[s + t];
      const double c = w.gvc[s + t], sn = w.gvs[s + t];
      const double x = base[p * ld + row], y = base[q * ld + row];
      base[p * ld + row] = c * x + sn * y;
      base[q * ld + row] = c * y - sn * x;
    }
  }
}

// Copy the K non-deflated columns of merge m into a dense n_m x K buffer
// (column `grp` when grouped, else column j).  One CTA per (column, row chunk).
// One warp per (column, segment of GS_SEG rows), lanes along the rows: the
// bottom levels have many short columns (a CTA per column would schedule
// hundreds of thousands of blocks that copy a few dozen values each).
constexpr int GS_SEG = 256;

__device__ __forceinline__ int gs_merge(const int *__restrict__ rootoff, int P, int r) {
  int lo = 0, hi = P;
  while (hi - lo > 1) { int mid = (lo + hi) >> 1; if (rootoff[mid] <= r) lo = mid; else hi = mid; }
  return lo;
}

__global__ void k_gather(int P, int nseg, const int *__restrict__ ms, const int *__restrict__ mn,
                         const int *__restrict__ rootoff, const int *__restrict__ ndslot,
                         const int *__restrict__ grp, const long long *__restrict__ boff,
                         const double *__restrict__ Q, long long ldq, double *__restrict__ B,
                         const int2 *__restrict__ sup) {
  const long long wg = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int r = (int)(wg / nseg), q = (int)(wg - (long long)r * nseg);
  if (r >= rootoff[P]) return;
  const int m = gs_merge(rootoff, P, r), j = r - rootoff[m];
  const int s = ms[m], n = mn[m];
  const int i0 = q * GS_SEG, i1 = min(n, i0 + GS_SEG);
  if (i0 >= i1) return;
  const int col = grp ? grp[s + j] : j;
  const int slot = ndslot[s + j];
  const double *src = Q + (long long)slot * ldq + s;
  double *dst = B + boff[m] + (long long)col * n;
  int vlo = 0, vhi = n;  // rows of the column that hold data (zero elsewhere)
  if (sup) { const int2 sr = sup[slot]; vlo = max(0, sr.x - s); vhi = min(n, sr.y - s); }
  for (int i = i0 + lane; i < i1; i += 32) dst[i] = (i >= vlo && i < vhi) ? src[i] : 0.0;
}

// Write the new eigenvectors (columns of T, n_m x K) into the non-deflated slots.
__global__ void k_scatter(int P, int nseg, const int *__restrict__ ms, const int *__restrict__ mn,
                          const int *__restrict__ rootoff, const int *__restrict__ ndslot,
                          const long long *__restrict__ toff, const double *__restrict__ T,
                          double *__restrict__ Q, long long ldq, int2 *__restrict__ sup) {
  const long long wg = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int r = (int)(wg / nseg), q = (int)(wg - (long long)r * nseg);
  if (r >= rootoff[P]) return;
  const int m = gs_merge(rootoff, P, r), j = r - rootoff[m];
  const int s = ms[m], n = mn[m];
  const int i0 = q * GS_SEG, i1 = min(n, i0 + GS_SEG);
  if (i0 >= i1) return;
  const double *src = T + toff[m] + (long long)j * n;
  double *dst = Q + (long long)ndslot[s + j] * ldq + s;
  if (sup && q == 0 && lane == 0) sup[ndslot[s + j]] = make_int2(s, s + n);
  for (int i = i0 + lane; i < i1; i += 32) dst[i] = src[i];
}

// New ascending order of each merged block: roots (ascending) merged with the
// deflated eigenvalues (ascending), roots first on ties (DLAMRG at
// mdlaed1.f90:221); eigenvalues of the rewritten slots are set to the roots.
template <int MT>
__global__ void __launch_bounds__(MT)
k_merge_finish(int P, const int *__restrict__ ms, const int *__restrict__ mn,
               const int *__restrict__ mK, const double *__restrict__ lam,
               const LevelScratch w, int *__restrict__ perm, double *__restrict__ Dp) {
  constexpr int LS = 2048;
  __shared__ double sl[LS];
  const int m = blockIdx.x;
  const int s = ms[m], n = mn[m], K = mK[m];
  const int nd = n - K;
  // the (short) list of new eigenvalues in shared memory for the searches of
  // the long deflated list
  const bool in_s = K <= LS;
  if (in_s) {
    for (int j = threadIdx.x; j < K; j += MT) sl[j] = lam[s + j];
    __syncthreads();
  }
  const double *lm = in_s ? sl : lam + s;
  for (int j = threadIdx.x; j < K; j += MT) {
    const double a = lm[j];
    int lo = 0, hi = nd;
    while (lo < hi) { int mid = (lo + hi) >> 1; if (w.dfval[s + mid] < a) lo = mid + 1; else hi = mid; }
    const int slot = w.ndslot[s + j];
    perm[s + j + lo] = slot;
    Dp[slot] = a;
  }
  for (int a_ = threadIdx.x; a_ < nd; a_ += MT) {
    const double b = w.dfval[s + a_];
    int lo = 0, hi = K;
    while (lo < hi) { int mid = (lo + hi) >> 1; if (lm[mid] <= b) lo = mid + 1; else hi = mid; }
    perm[s + a_ + lo] = w.dfslot[s + a_];
  }
}

// The finish of all merges of a level with one thread per position
// (positions of merge m: poff[m] .. poff[m+1]-1, its first K[m] the new roots):
// the same ascending order as k_merge_finish, without one CTA per merge
// serialising the top levels.
__global__ void k_merge_finish_grid(int P, const int *__restrict__ poff, const int *__restrict__ ms,
                                    const int *__restrict__ mK, const double *__restrict__ lam,
                                    const LevelScratch w, int *__restrict__ perm,
                                    double *__restrict__ Dp) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= poff[P]) return;
  int lo = 0, hi = P;
  while (hi - lo > 1) { const int md = (lo + hi) >> 1; if (poff[md] <= t) lo = md; else hi = md; }
  const int m = lo, i = t - poff[m];
  const int s = ms[m], K = mK[m], nd = poff[m + 1] - poff[m] - K;
  if (i < K) {  // new root: count deflated values below it
    const double a = lam[s + i];
    int a0 = 0, b0 = nd;
    while (a0 < b0) { const int md = (a0 + b0) >> 1; if (w.dfval[s + md] < a) a0 = md + 1; else b0 = md; }
    const int slot = w.ndslot[s + i];
    perm[s + i + a0] = slot;
    Dp[slot] = a;
  } else {      // deflated: count roots at or below it
    const int j = i - K;
    const double b = w.dfval[s + j];
    int a0 = 0, b0 = K;
    while (a0 < b0) { const int md = (a0 + b0) >> 1; if (lam[s + md] <= b) a0 = md + 1; else b0 = md; }
    perm[s + j + a0] = w.dfslot[s + j];
  }
}

// Final column permutation (mdlaed0.f90:355-362): Z(:, i) = Q(:, perm(i)),
// w(i) = Dp(perm(i)).  One CTA per column.
__global__ void k_final_gather(int n, const int *__restrict__ perm, const double *__restrict__ Dp,
                               const double *__restrict__ Q, long long ldq, double *__restrict__ Z,
                               long long ldz, double *__restrict__ wout,
                               const int2 *__restrict__ sup) {
  const int c = blockIdx.x;
  if (c >= n) return;
  const long long p = perm[c];
  if (sup) {  // read only the rows the column holds data on; zeros elsewhere
    const int2 r = sup[p];
    const double *s1 = Q + p * ldq;
    double *dst = Z + (long long)c * ldz;
    for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = (i >= r.x && i < r.y) ? s1[i] : 0.0;
    if (threadIdx.x == 0) wout[c] = Dp[p];
    return;
  }
  const double2 *src = reinterpret_cast<const double2 *>(Q + p * ldq);
  double *dst = Z + (long long)c * ldz;
  // 16-byte vector copies only when both column starts are 16-byte aligned
  if ((((uintptr_t)(Q + p * ldq) | (uintptr_t)dst) & 15) == 0 && (n % 2 == 0)) {
    double2 *d2 = reinterpret_cast<double2 *>(dst);
    for (int i = threadIdx.x; i < n / 2; i += blockDim.x) d2[i] = src[i];
  } else {
    const double *s1 = Q + p * ldq;
    for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = s1[i];
  }
  if (threadIdx.x == 0) wout[c] = Dp[p];
}

// Packed form of the final permutation for host outputs: output column c
// (slot perm[c]) holds data only on rows sup[slot] = [x, y); those rows go to
// out[off[c] ..] back to back (off: prefix sum of y - x, computed on the host
// from the same sup), w(c) = Dp(perm(c)).  One CTA per column.
__global__ void k_pack_columns(int n, const int *__restrict__ perm, const double *__restrict__ Dp,
                               const double *__restrict__ Q, long long ldq,
                               const int2 *__restrict__ sup, const long long *__restrict__ off,
                               double *__restrict__ out, double *__restrict__ wout) {
  const int c = blockIdx.x;
  if (c >= n) return;
  const long long p = perm[c];
  const int2 r = sup[p];
  const double *src = Q + p * ldq;
  double *dst = out + off[c];
  for (int i = r.x + threadIdx.x; i < r.y; i += blockDim.x) dst[i - r.x] = src[i];
  if (threadIdx.x == 0) wout[c] = Dp[p];
}

// COMPZ = 'V': the packed columns (output order, column c at soff[c] with
// soff[c+1] - soff[c] rows) rewritten in the order of `order` (dst column j =
// source column order[j], at doff[j]), so that columns sharing a support
// segment sit back to back as one dense m x k operand.  One CTA per column.
__global__ void k_repack_columns(int n, const int *__restrict__ order,
                                 const long long *__restrict__ soff,
                                 const long long *__restrict__ doff,
                                 const double *__restrict__ src, double *__restrict__ dst) {
  const int j = blockIdx.x;
  if (j >= n) return;
  const int c = order[j];
  const long long s = soff[c], len = soff[c + 1] - soff[c], d = doff[j];
  for (long long i = threadIdx.x; i < len; i += blockDim.x) dst[d + i] = src[s + i];
}

// out(:, order[j]) = T(:, j) for j < n, rows 0..m-1 (T leading dimension ldt,
// out ldo): the products of the support groups put back in output order.
// Grid (n columns, row chunks of 2048); 16 bytes per element.
__global__ void k_scatter_columns(int n, int m, const int *__restrict__ order,
                                  const double *__restrict__ T, long long ldt,
                                  double *__restrict__ out, long long ldo) {
  const int j = blockIdx.x;
  if (j >= n) return;
  const double *src = T + (long long)j * ldt;
  double *dst = out + (long long)order[j] * ldo;
  const int r0 = blockIdx.y * 2048, r1 = min(m, r0 + 2048);
  for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) dst[i] = src[i];
}

// ------------------------------------------------ many problems per call --
// Problems of one call sit at global positions P[p] .. P[p+1]-1 and share one
// Q with leading dimension ldq >= max n_p: problem p's eigenvector block is the
// column-major n_p x n_p matrix at Q + P[p] * (ldq + 1) with leading dim ldq,
// so every level kernel addresses it with global positions unchanged.

__device__ __forceinline__ int problem_of(const long long *__restrict__ P, int np, long long c) {
  int lo = 0, hi = np - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(P + mid) <= c) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Zero the diagonal blocks of all problems (one CTA per global column).
__global__ void k_zero_blocks(int np, const long long *__restrict__ P, double *__restrict__ Q,
                              long long ldq) {
  const long long c = blockIdx.x;
  const int p = problem_of(P, np, c);
  const long long r0 = __ldg(P + p), n = __ldg(P + p + 1) - r0;
  double *col = Q + c * ldq + r0;
  for (long long i = threadIdx.x; i < n; i += blockDim.x) col[i] = 0.0;
}

// Undo the per-block scaling of the eigenvalues: block b covers positions
// bs[b] .. bs[b] + bm[b] - 1 (slots of Dp).
__global__ void k_scale_blocks(int nb, const int *__restrict__ bs, const int *__restrict__ bm,
                               const double *__restrict__ bscl, double *__restrict__ Dp) {
  for (int b = blockIdx.y; b < nb; b += gridDim.y) {
    const int s = bs[b], m = bm[b];
    const double a = bscl[b];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x)
      Dp[s + i] *= a;
  }
}

// Final ordering of every problem: column j of problem p's output is the
// global slot perm[P[p] + j]; its eigenvalue is Dp[slot].  Z[p], W[p] are the
// per-problem output pointers, ldz[p] their leading dimensions.
__global__ void k_final_gather_batch(int np, const long long *__restrict__ P,
                                     const int *__restrict__ perm, const double *__restrict__ Dp,
                                     const double *__restrict__ Q, long long ldq,
                                     double *const *__restrict__ Z, const long long *__restrict__ ldz,
                                     double *const *__restrict__ W, const int2 *__restrict__ sup) {
  const long long c = blockIdx.x;
  const int p = problem_of(P, np, c);
  const long long r0 = __ldg(P + p), n = __ldg(P + p + 1) - r0, j = c - r0;
  const long long slot = perm[c];
  const double *src = Q + slot * ldq + r0;
  double *dst = Z[p] + j * ldz[p];
  long long lo = 0, hi = n;  // rows holding data (global rows sup[slot]) relative to r0
  if (sup) { const int2 r = sup[slot]; lo = r.x - r0; hi = r.y - r0; }
  for (long long i = threadIdx.x; i < n; i += blockDim.x) dst[i] = (i >= lo && i < hi) ? src[i] : 0.0;
  if (threadIdx.x == 0) W[p][j] = Dp[slot];
}

// ---------------------------------------------------------------- launch --
static int merge_threads(int maxn) {
  return maxn <= 64 ? 64 : maxn <= 256 ? 128 : maxn <= 2048 ? 256 : 512;
}

void launch_merge_front(int P, int total, const int *poff, const int *ms, const int *mn,
                        const int *mn1, const double *e, const double *Q, long long ldq,
                        const double *Dp, const int *perm, const LevelScratch &w,
                        const double *zsrc, const double *rsrc, int flags, cudaStream_t st,
                        const int2 *sup) {
  if (P <= 0 || total <= 0) return;
  k_merge_front<<<(total + 255) / 256, 256, 0, st>>>(P, poff, ms, mn, mn1, e, Q, ldq, Dp, perm,
                                                     w, zsrc, rsrc, flags, sup);
}

void launch_merge_prepare(int P, int maxn, const int *ms, const int *mn, const int *mn1,
                          const double *e, const double *Q, long long ldq, double *Dp, int *perm,
                          const LevelScratch &w, int *out, double *orho, cudaStream_t st,
                          const double *zsrc, const double *rsrc, int flags, const int2 *sup) {
  if (P <= 0) return;
  if ((flags & PREP_FRONT) && maxn > PCL_MIN_N) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(P * PCL_G));
    cfg.blockDim = dim3(PCL_T);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = PCL_G;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (cudaLaunchKernelEx(&cfg, k_merge_prepare_cl<PCL_T>, P, ms, mn, mn1, e, Dp, perm, w, out,
                           orho, rsrc) == cudaSuccess)
      return;
    (void)cudaGetLastError();  // no cluster launch here: the one-CTA kernel below
  }
#define PREP_CASE(T)                                                                        \
  case T:                                                                                  \
    k_merge_prepare<T><<<P, T, 0, st>>>(P, ms, mn, mn1, e, Q, ldq, Dp, perm, w, out, orho, \
                                        zsrc, rsrc, flags, sup);                           \
    break;
  switch (merge_threads(maxn)) {
    PREP_CASE(64)
    PREP_CASE(128)
    PREP_CASE(256)
    default:
    PREP_CASE(512)
  }
#undef PREP_CASE
}
void launch_givens(int P, int maxn, const int *ms, const int *mn, const int *ng,
                   const LevelScratch &w, double *Q, long long ldq, cudaStream_t st, double *Zr,
                   int nz, long long zld) {
  if (P <= 0) return;
  if (!Zr) nz = 0;
  dim3 grid((maxn + nz + 255) / 256, std::min(P, 65535));
  k_givens<<<grid, 256, 0, st>>>(P, ms, mn, ng, w, Q, ldq, Zr, nz, zld);
}
void launch_gather(int P, int total, int maxn, const int *ms, const int *mn, const int *rootoff,
                   const int *ndslot, const int *grp, const long long *boff, const double *Q,
                   long long ldq, double *B, cudaStream_t st, const int2 *sup) {
  if (total <= 0) return;
  const int nseg = (maxn + GS_SEG - 1) / GS_SEG;
  const long long warps = (long long)total * nseg;
  k_gather<<<(unsigned)((warps + 7) / 8), 256, 0, st>>>(P, nseg, ms, mn, rootoff, ndslot, grp, boff,
                                                        Q, ldq, B, sup);
}
void launch_scatter(int P, int total, int maxn, const int *ms, const int *mn, const int *rootoff,
                    const int *ndslot, const long long *toff, const double *T, double *Q,
                    long long ldq, cudaStream_t st, int2 *sup) {
  if (total <= 0) return;
  const int nseg = (maxn + GS_SEG - 1) / GS_SEG;
  const long long warps = (long long)total * nseg;
  k_scatter<<<(unsigned)((warps + 7) / 8), 256, 0, st>>>(P, nseg, ms, mn, rootoff, ndslot, toff, T,
                                                         Q, ldq, sup);
}
void launch_widen(int P, int maxn, const int *ms, const int *mn, const int *ng,
                  const LevelScratch &w, double *Q, long long ldq, int2 *sup, cudaStream_t st) {
  if (P <= 0 || !sup) return;
  k_widen<<<std::min(P, 65535), maxn <= 256 ? 128 : 512, 0, st>>>(P, ms, mn, ng, w, Q, ldq, sup);
}
void launch_merge_finish(int P, int maxn, const int *ms, const int *mn, const int *mK,
                         const double *lam, const LevelScratch &w, int *perm, double *Dp,
                         cudaStream_t st) {
  if (P <= 0) return;
  switch (merge_threads(maxn)) {
    case 64: k_merge_finish<64><<<P, 64, 0, st>>>(P, ms, mn, mK, lam, w, perm, Dp); break;
    case 128: k_merge_finish<128><<<P, 128, 0, st>>>(P, ms, mn, mK, lam, w, perm, Dp); break;
    case 256: k_merge_finish<256><<<P, 256, 0, st>>>(P, ms, mn, mK, lam, w, perm, Dp); break;
    default: k_merge_finish<512><<<P, 512, 0, st>>>(P, ms, mn, mK, lam, w, perm, Dp); break;
  }
}
void launch_merge_finish_grid(int P, int total, const int *poff, const int *ms, const int *mK,
                              const double *lam, const LevelScratch &w, int *perm, double *Dp,
                              cudaStream_t st) {
  if (P > 0 && total > 0)
    k_merge_finish_grid<<<(total + 255) / 256, 256, 0, st>>>(P, poff, ms, mK, lam, w, perm, Dp);
}
void launch_final_gather(int n, const int *perm, const double *Dp, const double *Q, long long ldq,
                         double *Z, long long ldz, double *wout, cudaStream_t st,
                         const int2 *sup) {
  if (n > 0) k_final_gather<<<n, 256, 0, st>>>(n, perm, Dp, Q, ldq, Z, ldz, wout, sup);
}
void launch_pack_columns(int n, const int *perm, const double *Dp, const double *Q, long long ldq,
                         const int2 *sup, const long long *off, double *out, double *wout,
                         cudaStream_t st) {
  if (n > 0) k_pack_columns<<<n, 128, 0, st>>>(n, perm, Dp, Q, ldq, sup, off, out, wout);
}
void launch_repack_columns(int n, const int *order, const long long *soff, const long long *doff,
                           const double *src, double *dst, cudaStream_t st) {
  if (n > 0) k_repack_columns<<<n, 128, 0, st>>>(n, order, soff, doff, src, dst);
}
void launch_scatter_columns(int n, int m, const int *order, const double *T, long long ldt,
                            double *out, long long ldo, cudaStream_t st) {
  if (n > 0 && m > 0)
    k_scatter_columns<<<dim3(n, (m + 2047) / 2048), 256, 0, st>>>(n, m, order, T, ldt, out, ldo);
}
void launch_zero_blocks(int np, long long total, const long long *P, double *Q, long long ldq,
                        cudaStream_t st) {
  if (np > 0 && total > 0) k_zero_blocks<<<(unsigned)total, 256, 0, st>>>(np, P, Q, ldq);
}
void launch_scale_blocks(int nb, const int *bs, const int *bm, const double *bscl, double *Dp,
                         cudaStream_t st) {
  if (nb > 0) k_scale_blocks<<<dim3(64, std::min(nb, 65535)), 256, 0, st>>>(nb, bs, bm, bscl, Dp);
}
void launch_final_gather_batch(int np, long long total, const long long *P, const int *perm,
                               const double *Dp, const double *Q, long long ldq, double *const *Z,
                               const long long *ldz, double *const *W, cudaStream_t st,
                               const int2 *sup) {
  if (np > 0 && total > 0)
    k_final_gather_batch<<<(unsigned)total, 256, 0, st>>>(np, P, perm, Dp, Q, ldq, Z, ldz, W,
                                                          sup);
}

}  // namespace hss
