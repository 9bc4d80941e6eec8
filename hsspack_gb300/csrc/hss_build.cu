// hss_build.cu -- HSS compression of the Cauchy-like eigenvector matrix and the
// fast HSS multiply on sm_103a (DHSSEVC, SRC/CauchyHssEig.f90:2444-2598).
//
//   C(i,j) = u_i v_j / (F_i - lam_j),  lam_j = F_j + DIFL_j,   K x K
//
// Construction (Cauchy2hssEig_omp, :1945-2250) walks the HSS tree bottom-up.
// At each level every node compresses its block row against all other
// current columns, then its block column against all other current rows, by
// a structured strong rank-revealing LU that only touches the O(M + N)
// generators (rrluCauchyEig{row,col}, :7-467).  One CTA owns one node; all
// nodes of a level run in one launch.  The node's own generators live in
// shared memory, the "other side" generators (length up to K) in a private
// global scratch slice that stays L2-resident.  Pivot searches are block-wide
// argmax reductions with Fortran MAXLOC tie-breaking; every pivot decision is
// FP64.  After each half-level a single-CTA kernel compacts the surviving
// skeleton generators in the reference's order (:2140-2166, :2196-2227).
//
// Multiply (fastHssmmL_omp, SRC/ConstructHssd.f90:1394-1630): X (n x K) times
// the HSS matrix, as grouped GEMMs per tree level: upsweep G = X U, sibling
// products F = G B, downsweep F V, leaves Y = X D + F V.
#include <algorithm>
#include <climits>
#include <cstring>
#include <vector>

#include <cooperative_groups.h>

#include "hss_common.cuh"
#include "hss_gemm.h"
#include "hss_hss.h"
#include "hss_plan.h"
#include "hss_kernels.h"
#include "hss_pool.h"
#include "../../include/hsspack_gb300.h"

namespace hss {

namespace cg = cooperative_groups;

#define HCK(x)                                                                              \
  do {                                                                                      \
    cudaError_t e_ = (x);                                                                   \
    if (e_ != cudaSuccess) throw HssError{std::string(#x) + ": " + cudaGetErrorString(e_)}; \
  } while (0)

constexpr int HT = 256;        // threads per node CTA
constexpr int HSS_RMIN = 256;  // rank capacity floor

// ------------------------------------------------------------- host tree --
static void perfect_tree(int n, int off, std::vector<int> &par) {
  if (n == 1) { par[off + 1] = 0; return; }
  int h = (n - 1) / 2;
  perfect_tree(h, off, par);
  perfect_tree(h, off + h, par);
  par[off + h] = off + n; par[off + 2 * h] = off + n; par[off + n] = 0;
}
static void n2tree(int n, int off, std::vector<int> &par) {
  if (n == 1) { par[off + 1] = 0; return; }
  int p2 = 1;
  while (p2 * 2 <= n) p2 *= 2;
  int n1 = p2 - 1;
  perfect_tree(n1, off, par);
  n2tree(n - n1 - 1, off + n1, par);
  par[off + n1] = off + n; par[off + n - 1] = off + n; par[off + n] = 0;
}

HostTree make_tree(int K, int ni) {
  HostTree t;
  int lm = K / ni, mr = K % ni;
  if (lm == 0) { lm = 1; t.m.assign(1, K); }
  else {
    t.m.assign(lm, ni);
    if (mr >= ni / 2) { t.m.push_back(mr); ++lm; } else t.m[lm - 1] += mr;
  }
  t.lm = lm;
  t.ltr = 2 * lm - 1;
  t.parent.assign(t.ltr + 1, 0);
  n2tree(t.ltr, 0, t.parent);
  t.c1.assign(t.ltr + 1, 0); t.c2.assign(t.ltr + 1, 0);
  for (int i = 1; i < t.ltr; ++i) {
    int p = t.parent[i];
    if (t.c1[p] == 0) t.c1[p] = i; else t.c2[p] = i;
  }
  t.depth.assign(t.ltr + 1, 0);
  for (int i = t.ltr - 1; i >= 1; --i) t.depth[i] = t.depth[t.parent[i]] + 1;
  int lvl = 0, p = 1;
  while (p < t.ltr + 1) { p *= 2; ++lvl; }
  t.lvl = lvl - 1;
  t.ttr.assign(t.lvl + 1, {});
  for (int j = 1; j < t.ltr; ++j) t.ttr[t.depth[j]].push_back(j);
  t.leafstart.assign(t.ltr + 1, 0);
  for (int i = 1, acc = 0, it = 0; i <= t.ltr; ++i)
    if (t.leaf(i)) { t.leafstart[i] = acc; acc += t.m[it++]; }
  t.mmax = *std::max_element(t.m.begin(), t.m.end());
  return t;
}

// ------------------------------------------------------- device helpers --
__device__ __forceinline__ ArgMax block_argmax(ArgMax a, ArgMax *red) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  a = warp_argmax(a);
  __syncthreads();
  if (lane == 0) red[w] = a;
  __syncthreads();
  ArgMax r = red[0];
  for (int i = 1; i < (int)(blockDim.x >> 5); ++i) r = argmax_merge(r, red[i]);
  return r;
}

__device__ __forceinline__ double warp_prod(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v *= __shfl_xor_sync(HSS_FULL, v, o);
  return v;
}

// ---- cluster cooperation of one node's RRLU --------------------------------
// A node's RRLU may run on a cluster of G CTAs (G = 1, 2, 4, 8): every CTA holds
// the same node-side arrays in its shared memory and repeats the node-side work
// identically; the other-side positions (the long side, up to K) are split
// between the CTAs, their partial argmaxes combined through distributed shared
// memory, and swaps of other-side entries done by rank 0 between cluster
// barriers.  Other-side entries are read through L2 (ld.global.cg) so that a
// CTA never sees a stale L1 copy of an entry another CTA of the cluster wrote.
struct ArgMax3 {
  double v;
  int i;  // position (first wins on ties)
  int a;  // auxiliary index carried with the winner
};

__device__ __forceinline__ void csync(int G) {
  if (G > 1) cg::this_cluster().sync();
  else __syncthreads();
}

// the cluster-wide best of each CTA's (value, position, aux), identical in every
// CTA; slot: two shared slots used alternately (a slot is rewritten only after
// the next cluster barrier, by which time every CTA has read it)
__device__ __forceinline__ ArgMax3 cluster_best(ArgMax3 x, int G, ArgMax3 *slot, int &phase) {
  if (G == 1) return x;
  cg::cluster_group cl = cg::this_cluster();
  if (threadIdx.x == 0) slot[phase] = x;
  cl.sync();
  ArgMax3 r{-1.0, INT_MAX, 0};
  for (int q = 0; q < G; ++q) {
    const ArgMax3 y = *cl.map_shared_rank(slot + phase, q);
    if (y.v > r.v || (y.v == r.v && y.i < r.i)) r = y;
  }
  phase ^= 1;
  return r;
}

// Structured strong RRLU of one node (row or column case).  Node side (length
// M) in shared memory, other side (length N) in global scratch.  The scans and
// generator updates over the N other-side entries are FP64-pipe bound, so their
// divides go through qdiv (within 1.5 ulp); the pivot values and the generator
// entries written out use correctly rounded divides.
//   ROW:  C(i,j) = A_i V_j / (F_{PL_i} - lam_{PU_j})
//   COL:  C(i,j) = A_i V_j / (lam_{PL_i} - F_{PU_j})
// Returns Rk; on exit A/PL/F are permuted, Z holds the Schur row generators,
// W the column generators of the interpolation block, PQ the row permutation.
// G, crank: the cluster size and this CTA's rank in it (1, 0 without a cluster).
template <bool ROW>
__device__ int rrlu_node(const PoleDiff &P, double *F, double *A, double *Z, double *W, int *PL,
                         int *PQ, double *V, int *PU, int M, int N, double tol, int rmax,
                         int *overflow, int *nswap, double rho, int G, int crank) {
  __shared__ ArgMax red[HT / 32];
  __shared__ ArgMax3 cslot[2];
  __shared__ int s_rk;
  int cphase = 0;
  const int tid = threadIdx.x;
  const int jstep = G * HT, joff = crank * HT;  // this CTA's share of the other side
  auto Vr = [&](int j) -> double { return __ldcg(V + j); };
  auto PUr = [&](int j) -> int { return __ldcg(PU + j); };
  // row poles: ROW -> F values (old poles); COL -> lam values (index PL)
  auto den = [&](int pl, int pu) -> double {  // C denominator for pole indices
    return ROW ? P.fd(pl, pu) : -P.fd(pu, pl);
  };
  auto rowdiff = [&](int i, int j) -> double {  // row pole i minus row pole j
    return ROW ? P.fv(F[i], F[j]) : P.dd(PL[i], PL[j]);
  };
  for (int i = tid; i < M; i += HT) { Z[i] = A[i]; PQ[i] = i; }
  if (tid == 0) s_rk = -1;
  __syncthreads();
  const int mn = min(M, N);
  double Amax = 0.0;
  auto colmax = [&](int k) -> int {
    ArgMax a{-1.0, INT_MAX};
    const int puk = PUr(k);
    for (int i = k + tid; i < M; i += HT) {
      const double t = fabs(qdiv(Z[i], den(PL[i], puk)));
      if (t > a.v) { a.v = t; a.i = i; }
    }
    a = block_argmax(a, red);
    return a.i == INT_MAX ? k : a.i;
  };
  auto colmax_v = [&](int k, int &arg) -> double {
    ArgMax a{-1.0, INT_MAX};
    const int puk = PUr(k);
    for (int i = k + tid; i < M; i += HT) {
      const double t = fabs(qdiv(Z[i], den(PL[i], puk)));
      if (t > a.v) { a.v = t; a.i = i; }
    }
    a = block_argmax(a, red);
    arg = a.i == INT_MAX ? k : a.i;
    return a.v;
  };
  auto rowmax_v = [&](int k, int &arg) -> double {
    ArgMax a{-1.0, INT_MAX};
    for (int j = k + joff + tid; j < N; j += jstep) {
      const double t = fabs(qdiv(Vr(j), den(PL[k], PUr(j))));
      if (t > a.v) { a.v = t; a.i = j; }
    }
    a = block_argmax(a, red);
    const ArgMax3 c = cluster_best(ArgMax3{a.v, a.i, 0}, G, cslot, cphase);
    arg = c.i == INT_MAX ? k : c.i;
    return c.v;
  };
  auto swap_row = [&](int a, int b) {
    __syncthreads();
    if (tid == 0 && a != b) {
      double t; int ti;
      t = F[a]; F[a] = F[b]; F[b] = t;
      t = Z[a]; Z[a] = Z[b]; Z[b] = t;
      t = A[a]; A[a] = A[b]; A[b] = t;
      ti = PL[a]; PL[a] = PL[b]; PL[b] = ti;
      ti = PQ[a]; PQ[a] = PQ[b]; PQ[b] = ti;
    }
    __syncthreads();
  };
  auto swap_col = [&](int a, int b) {
    csync(G);
    if (crank == 0 && tid == 0 && a != b) {
      const double t = Vr(a); V[a] = Vr(b); V[b] = t;
      const int ti = PUr(a); PU[a] = PUr(b); PU[b] = ti;
    }
    csync(G);
  };
  int Rk = mn;
  // the other-side update pass of step k also finds row k+1's maximum over the
  // updated entries (the scan step k+1 would start with), unless a strong swap
  // changes the rows or entries in between
  bool have_next = false;
  ArgMax next_best{-1.0, INT_MAX};
  for (int k = 0; k < mn; ++k) {
    if (k >= rmax) {  // would exceed the generator capacity
      if (tid == 0 && crank == 0) atomicOr(overflow, 1);
      Rk = k;
      break;
    }
    {  // Gu's variant of complete pivoting (CauchyPivtEig, :571-680)
      int jl, ju;
      double jkL = colmax_v(k, jl);
      double jkU;
      if (have_next) {  // row k's maximum was found during step k-1's update pass
        const ArgMax3 c = cluster_best(ArgMax3{next_best.v, next_best.i, 0}, G, cslot, cphase);
        ju = c.i == INT_MAX ? k : c.i;
        jkU = c.v;
      } else {
        jkU = rowmax_v(k, ju);
      }
      have_next = false;
      jkL *= fabs(Vr(k));
      jkU *= fabs(Z[k]);
      const double piv = fabs(Z[k] * Vr(k) / den(PL[k], PUr(k)));
      if (!(jkL <= piv && jkU <= piv)) {
        bool fromcol = jkL > jkU;
        for (int guard = 0; guard < 4 * (M + N) + 8; ++guard) {
          if (fromcol) {
            swap_row(k, jl);
            rowmax_v(k, ju);
            if (ju == k) break;
            fromcol = false;
          }
          swap_col(k, ju);
          jl = colmax(k);
          if (jl == k) break;
          fromcol = true;
        }
      }
    }
    __syncthreads();
    double Ukk = Z[k] * Vr(k) / den(PL[k], PUr(k));
    Amax = fmax(Amax, fabs(Ukk));
    if (fabs(Ukk) < tol * Amax) {
      // complete pivoting over the Schur complement (CauchyPivtEig_CP)
      ArgMax best{-1.0, INT_MAX};
      int bi_loc = k;
      for (int j = k + joff + tid; j < N; j += jstep) {
        double cm = -1.0;
        int a = k;
        const int puj = PUr(j);
        for (int i = k; i < M; ++i) {
          const double t = fabs(qdiv(Z[i], den(PL[i], puj)));
          if (t > cm) { cm = t; a = i; }
        }
        const double t = fabs(cm * Vr(j));
        if (t > best.v) { best.v = t; best.i = j; bi_loc = a; }
      }
      __shared__ int s_bi;
      ArgMax r = block_argmax(best, red);
      if (tid == 0 && r.i == INT_MAX) s_bi = k;
      __syncthreads();
      if (r.i != INT_MAX && best.i == r.i && best.v == r.v) s_bi = bi_loc;
      __syncthreads();
      const ArgMax3 c = cluster_best(ArgMax3{r.v, r.i, s_bi}, G, cslot, cphase);
      const int bj = c.i == INT_MAX ? k : c.i;
      const int bi = c.i == INT_MAX ? k : c.a;
      swap_row(k, bi);
      swap_col(k, bj);
      Ukk = Z[k] * Vr(k) / den(PL[k], PUr(k));
      Amax = fmax(Amax, fabs(Ukk));
      if (fabs(Ukk) < tol * Amax) { Rk = k; break; }
    }
    // Schur-complement generator updates
    const double Fk = ROW ? F[k] : 0.0;
    const int puk = PUr(k);
    for (int j = k + 1 + tid; j < M; j += HT)
      Z[j] *= qdiv(rowdiff(j, k), den(PL[j], puk));
    const bool fuse = k + 1 < mn && k + 1 < M;
    const int pln = fuse ? PL[k + 1] : 0;
    ArgMax nb{-1.0, INT_MAX};
    for (int j = k + 1 + joff + tid; j < N; j += jstep) {
      const int puj = PUr(j);
      const double vj = Vr(j) * (ROW ? qdiv(P.dd(puj, puk), -P.fd(PL[k], puj))
                                     : qdiv(P.fv(__ldg(P.F + puj), __ldg(P.F + puk)), P.fd(puj, PL[k])));
      V[j] = vj;
      if (fuse) {  // |C(k+1, j)| / |A(k+1)| of the next step's Schur complement
        const double t = fabs(qdiv(vj, den(pln, puj)));
        if (t > nb.v) { nb.v = t; nb.i = j; }
      }
    }
    if (fuse) {
      next_best = block_argmax(nb, red);
      have_next = true;
    }
    for (int j = tid; j < k; j += HT)
      W[j] *= ROW ? qdiv(-P.fd(PL[j], puk), P.fv(Fk, F[j]))
                  : qdiv(P.fd(puk, PL[j]), P.dd(PL[k], PL[j]));
    if (tid < 32) {  // W[k] = den(k,k)/A[k] * prod_{j<k} ...
      double pr = 1.0;
      for (int j = tid; j < k; j += 32) {
        const int puj = PUr(j);
        pr *= ROW ? (-P.fd(PL[k], puj)) / P.fv(F[j], Fk) : P.fd(puj, PL[k]) / P.dd(PL[j], PL[k]);
      }
      pr = warp_prod(pr);
      if (tid == 0) W[k] = (den(PL[k], puk) / A[k]) * pr;
    }
    csync(G);  // every CTA reads the updated V[k+1] next
    // strong swaps every 10 steps when an interpolation entry exceeds rho
    // (searchMax2Eig[m] with rho = 1.5, CauchyHssEig.f90:98-99; searchMax2 with
    // rho = 1.02 for generic Cauchy matrices, CauchyHss_VP2.f90:70-71)
    if ((k + 1) % 10 == 0) {
      for (int guard = 0; guard < M + 8; ++guard) {
        ArgMax best{-1.0, INT_MAX};
        int ii_loc = 0;
        for (int j = tid; j <= k; j += HT) {
          double cm = -1.0;
          int a = k + 1;
          for (int i = k + 1; i < M; ++i) {
            const double t = fabs(qdiv(Z[i], rowdiff(i, j)));
            if (t > cm) { cm = t; a = i; }
          }
          const double t = cm * fabs(W[j]);
          if (t > best.v) { best.v = t; best.i = j; ii_loc = a; }
        }
        __shared__ int s_jj;
        ArgMax r = block_argmax(best, red);
        if (tid == 0) s_jj = (r.i == INT_MAX) ? M : -1;
        __syncthreads();
        if (r.i != INT_MAX && best.i == r.i && best.v == r.v) s_jj = ii_loc;
        __syncthreads();
        const int ii = r.i == INT_MAX ? 0 : r.i, jj = s_jj;
        if (!(r.v > rho) || jj >= M) break;
        have_next = false;  // rows and other-side entries change
        if (tid == 0 && crank == 0) atomicAdd(nswap, 1);
        for (int j = k + 1 + joff + tid; j < N; j += jstep) {
          const int puj = PUr(j);
          V[j] = Vr(j) * (ROW ? qdiv(-P.fd(PL[ii], puj), -P.fd(PL[jj], puj))
                              : qdiv(P.fd(puj, PL[ii]), P.fd(puj, PL[jj])));
        }
        double ujj = 0.0, wii = 0.0;
        if (tid < 32) {
          double pu = 1.0, pw = 1.0;
          for (int j = tid; j <= k; j += 32) {
            if (j == ii) continue;
            const int puj = PUr(j);
            if (ROW) {
              pu *= P.fv(F[ii], F[j]) / P.fd(PL[ii], puj);
              pw *= (-P.fd(PL[jj], puj)) / P.fv(F[j], F[jj]);
            } else {
              pu *= P.dd(PL[ii], PL[j]) / (-P.fd(puj, PL[ii]));
              pw *= P.fd(puj, PL[jj]) / P.dd(PL[j], PL[jj]);
            }
          }
          pu = warp_prod(pu);
          pw = warp_prod(pw);
          const int puii = PUr(ii);
          ujj = A[ii] * (rowdiff(ii, jj) / den(PL[ii], puii)) * pu;
          wii = (ROW ? P.fd(PL[jj], puii) : -P.fd(puii, PL[jj])) / A[jj] * pw;
        }
        __syncthreads();
        // Z, W updates use the pre-swap poles
        double zn[(512 + HT - 1) / HT];
        int cnt = 0;
        for (int j = k + 1 + tid; j < M; j += HT, ++cnt)
          zn[cnt] = (j != jj) ? Z[j] * (rowdiff(j, jj) / rowdiff(j, ii)) : Z[j];
        double wn = 0.0;
        if (tid <= k && tid != ii) wn = W[tid] * (rowdiff(tid, ii) / rowdiff(tid, jj));
        double wn2[(256 + HT - 1) / HT];
        int c2 = 0;
        for (int j = tid + HT; j <= k; j += HT, ++c2)
          wn2[c2] = (j != ii) ? W[j] * (rowdiff(j, ii) / rowdiff(j, jj)) : W[j];
        __syncthreads();
        cnt = 0;
        for (int j = k + 1 + tid; j < M; j += HT, ++cnt) Z[j] = zn[cnt];
        if (tid <= k && tid != ii) W[tid] = wn;
        c2 = 0;
        for (int j = tid + HT; j <= k; j += HT, ++c2) W[j] = wn2[c2];
        if (tid == 0) {
          Z[jj] = ujj;
          W[ii] = wii;
          int ti = PL[ii]; PL[ii] = PL[jj]; PL[jj] = ti;
          ti = PQ[ii]; PQ[ii] = PQ[jj]; PQ[jj] = ti;
          double t = F[ii]; F[ii] = F[jj]; F[jj] = t;
          t = A[ii]; A[ii] = A[jj]; A[jj] = t;
        }
        __syncthreads();
      }
      csync(G);  // the swaps' other-side updates before the next step's scans
    }
  }
  // no CTA leaves while another may still read its shared slots
  if (G > 1) csync(G);
  return Rk;
}

// Row compression of every node of one level: node block row against all
// other current columns (ComprcauchyEig 'r', :2338-2380).
constexpr int MMAXS = 512;  // max rows of a node handled in shared memory

__global__ void __launch_bounds__(HT)
k_hss_rows(HssDev h, const int *__restrict__ nodes, int nn, double tol, int csz) {
  __shared__ double F[MMAXS], A[MMAXS], Z[MMAXS], W[MMAXS];
  __shared__ int PL[MMAXS], PQ[MMAXS], INV[MMAXS];
  const int a = blockIdx.x / csz;  // the node; a cluster of G CTAs shares it
  const int crank = csz > 1 ? (int)cg::this_cluster().block_rank() : 0;
  if (a >= nn) return;
  const int node = nodes[a];
  const int tid = threadIdx.x;
  const int r0 = h.lr0[node], M = h.lr1[node] - r0 + 1;
  const int c0 = h.lc0[node], nc = h.lc1[node] - c0 + 1;
  const int lca = *h.lca, N = lca - nc;
  if (M > MMAXS) { if (tid == 0) atomicOr(h.flag, 2); return; }
  double *V = h.oval + (long long)a * h.K;
  int *PU = h.oidx + (long long)a * h.K;
  for (int j = crank * HT + tid; j < lca; j += csz * HT) {  // this CTA's share of the copy
    if (j < c0) { V[j] = h.V[j]; PU[j] = h.PU[j]; }
    else if (j > h.lc1[node]) { V[j - nc] = h.V[j]; PU[j - nc] = h.PU[j]; }
  }
  for (int i = tid; i < M; i += HT) {
    A[i] = h.U[r0 + i];
    PL[i] = h.PL[r0 + i];
    F[i] = h.FF[PL[i]];
    W[i] = 0.0;
  }
  csync(csz);
  PoleDiff P{h.FF, h.DIFL, h.DIFR, h.sq};
  int Rk = rrlu_node<true>(P, F, A, Z, W, PL, PQ, V, PU, M, N, tol, h.rmax, h.flag, h.flag + 1,
                           h.rho, csz, crank);
  if (crank != 0) return;  // rank 0 writes the node's results
  __syncthreads();
  for (int i = tid; i < M; i += HT) { h.U[r0 + i] = A[i]; h.PL[r0 + i] = PL[i]; INV[PQ[i]] = i; }
  __syncthreads();
  const int mn = min(M, N);
  double *G = h.Ug + (long long)node * h.ucap;
  if (Rk < (h.vp2 ? M : mn)) {
    for (int idx = tid; idx < M * Rk; idx += HT) {
      const int r = idx % M, j = idx / M, p = INV[r];
      G[idx] = (p < Rk) ? (p == j ? 1.0 : 0.0) : Z[p] * W[j] / P.fv(F[p], F[j]);
    }
  } else {
    Rk = M;
    if ((long long)M * M > h.ucap) { if (tid == 0) atomicOr(h.flag, 1); Rk = 0; }
    else
      for (int idx = tid; idx < M * M; idx += HT) {
        const int r = idx % M, j = idx / M;
        G[idx] = (INV[r] == j) ? 1.0 : 0.0;
      }
  }
  if (tid == 0) { h.Ur[node] = M; h.Uc[node] = Rk; }
}

// Column compression: node block column against all other current rows
// (ComprcauchyEig 'c', :2382-2430).  The transposed block has the node's
// roots as row poles.
__global__ void __launch_bounds__(HT)
k_hss_cols(HssDev h, const int *__restrict__ nodes, int nn, double tol, int csz) {
  __shared__ double F[MMAXS], A[MMAXS], Z[MMAXS], W[MMAXS];
  __shared__ int PL[MMAXS], PQ[MMAXS], INV[MMAXS];
  const int a = blockIdx.x / csz;  // the node; a cluster of G CTAs shares it
  const int crank = csz > 1 ? (int)cg::this_cluster().block_rank() : 0;
  if (a >= nn) return;
  const int node = nodes[a];
  const int tid = threadIdx.x;
  const int c0 = h.lc0[node], M = h.lc1[node] - c0 + 1;  // node columns
  const int r0 = h.lr0[node], nr = h.lr1[node] - r0 + 1;
  const int lda = *h.lda, N = lda - nr;
  if (M > MMAXS) { if (tid == 0) atomicOr(h.flag, 2); return; }
  double *V = h.oval + (long long)a * h.K;
  int *PU = h.oidx + (long long)a * h.K;
  for (int j = crank * HT + tid; j < lda; j += csz * HT) {  // this CTA's share of the copy
    if (j < r0) { V[j] = h.U[j]; PU[j] = h.PL[j]; }
    else if (j > h.lr1[node]) { V[j - nr] = h.U[j]; PU[j - nr] = h.PL[j]; }
  }
  for (int i = tid; i < M; i += HT) {
    A[i] = h.V[c0 + i];
    PL[i] = h.PU[c0 + i];
    F[i] = 0.0;
    W[i] = 0.0;
  }
  csync(csz);
  PoleDiff P{h.FF, h.DIFL, h.DIFR, h.sq};
  int Rk = rrlu_node<false>(P, F, A, Z, W, PL, PQ, V, PU, M, N, tol, h.rmax, h.flag, h.flag + 1,
                            h.rho, csz, crank);
  if (crank != 0) return;  // rank 0 writes the node's results
  __syncthreads();
  for (int i = tid; i < M; i += HT) { h.V[c0 + i] = A[i]; h.PU[c0 + i] = PL[i]; INV[PQ[i]] = i; }
  __syncthreads();
  const int mn = min(M, N);
  double *G = h.Vg + (long long)node * h.vcap;
  if (Rk < (h.vp2 ? M : mn)) {
    for (int idx = tid; idx < Rk * M; idx += HT) {
      const int i = idx % Rk, c = idx / Rk, p = INV[c];
      G[idx] = (p < Rk) ? (p == i ? 1.0 : 0.0) : -W[i] * Z[p] / P.dd(PL[i], PL[p]);
    }
  } else {
    Rk = M;
    if ((long long)M * M > h.vcap) { if (tid == 0) atomicOr(h.flag, 1); Rk = 0; }
    else
      for (int idx = tid; idx < M * M; idx += HT) {
        const int i = idx % M, c = idx / M;
        G[idx] = (INV[c] == i) ? 1.0 : 0.0;
      }
  }
  if (tid == 0) { h.Vr[node] = Rk; h.Vc[node] = M; }
}

// Compact the surviving generators: skeletons of this level's nodes (in level
// order), then the untouched leaves of the levels above (deepest first).
// rows = true: U/PL/lr, else V/PU/lc.  Also sets the ranges of the parents at
// the next level up once both halves are compacted.
__global__ void k_hss_compact(HssDev h, const int *__restrict__ nodes, int nn,
                              const int *__restrict__ above, int na,
                              const int *__restrict__ parents, int np, int rows) {
  __shared__ int off[1024 + 1];
  const int tid = threadIdx.x;
  int *r0 = rows ? h.lr0 : h.lc0, *r1 = rows ? h.lr1 : h.lc1;
  const int *rk = rows ? h.Uc : h.Vr;
  double *val = rows ? h.U : h.V, *tval = rows ? h.Ut : h.Vt;
  int *idx = rows ? h.PL : h.PU, *tidx = rows ? h.PLt : h.PUt;
  const int tot = nn + na;
  if (tid == 0) {
    int acc = 0;
    for (int a = 0; a < tot; ++a) {
      off[a] = acc;
      const int node = a < nn ? nodes[a] : above[a - nn];
      acc += a < nn ? rk[node] : (r1[node] - r0[node] + 1);
    }
    off[tot] = acc;
  }
  __syncthreads();
  for (int a = 0; a < tot; ++a) {
    const int node = a < nn ? nodes[a] : above[a - nn];
    const int len = off[a + 1] - off[a], src = r0[node];
    for (int i = tid; i < len; i += blockDim.x) {
      tval[off[a] + i] = val[src + i];
      tidx[off[a] + i] = idx[src + i];
    }
  }
  __syncthreads();
  const int total = off[tot];
  for (int i = tid; i < total; i += blockDim.x) { val[i] = tval[i]; idx[i] = tidx[i]; }
  __syncthreads();
  if (tid == 0) {
    for (int a = 0; a < tot; ++a) {
      const int node = a < nn ? nodes[a] : above[a - nn];
      r0[node] = off[a];
      r1[node] = off[a + 1] - 1;
    }
    if (rows) *h.lda = total; else *h.lca = total;
  }
  __syncthreads();
  if (!rows && tid == 0) {  // parents of the next level up: union of children
    for (int a = 0; a < np; ++a) {
      // parents[] lists (parent, child1, child2) triples
      const int p = parents[3 * a], x = parents[3 * a + 1], y = parents[3 * a + 2];
      h.lr0[p] = h.lr0[x]; h.lr1[p] = h.lr1[y];
      h.lc0[p] = h.lc0[x]; h.lc1[p] = h.lc1[y];
    }
  }
}

// B generator of each node: skeleton rows of the node x skeleton columns of
// its sibling (CauchyHssEig.f90:2230-2244).
__global__ void k_hss_B(HssDev h, const int *__restrict__ pairs, int nn) {
  const int a = blockIdx.x;
  if (a >= nn) return;
  const int node = pairs[2 * a], sib = pairs[2 * a + 1];
  const int r0 = h.lr0[node], m = h.lr1[node] - r0 + 1;
  const int c0 = h.lc0[sib], n = h.lc1[sib] - c0 + 1;
  PoleDiff P{h.FF, h.DIFL, h.DIFR, h.sq};
  double *B = h.Bg + (long long)node * h.bcap;
  if ((long long)m * n > h.bcap) { if (threadIdx.x == 0) atomicOr(h.flag, 1); return; }
  for (int idx = threadIdx.x; idx < m * n; idx += blockDim.x) {
    const int i = idx % m, j = idx / m;
    B[idx] = h.U[r0 + i] * h.V[c0 + j] / P.fd(h.PL[r0 + i], h.PU[c0 + j]);
  }
  if (threadIdx.x == 0) { h.Br[node] = m; h.Bc[node] = n; }
}

// Leaf diagonal blocks from the original generators (CauchylikeEig, :2089-2100).
__global__ void k_hss_leafD(HssDev h, const int *__restrict__ leaves, const int *__restrict__ lstart,
                            const int *__restrict__ lsize, int nl, const double *__restrict__ u,
                            const double *__restrict__ v) {
  for (int a = blockIdx.y; a < nl; a += gridDim.y) {
    const int node = leaves[a], s = lstart[a], m = lsize[a];
    PoleDiff P{h.FF, h.DIFL, h.DIFR, h.sq};
    double *D = h.Dg + h.doff[a];
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < m * m; idx += gridDim.x * blockDim.x) {
      const int i = idx % m, j = idx / m;
      D[idx] = u[s + i] * v[s + j] / P.fd(s + i, s + j);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) h.Dm[node] = m;
  }
}

__global__ void k_init_gens(int K, const double *__restrict__ u, const double *__restrict__ v,
                            double *U, double *V, int *PL, int *PU) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < K) { U[i] = u[i]; V[i] = v[i]; PL[i] = i; PU[i] = i; }
}

// --------------------------------------------------------------- host ----
// CTAs per node of a level (a thread-block cluster): doubled while the level
// stays within HSS_CLUSTER_CTAS CTAs, up to a portable cluster of 8.  Levels of
// 8 nodes or fewer run one CTA per node: their other side (the skeletons of the
// remaining nodes) is short, and the cluster barriers of every pivot step cost
// more than the split scans save (measured on the 8192-point Cauchy merge).
constexpr int HSS_CLUSTER_MAX = 8;
constexpr int HSS_CLUSTER_CTAS = 304;  // two CTAs per SM
static int hss_cluster_size(int nn) {
  int G = 1;
  if (nn <= 8) return 1;
  while (G < HSS_CLUSTER_MAX && (long long)nn * G * 2 <= HSS_CLUSTER_CTAS) G *= 2;
  return G;
}

static void launch_node_rrlu(void (*kern)(HssDev, const int *, int, double, int),
                             const HssDev &h, const int *dn, int nn, double tol,
                             cudaStream_t st) {
  const int G = hss_cluster_size(nn);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(nn * G));
  cfg.blockDim = dim3(HT);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)G;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  HCK(cudaLaunchKernelEx(&cfg, kern, h, dn, nn, tol, G));
}
template <class T>
static T *up(const char *name, const std::vector<T> &v, cudaStream_t st) {
  T *d = pool<T>(name, std::max<size_t>(v.size(), 1));
  if (!v.empty()) stage_h2d(d, v.data(), v.size() * sizeof(T), st);
  return d;
}

// Build the HSS generators on the device; on return the ranks are on the host.
static int hss_construct(HssPlan &pl, int K, int ni, double tol, const double *F, const double *u,
                         const double *v, const double *difl, const double *difr, cudaStream_t st,
                         bool sq = false, double rho = 1.5, bool vp2 = false) {
  int launches = 0;
  pl.t = make_tree(K, ni);
  const HostTree &t = pl.t;
  const int ltr = t.ltr;
  const int rmax = std::max(HSS_RMIN, t.mmax);
  HssDev &h = pl.h;
  h.FF = F; h.DIFL = difl; h.DIFR = difr; h.sq = sq;
  h.K = K; h.ltr = ltr; h.rmax = rmax; h.rho = rho; h.vp2 = vp2;
  h.U = pool<double>("hs_U", K); h.V = pool<double>("hs_V", K);
  h.PL = pool<int>("hs_PL", K); h.PU = pool<int>("hs_PU", K);
  h.Ut = pool<double>("hs_Ut", K); h.Vt = pool<double>("hs_Vt", K);
  h.PLt = pool<int>("hs_PLt", K); h.PUt = pool<int>("hs_PUt", K);
  int *ints = pool<int>("hs_ints", (size_t)11 * (ltr + 1) + 8);
  HCK(cudaMemsetAsync(ints, 0, sizeof(int) * ((size_t)11 * (ltr + 1) + 8), st));
  int *q = ints;
  h.lr0 = q; q += ltr + 1; h.lr1 = q; q += ltr + 1; h.lc0 = q; q += ltr + 1; h.lc1 = q; q += ltr + 1;
  h.Ur = q; q += ltr + 1; h.Uc = q; q += ltr + 1; h.Vr = q; q += ltr + 1; h.Vc = q; q += ltr + 1;
  h.Br = q; q += ltr + 1; h.Bc = q; q += ltr + 1; h.Dm = q; q += ltr + 1;
  h.lda = q; h.lca = q + 1; h.flag = q + 2;
  const long long rows_cap = std::max(t.mmax, 2 * rmax);
  h.ucap = rows_cap * rmax;
  h.vcap = rows_cap * rmax;
  h.bcap = (long long)rmax * rmax;
  h.Ug = pool<double>("hs_Ug", (size_t)(ltr + 1) * h.ucap);
  h.Vg = pool<double>("hs_Vg", (size_t)(ltr + 1) * h.vcap);
  h.Bg = pool<double>("hs_Bg", (size_t)(ltr + 1) * h.bcap);
  size_t maxlev = 1;
  for (int L = 1; L <= t.lvl; ++L) maxlev = std::max(maxlev, t.ttr[L].size());
  h.oval = pool<double>("hs_oval", maxlev * K);
  h.oidx = pool<int>("hs_oidx", maxlev * K);
  // leaf ranges, diagonal blocks
  std::vector<int> lr0(ltr + 1, 0), lr1(ltr + 1, -1), leaves, lstart, lsize;
  std::vector<long long> doff;
  long long dtot = 0;
  for (int i = 1, it = 0; i <= ltr; ++i)
    if (t.leaf(i)) {
      lr0[i] = t.leafstart[i]; lr1[i] = t.leafstart[i] + t.m[it] - 1;
      leaves.push_back(i); lstart.push_back(t.leafstart[i]); lsize.push_back(t.m[it]);
      doff.push_back(dtot); dtot += (long long)t.m[it] * t.m[it];
      ++it;
    }
  pl.doff = doff;
  h.Dg = pool<double>("hs_Dg", dtot);
  h.doff = up("hs_doff", doff, st);
  HCK(cudaMemcpyAsync(h.lr0, lr0.data(), sizeof(int) * (ltr + 1), cudaMemcpyHostToDevice, st));
  HCK(cudaMemcpyAsync(h.lr1, lr1.data(), sizeof(int) * (ltr + 1), cudaMemcpyHostToDevice, st));
  HCK(cudaMemcpyAsync(h.lc0, lr0.data(), sizeof(int) * (ltr + 1), cudaMemcpyHostToDevice, st));
  HCK(cudaMemcpyAsync(h.lc1, lr1.data(), sizeof(int) * (ltr + 1), cudaMemcpyHostToDevice, st));
  int kk[2] = {K, K};
  HCK(cudaMemcpyAsync(h.lda, kk, sizeof kk, cudaMemcpyHostToDevice, st));
  k_init_gens<<<(K + 255) / 256, 256, 0, st>>>(K, u, v, h.U, h.V, h.PL, h.PU);
  int *dleaves = up("hs_leaves", leaves, st), *dls = up("hs_ls", lstart, st),
      *dlz = up("hs_lz", lsize, st);
  {
    dim3 g((t.mmax * t.mmax + 255) / 256, (unsigned)std::min<size_t>(leaves.size(), 65535));
    k_hss_leafD<<<g, 256, 0, st>>>(h, dleaves, dls, dlz, (int)leaves.size(), u, v);
  }
  launches += 2;
  // per level node lists (processing order)
  for (int LL = t.lvl; LL >= 1; --LL) {
    const std::vector<int> &nodes = t.ttr[LL];
    std::vector<int> above, parents, pairs;
    for (int LLt = LL - 1; LLt >= 1; --LLt)
      for (int nd : t.ttr[LLt])
        if (t.leaf(nd)) above.push_back(nd);
    if (LL > 1)
      for (int nd : t.ttr[LL - 1])
        if (!t.leaf(nd)) { parents.push_back(nd); parents.push_back(t.c1[nd]); parents.push_back(t.c2[nd]); }
    for (int nd : nodes) { pairs.push_back(nd); pairs.push_back(t.sibling(nd)); }
    if (nodes.size() + above.size() > 1024) throw HssError{"HSS tree too wide"};
    char nm[32];
    snprintf(nm, sizeof nm, "hs_nodes%d", LL);
    int *dn = up(nm, nodes, st);
    snprintf(nm, sizeof nm, "hs_above%d", LL);
    int *da = up(nm, above, st);
    snprintf(nm, sizeof nm, "hs_par%d", LL);
    int *dp = up(nm, parents, st);
    snprintf(nm, sizeof nm, "hs_pairs%d", LL);
    int *dpr = up(nm, pairs, st);
    const int nn = (int)nodes.size();
    launch_node_rrlu(k_hss_rows, h, dn, nn, tol, st);
    k_hss_compact<<<1, 512, 0, st>>>(h, dn, nn, da, (int)above.size(), dp, 0, 1);
    launch_node_rrlu(k_hss_cols, h, dn, nn, tol, st);
    k_hss_compact<<<1, 512, 0, st>>>(h, dn, nn, da, (int)above.size(), dp, (int)parents.size() / 3, 0);
    k_hss_B<<<nn, 256, 0, st>>>(h, dpr, nn);
    launches += 5;
  }
  // ranks and dims to the host (one sync per HSS merge)
  std::vector<int> hint((size_t)11 * (ltr + 1) + 8);
  HCK(cudaMemcpyAsync(hint.data(), ints, sizeof(int) * hint.size(), cudaMemcpyDeviceToHost, st));
  HCK(cudaStreamSynchronize(st));
  auto seg = [&](int k) { return std::vector<int>(hint.begin() + (size_t)k * (ltr + 1), hint.begin() + (size_t)(k + 1) * (ltr + 1)); };
  pl.Ur = seg(4); pl.Uc = seg(5); pl.Vr = seg(6); pl.Vc = seg(7); pl.Br = seg(8); pl.Bc = seg(9); pl.Dm = seg(10);
  const int flag = hint[(size_t)11 * (ltr + 1) + 2];
  pl.ok = (flag == 0);
  for (int i = 1; i < ltr; ++i) pl.max_rank = std::max(pl.max_rank, std::max(pl.Uc[i], pl.Vr[i]));
  return launches;
}

// Y (nrows x K, ldy) = X (nrows x K, ldx) * H, FP64 grouped GEMMs per level.
int hss_multiply(const HssPlan &pl, const double *X, long long ldx, int nrows, double *Y,
                 long long ldy, int precision, cudaStream_t st, double *flops, long long *bytes) {
  const HostTree &t = pl.t;
  const HssDev &h = pl.h;
  const int ltr = t.ltr;
  int launches = 0;
  auto launch = [&](std::vector<GemmDesc> &probs, const char *name) {
    (void)name;
    if (probs.empty()) return;
    for (auto &p : probs) {
      if (flops) *flops += 2.0 * p.M * p.N * p.K;
      if (bytes) *bytes += 8LL * ((long long)p.M * p.K + (long long)p.K * p.N + (long long)p.M * p.N);
    }
    launch_gemm(probs, precision, st);
    launches += precision ? 3 : 1;
  };
  if (t.lm == 1) {
    std::vector<GemmDesc> p{{X, h.Dg, Y, (int)ldx, pl.Dm[ltr], (int)ldy, nrows, pl.Dm[ltr], pl.Dm[ltr], 0, 0}};
    launch(p, "hm_p0");
    return launches;
  }
  std::vector<long long> lg(ltr + 1, 0), lf(ltr + 1, 0);
  long long ncg = 0, ncf = 0;
  for (int LL = t.lvl; LL >= 1; --LL)
    for (int nd : t.ttr[LL]) { lg[nd] = ncg; ncg += pl.Uc[nd]; }
  for (int LL = 1; LL <= t.lvl; ++LL)
    for (int nd : t.ttr[LL]) { lf[nd] = ncf; ncf += pl.Bc[t.sibling(nd)]; }
  double *G = pool<double>("hm_G", (size_t)nrows * std::max<long long>(ncg, 1));
  double *Fm = pool<double>("hm_F", (size_t)nrows * std::max<long long>(ncf, 1));
  auto Ug = [&](int nd) { return h.Ug + (long long)nd * h.ucap; };
  auto Vg = [&](int nd) { return h.Vg + (long long)nd * h.vcap; };
  auto Bg = [&](int nd) { return h.Bg + (long long)nd * h.bcap; };
  // upsweep
  for (int LL = t.lvl; LL >= 1; --LL) {
    std::vector<GemmDesc> probs;
    for (int nd : t.ttr[LL]) {
      if (pl.Uc[nd] == 0) continue;
      const double *A = t.leaf(nd) ? X + (long long)t.leafstart[nd] * ldx : G + lg[t.c1[nd]] * nrows;
      const int lda = t.leaf(nd) ? (int)ldx : nrows;
      probs.push_back({A, Ug(nd), G + lg[nd] * nrows, lda, pl.Ur[nd], nrows, nrows, pl.Uc[nd],
                       pl.Ur[nd], 0, 0});
    }
    char nm[24];
    snprintf(nm, sizeof nm, "hm_up%d", LL);
    launch(probs, nm);
  }
  // downsweep: F_i (+)= G_sib B_sib ; F_children = F_i V_i
  for (int LL = 1; LL <= t.lvl; ++LL) {
    std::vector<GemmDesc> pb, pv;
    for (int nd : t.ttr[LL]) {
      const int sb = t.sibling(nd);
      pb.push_back({G + lg[sb] * nrows, Bg(sb), Fm + lf[nd] * nrows, nrows, std::max(pl.Br[sb], 1),
                    nrows, nrows, pl.Bc[sb], pl.Br[sb], LL == 1 ? 0 : 1, 0});
      if (!t.leaf(nd))
        pv.push_back({Fm + lf[nd] * nrows, Vg(nd), Fm + lf[t.c1[nd]] * nrows, nrows,
                      std::max(pl.Vr[nd], 1), nrows, nrows, pl.Vc[nd], pl.Vr[nd], 0, 0});
    }
    char nm[24];
    snprintf(nm, sizeof nm, "hm_b%d", LL);
    launch(pb, nm);
    snprintf(nm, sizeof nm, "hm_v%d", LL);
    launch(pv, nm);
  }
  // leaves: Y_i = X_i D_i, then Y_i += F_i V_i
  std::vector<GemmDesc> pd, pf;
  int li = 0;
  for (int nd = 1; nd < ltr; ++nd) {
    if (!t.leaf(nd)) continue;
    const int m = pl.Dm[nd];
    const long long c0 = t.leafstart[nd];
    pd.push_back({X + c0 * ldx, h.Dg + pl.doff[li], Y + c0 * ldy, (int)ldx, m, (int)ldy, nrows, m, m,
                  0, 0});
    pf.push_back({Fm + lf[nd] * nrows, Vg(nd), Y + c0 * ldy, nrows, std::max(pl.Vr[nd], 1), (int)ldy,
                  nrows, pl.Vc[nd], pl.Vr[nd], 1, 0});
    ++li;
  }
  launch(pd, "hm_d");
  launch(pf, "hm_f");
  return launches;
}

static void dense_product(int K, const double *F, const double *u, const double *v,
                          const double *difl, const double *difr, const double *X, long long ldx,
                          int nrows, double *Y, long long ldy, cudaStream_t st, bool sq = false) {
  double *C = pool<double>("hss_denseC", (size_t)K * K);
  launch_cauchy_eig(K, F, u, v, difl, difr, C, st, sq);
  std::vector<GemmDesc> g{{X, C, Y, (int)ldx, K, (int)ldy, nrows, K, K, 0, 0}};
  launch_gemm(g, 0, st);
}

static LevelView single_view(int K, cudaStream_t st) {
  std::vector<int> hv{0, K, 0, K};
  int *v = up("hss_view", hv, st);
  std::vector<double> r{1.0};
  double *rr = up("hss_view_rho", r, st);
  return LevelView{v, v + 1, rr, v + 2, 1};
}

int hss_merge(const HssMergeArgs &a, int *rank, cudaStream_t st) {
  int launches = 0;
  LevelView lv = single_view(a.K, st);
  launch_alpha(lv, a.K, a.dl, a.difl, a.difr, a.zhat, a.alpha, st);
  double *X = pool<double>("hss_X", (size_t)a.n * a.K);
  double *T = pool<double>("hss_T", (size_t)a.n * a.K);
  std::vector<int> hv{a.s, a.n, 0, a.K};
  int *dv = up("hss_gview", hv, st);
  std::vector<long long> z0{0};
  long long *boff = up("hss_boff", z0, st);
  launch_gather(1, a.K, a.n, dv, dv + 1, dv + 2, a.ndslot - a.s, nullptr, boff, a.Q, a.ldq, X, st,
                a.sup);
  launches += 2;
  HssPlan pl;
  stage_begin(HSS_ST_HSS_BUILD, st);
  launches += hss_construct(pl, a.K, a.leaf, a.tol, a.dl, a.zhat, a.alpha, a.difl, a.difr, st);
  stage_end(HSS_ST_HSS_BUILD, st, 0, 0.0);
  if (pl.ok) {
    stage_begin(HSS_ST_HSS_MM, st);
    double fl = 0.0;
    long long by = 0;
    launches += hss_multiply(pl, X, a.n, a.n, T, a.n, a.precision, st, &fl, &by);
    stage_end(HSS_ST_HSS_MM, st, by, fl);
    *rank = pl.max_rank;
  } else {  // rank capacity exceeded: exact dense product
    dense_product(a.K, a.dl, a.zhat, a.alpha, a.difl, a.difr, X, a.n, a.n, T, a.n, st);
    launches += 2;
    *rank = a.K;
  }
  launch_scatter(1, a.K, a.n, dv, dv + 1, dv + 2, a.ndslot - a.s, boff, T, a.Q, a.ldq, st, a.sup);
  return launches + 1;
}

// HSS path of one bidiagonal SVD merge (DHSSVCS, SRC/CauchyHssvd_VPS.f90:3587-3803):
// V2 <- V2 C_V with C_V(i,j) = zhat_i alpha_j / (d_i^2 - sigma_j^2), and
// U2 <- U2 C_U - U2(:, 0) beta^T with C_U(i,j) = d_i zhat_i beta_j /
// (d_i^2 - sigma_j^2): row 0 of C_U vanishes (d_0 = 0), and the -beta_j entries
// of DLASD3's first row are the rank-one term (the reference's DGER,
// SRC/mdlasd1.f90).  Both Cauchy-like matrices are compressed by the same
// structured RRLU in singular-value mode (differences of squares).
int svd_hss_merge(const SvdHssArgs &a, int *rank, cudaStream_t st) {
  int launches = 0;
  double *alpha = pool<double>("svh_alpha", a.K), *beta = pool<double>("svh_beta", a.K),
         *ud = pool<double>("svh_ud", a.K);
  launch_svd_norms(a.K, a.dl, a.difl, a.difr, a.zhat, alpha, beta, ud, st);
  const int rows = std::max(a.N, a.M);
  double *X = pool<double>("hss_X", (size_t)rows * a.K);
  double *T = pool<double>("hss_T", (size_t)rows * a.K);
  std::vector<long long> z0{0};
  long long *boff = up("hss_boff", z0, st);
  *rank = 0;
  for (int side = 0; side < 2; ++side) {  // 0: right vectors V, 1: left vectors U
    const int nr = side == 0 ? a.M : a.N;
    double *Q = side == 0 ? a.V : a.U;
    std::vector<int> hv{a.s, nr, 0, a.K};
    int *dv = up(side == 0 ? "svh_gv0" : "svh_gv1", hv, st);
    launch_gather(1, a.K, nr, dv, dv + 1, dv + 2, a.ndslot - a.s, nullptr, boff, Q, a.ld, X, st);
    const double *u = side == 0 ? a.zhat : ud;
    const double *v = side == 0 ? alpha : beta;
    HssPlan pl;
    stage_begin(HSS_ST_HSS_BUILD, st);
    // the SVD module's swap threshold (rrluCauchysvd, CauchyHssvd_VPS.f90:110)
    launches += hss_construct(pl, a.K, a.leaf, a.tol, a.dl, u, v, a.difl, a.difr, st, true, 1.1);
    stage_end(HSS_ST_HSS_BUILD, st, 0, 0.0);
    if (pl.ok) {
      stage_begin(HSS_ST_HSS_MM, st);
      double fl = 0.0;
      long long by = 0;
      launches += hss_multiply(pl, X, nr, nr, T, nr, a.precision, st, &fl, &by);
      stage_end(HSS_ST_HSS_MM, st, by, fl);
      *rank = std::max(*rank, pl.max_rank);
    } else {
      dense_product(a.K, a.dl, u, v, a.difl, a.difr, X, nr, nr, T, nr, st, true);
      *rank = a.K;
    }
    if (side == 1) launch_svd_rank1(nr, a.K, X, nr, beta, T, nr, st);
    launch_scatter(1, a.K, nr, dv, dv + 1, dv + 2, a.ndslot - a.s, boff, T, Q, a.ld, st);
    launches += 4;
  }
  return launches + 1;
}

// Generic Cauchy matrix in the merge representation: row poles F (the "old
// poles"), column poles D (the "roots"): DIFL_j = D_j - F_j, DIFR_j = D_j - F_{j+1},
// and the column generator -u.
__global__ void k_cauchy_repr(int n, const double *__restrict__ D, const double *__restrict__ F,
                              const double *__restrict__ u, double *__restrict__ difl,
                              double *__restrict__ difr, double *__restrict__ mu) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  difl[j] = D[j] - F[j];
  difr[j] = j + 1 < n ? D[j] - F[j + 1] : 0.0;
  mu[j] = -u[j];
}

// Out (cols x rows, ldo) = In^T for In (rows x cols, ldi): 32 x 32 tiles.
__global__ void k_transpose(int rows, int cols, const double *__restrict__ In, long long ldi,
                            double *__restrict__ Out, long long ldo) {
  __shared__ double t[32][33];
  const int r0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int r = r0 + threadIdx.x, cc = c0 + k;
    if (r < rows && cc < cols) t[k][threadIdx.x] = In[(long long)cc * ldi + r];
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int cc = c0 + threadIdx.x, r = r0 + k;
    if (r < rows && cc < cols) Out[(long long)r * ldo + cc] = t[threadIdx.x][k];
  }
}

void transpose(int rows, int cols, const double *In, long long ldi, double *Out, long long ldo,
               cudaStream_t st) {
  dim3 g((rows + 31) / 32, (cols + 31) / 32);
  k_transpose<<<g, dim3(32, 8), 0, st>>>(rows, cols, In, ldi, Out, ldo);
}

// CauchyHssMM (SRC/cauchyhssmm.f90:1): B (n x ncb, ldb) <- C B with
// C_ij = u_i v_j / (D_i - F_j) compressed to HSS (leaf ni, tolerance tol).
// Computed as (B^T C^T)^T: C^T is Cauchy-like with row poles F, column poles D
// and generators (v, -u), so the structured RRLU and the multiply of the merge
// apply unchanged.  times[0] / times[1]: construction / multiplication (ms).
int hss_cauchyhssmm_core(int n, const double *D, const double *F, const double *u,
                         const double *v, int ni, double tol, int precision, double *B,
                         long long ldb, int ncb, int *rank, float *times, cudaStream_t st) {
  double *difl = pool<double>("chm_difl", n), *difr = pool<double>("chm_difr", n),
         *mu = pool<double>("chm_mu", n);
  double *X = pool<double>("chm_X", (size_t)ncb * n), *Y = pool<double>("chm_Y", (size_t)ncb * n);
  cudaEvent_t e0, e1, e2;
  HCK(cudaEventCreate(&e0)); HCK(cudaEventCreate(&e1)); HCK(cudaEventCreate(&e2));
  HCK(cudaEventRecord(e0, st));
  k_cauchy_repr<<<(n + 255) / 256, 256, 0, st>>>(n, D, F, u, difl, difr, mu);
  HssPlan pl;
  // the generic Cauchy module's swap threshold and full-rank rule (rrluCauchy,
  // CauchyHss_VP2.f90:70; comprcauchy, :650)
  int launches = 1 + hss_construct(pl, n, ni, tol, F, v, mu, difl, difr, st, false, 1.02, true);
  HCK(cudaEventRecord(e1, st));
  transpose(n, ncb, B, ldb, X, ncb, st);
  if (pl.ok) {
    launches += hss_multiply(pl, X, ncb, ncb, Y, ncb, precision, st);
    *rank = pl.max_rank;
  } else {
    dense_product(n, F, v, mu, difl, difr, X, ncb, ncb, Y, ncb, st);
    *rank = n;
  }
  transpose(ncb, n, Y, ncb, B, ldb, st);
  HCK(cudaEventRecord(e2, st));
  HCK(cudaEventSynchronize(e2));
  if (times) {
    HCK(cudaEventElapsedTime(&times[0], e0, e1));
    HCK(cudaEventElapsedTime(&times[1], e1, e2));
  }
  cudaEventDestroy(e0); cudaEventDestroy(e1); cudaEventDestroy(e2);
  return launches + 2;
}

int hss_dhssevc_core(int K, int ni, double tol, int precision, const double *F, const double *u,
                     const double *v, const double *difl, const double *difr, double *Q,
                     long long ldq, int nrows, int *rank, cudaStream_t st, float *times, bool sq,
                     double swap_rho) {
  double *T = pool<double>("hss_T", (size_t)nrows * K);
  cudaEvent_t e0 = nullptr, e1 = nullptr, e2 = nullptr;
  if (times) {
    HCK(cudaEventCreate(&e0)); HCK(cudaEventCreate(&e1)); HCK(cudaEventCreate(&e2));
    HCK(cudaEventRecord(e0, st));
  }
  HssPlan pl;
  int launches = hss_construct(pl, K, ni, tol, F, u, v, difl, difr, st, sq, swap_rho);
  if (times) HCK(cudaEventRecord(e1, st));
  if (pl.ok) {
    launches += hss_multiply(pl, Q, ldq, nrows, T, nrows, precision, st);
    *rank = pl.max_rank;
  } else {
    dense_product(K, F, u, v, difl, difr, Q, ldq, nrows, T, nrows, st, sq);
    *rank = K;
  }
  HCK(cudaMemcpy2DAsync(Q, ldq * sizeof(double), T, nrows * sizeof(double), nrows * sizeof(double), K,
                        cudaMemcpyDeviceToDevice, st));
  if (times) {  // construction / product (with the copy back) in ms
    HCK(cudaEventRecord(e2, st));
    HCK(cudaEventSynchronize(e2));
    HCK(cudaEventElapsedTime(&times[0], e0, e1));
    HCK(cudaEventElapsedTime(&times[1], e1, e2));
    cudaEventDestroy(e0); cudaEventDestroy(e1); cudaEventDestroy(e2);
  }
  return launches + 1;
}

}  // namespace hss
