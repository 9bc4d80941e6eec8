// hss_plan.h -- host-side HSS tree and generator storage shared by the
// Cauchy-like construction (hss_build.cu), the dense construction (mat2hss.cu)
// and the fast HSS multiply.
#pragma once
#include <cuda_runtime.h>

#include <vector>

namespace hss {

// npart / n2tree / GetTreeInfo (SRC/aux_hss.f90:238-307, :737-827): nodes
// 1..ltr in post order, parent[root] = 0, depth[root] = 0.
struct HostTree {
  int lm = 0, ltr = 0, lvl = 0, mmax = 0;
  std::vector<int> m, parent, c1, c2, depth, leafstart;
  std::vector<std::vector<int>> ttr;
  bool leaf(int i) const { return c1[i] == 0 && c2[i] == 0; }
  int sibling(int i) const { int p = parent[i]; return c1[p] == i ? c2[p] : c1[p]; }
};

HostTree make_tree(int K, int ni);

// Node state shared by the row and column kernels.
struct HssDev {
  const double *FF, *DIFL, *DIFR;  // poles and root gaps (length K)
  bool sq;                         // singular-value mode (differences of squares)
  int K, ltr, rmax;
  double rho;                      // strong-swap threshold of the RRLU (1.5 eigen/SVD, 1.02 VP2)
  // full-rank rule: false as ComprcauchyEig (an identity generator once the
  // rank reaches min(M, N), CauchyHssEig.f90:2380); true as the generic
  // module's comprcauchy (the interpolation generator whenever Rk < M,
  // CauchyHss_VP2.f90:650)
  bool vp2;
  // current compressed generators (row side: U, PL; column side: V, PU)
  double *U, *V;
  int *PL, *PU;
  double *Ut, *Vt;  // compaction temporaries
  int *PLt, *PUt;
  int *lr0, *lr1, *lc0, *lc1;    // per node ranges in the current arrays
  int *Ur, *Uc, *Vr, *Vc, *Br, *Bc, *Dm;
  double *Ug, *Vg, *Bg, *Dg;     // generator storage
  long long ucap, vcap, bcap;    // per node capacity (doubles)
  const long long *doff;         // leaf diagonal block offsets
  double *oval;                  // per node "other side" scratch (values)
  int *oidx;                     //                              (pole indices)
  int *lda, *lca;                // current row / column counts
  int *flag;                     // [0]: rank overflow, [1]: swap count
};

struct HssPlan {
  HostTree t;
  HssDev h;
  std::vector<int> Uc, Ur, Vr, Vc, Br, Bc, Dm;
  std::vector<long long> doff;
  bool ok = true;
  int max_rank = 0;
};

// Y (nrows x K, ldy) = X (nrows x K, ldx) * H for the HSS matrix H of pl
// (upsweep G = X U, sibling products F = G B, downsweep F V, leaves X D + F V).
int hss_multiply(const HssPlan &pl, const double *X, long long ldx, int nrows, double *Y,
                 long long ldy, int precision, cudaStream_t st, double *flops = nullptr,
                 long long *bytes = nullptr);

// Out (cols x rows, ldo) = In^T for In (rows x cols, ldi).
void transpose(int rows, int cols, const double *In, long long ldi, double *Out, long long ldo,
               cudaStream_t st);

}  // namespace hss
