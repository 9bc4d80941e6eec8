// hss_kernels.h -- host-side launch wrappers of the device kernels.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

namespace hss {

// Merges of one DC level that have K > 0, compacted: merge m owns positions
// [s[m], s[m] + K[m]) of the level arrays; rootoff = prefix sum of K (P + 1).
struct LevelView {
  const int *s;
  const int *K;
  const double *rho;
  const int *rootoff;
  int P;
};

struct LevelScratch {
  int *srt;
  double *ds;
  double *zs;
  unsigned char *typ;
  int *cand;
  double *dl;
  double *zw;
  int *ndslot;
  int *grp;
  int *dfslot;
  double *dfval;
  int *gvp, *gvq;
  double *gvc, *gvs;
  int *l1slot, *l2slot;  // deflated by small z / by rotation, before merging
  double *l1val, *l2val;
};

// secular.cu
// lane-group width target of the secular kernels (pole terms per lane; 0: 8)
void set_secular_terms(int t);
// threads a secular level should reach before lanes per root shrink (0: 152 * 256)
void set_secular_threads(int t);
// sq: singular-value mode (poles d_i^2, outputs sigma and DIFL/DIFR = sigma - d)
// guess: per root start (see root_init), full: its bracket is the whole interval
// gref: exact starts of the refined pre-solve (launch_secular_guess32 with gref)
void launch_secular(const LevelView &lv, int total, int maxk, const double *dl, const double *zw,
                    double *lam, double *difl, double *difr, int *iters, int *status,
                    unsigned long long *itsum, const float *guess, cudaStream_t st,
                    bool sq = false, bool full = false, const float4 *gref = nullptr);
// starts for the FP64 iteration from an FP32 pre-solve (npos: positions of the
// level arrays, d32 / z32 their FP32 copies; sq: singular-value mode)
// gref (with d32lo, z2h, z2l, npos floats each): the refined pre-solve, one
// float-float evaluation and step after the FP32 iteration
void launch_secular_guess32(const LevelView &lv, int total, int maxk, int npos,
                            const double *dl, const double *zw, float *d32, float *z32,
                            float *guess, cudaStream_t st, bool sq = false,
                            float *d32lo = nullptr, float *z2h = nullptr, float *z2l = nullptr,
                            float4 *gref = nullptr);
// maxk: the largest K of the launch (lanes per root as the secular kernel;
// the default keeps a full warp per root)
void launch_lowner(const LevelView &lv, int total, const double *dl, const double *difl,
                   const double *difr, const double *zw, double *zhat, cudaStream_t st,
                   bool sq = false, int maxk = 1 << 30);
void launch_alpha(const LevelView &lv, int total, const double *dl, const double *difl,
                  const double *difr, const double *zhat, double *alpha, cudaStream_t st,
                  bool sq = false);
void launch_build_S(const LevelView &lv, int total, const double *dl, const double *difl,
                    const double *difr, const double *zhat, const int *grp,
                    const long long *soff, double *Sws, cudaStream_t st);
void launch_cauchy_eig(int K, const double *F, const double *u, const double *v,
                       const double *difl, const double *difr, double *C, cudaStream_t st,
                       bool sq = false);
void launch_cauchylike(int M, int N, const double *D, const double *F, const double *u,
                       const double *v, double *A, cudaStream_t st);

// the reciprocal of the pole sums (rcp_nr), for its accuracy test
void launch_rcp(int n, const double *x, double *y, cudaStream_t st);

// leaf.cu
void launch_leaf(int nleaf, const int *lstart, const int *lsize, int mmax, int nblk,
                 const double *d, const double *e, double *Q, long long ldq, double *Dp, int *perm,
                 int *status, cudaStream_t st, int2 *sup = nullptr);

// merge.cu
// prepare flags: the block is already in ascending order (no merge of two
// halves); every column is dense (no top / bottom block structure)
enum { PREP_SORTED = 1, PREP_DENSE = 2, PREP_FRONT = 4 /* order and z from k_merge_front */ };
// zsrc: z per slot instead of the rows of Q around the cut; rsrc: the coupling
// rho_in per merge instead of e[s + n1 - 1]
void launch_merge_prepare(int P, int maxn, const int *ms, const int *mn, const int *mn1, const double *e,
                          const double *Q, long long ldq, double *Dp, int *perm,
                          const LevelScratch &w, int *out, double *orho, cudaStream_t st,
                          const double *zsrc = nullptr, const double *rsrc = nullptr,
                          int flags = 0, const int2 *sup = nullptr);
// merged order and z of every position of a level (poff: prefix of mn, P + 1)
void launch_merge_front(int P, int total, const int *poff, const int *ms, const int *mn,
                        const int *mn1, const double *e, const double *Q, long long ldq,
                        const double *Dp, const int *perm, const LevelScratch &w,
                        const double *zsrc, const double *rsrc, int flags, cudaStream_t st,
                        const int2 *sup = nullptr);
// Zr (nz columns, leading dim zld): rows rotated with the Q columns
void launch_givens(int P, int maxn, const int *ms, const int *mn, const int *ng,
                   const LevelScratch &w, double *Q, long long ldq, cudaStream_t st,
                   double *Zr = nullptr, int nz = 0, long long zld = 0);
// sup (optional): per slot the rows [x, y) a column holds data on (zero
// elsewhere); gathers read within it, scatters set it to the merge's rows
void launch_gather(int P, int total, int maxn, const int *ms, const int *mn, const int *rootoff,
                   const int *ndslot, const int *grp, const long long *boff, const double *Q,
                   long long ldq, double *B, cudaStream_t st, const int2 *sup = nullptr);
void launch_scatter(int P, int total, int maxn, const int *ms, const int *mn, const int *rootoff,
                    const int *ndslot, const long long *toff, const double *T, double *Q,
                    long long ldq, cudaStream_t st, int2 *sup = nullptr);
// columns about to be rotated: zeros written outside their support, support
// widened to the merge's rows
void launch_widen(int P, int maxn, const int *ms, const int *mn, const int *ng,
                  const LevelScratch &w, double *Q, long long ldq, int2 *sup, cudaStream_t st);
void launch_merge_finish(int P, int maxn, const int *ms, const int *mn, const int *mK, const double *lam,
                         const LevelScratch &w, int *perm, double *Dp, cudaStream_t st);
// the finish of all merges with one thread per position (poff: prefix of the
// merges' sizes, P + 1 entries)
void launch_merge_finish_grid(int P, int total, const int *poff, const int *ms, const int *mK,
                              const double *lam, const LevelScratch &w, int *perm, double *Dp,
                              cudaStream_t st);
void launch_final_gather(int n, const int *perm, const double *Dp, const double *Q, long long ldq,
                         double *Z, long long ldz, double *wout, cudaStream_t st,
                         const int2 *sup = nullptr);
// packed final permutation: the supported rows of every output column back to
// back at out + off[c] (off from the host), w(c) = Dp(perm(c))
void launch_pack_columns(int n, const int *perm, const double *Dp, const double *Q, long long ldq,
                         const int2 *sup, const long long *off, double *out, double *wout,
                         cudaStream_t st);
void launch_repack_columns(int n, const int *order, const long long *soff, const long long *doff,
                           const double *src, double *dst, cudaStream_t st);
void launch_scatter_columns(int n, int m, const int *order, const double *T, long long ldt,
                            double *out, long long ldo, cudaStream_t st);
// many problems per call: P = global start of each problem (np + 1 entries),
// total = P[np]; problem p's block is Q + P[p] * (ldq + 1), leading dim ldq
void launch_zero_blocks(int np, long long total, const long long *P, double *Q, long long ldq,
                        cudaStream_t st);
void launch_scale_blocks(int nb, const int *bs, const int *bm, const double *bscl, double *Dp,
                         cudaStream_t st);
void launch_final_gather_batch(int np, long long total, const long long *P, const int *perm,
                               const double *Dp, const double *Q, long long ldq, double *const *Z,
                               const long long *ldz, double *const *W, cudaStream_t st,
                               const int2 *sup = nullptr);

// predictor.cu
int mlp_nparam();
int mlp_nfeat();
void launch_predict(int n, const float *feat, const void *Wb, const float *norm, float *guess,
                    cudaStream_t st);
void launch_train_targets(int K, const double *d, const double *difl, const double *difr,
                          const float *feat, float *X, float *T, cudaStream_t st);
// secular.cu: midpoint evaluation producing the predictor features, nf + 1
// floats per root at position s + j (the level layout)
void launch_secular_mid(const LevelView &lv, int total, int maxk, const double *dl,
                        const double *zw, float *feat, cudaStream_t st);
void launch_mlp_grad(int n, const float *X, const float *T, const float *norm, const float *W,
                     float *G, float *L, cudaStream_t st);
void launch_adam(int np, float *W, const float *G, float *M, float *V, float lr, int step,
                 void *Wb, cudaStream_t st);

// band.cu: banded divide and conquer (cuts, leaves, Z = Q^T W, Z updates)
void launch_band_cut_svd(int ncut, const int *cut_row, int kd, const double *AB, long long ldab,
                         double *Uc, double *Vc, double *Sc, int *status, cudaStream_t st);
void launch_band_leaf(int nleaf, const int *lstart, const int *lsize, const int *cut_above,
                      const int *cut_below, int mmax, int kd, const double *AB, long long ldab,
                      const double *Uc, const double *Vc, const double *Sc, double *Q,
                      long long ldq, double *Dp, int *perm, int *status, cudaStream_t st);
void launch_band_z(int P, int maxn, const int *ms, const int *mn, const int *mn1, const int *mcut,
                   int kd, const double *Q, long long ldq, const double *Uc, const double *Vc,
                   double *Z, long long zld, cudaStream_t st);
void launch_band_zupdate(const LevelView &lv, int total, const double *dl, const double *difl,
                         const double *difr, const double *zhat, const double *alpha,
                         const int *ndslot, double *Z, int nrest, long long zld, double *Zt,
                         cudaStream_t st);

// svd.cu: bidiagonal SVD divide and conquer
void launch_svd_leaf(int nleaf, const int *lstart, const int *lsize, const int *lsqre, int rmax,
                     const double *d, const double *e, double *U, long long ldu, double *V,
                     long long ldv, double *Dp, int *perm, int *status, cudaStream_t st);
void launch_svd_prepare(int P, int maxn, const int *ms, const int *mnl, const int *mnr,
                        const int *msq, const double *d, const double *e, double *U,
                        long long ldu, double *V, long long ldv, const double *Dp, const int *perm,
                        const LevelScratch &w, int *out, double *onrm, cudaStream_t st);
// U / V blocks (K x K per merge at boff); sigma rescaled by onrm
void launch_svd_vectors(const LevelView &lv, int total, const double *dl, const double *difl,
                        const double *difr, const double *zhat, const long long *boff, double *Ub,
                        double *Vb, cudaStream_t st);
void launch_svd_unscale(const LevelView &lv, int total, const double *onrm, double *lam,
                        cudaStream_t st);
// HSS path of one SVD merge: norms and U generator; the row-0 rank-one term
void launch_svd_norms(int K, const double *dl, const double *difl, const double *difr,
                      const double *zhat, double *alpha, double *beta, double *ud,
                      cudaStream_t st);
void launch_svd_rank1(int nrows, int K, const double *X, long long ldx, const double *beta,
                      double *T, long long ldt, cudaStream_t st);
// outputs in descending order: Uo (ldu), VT (ldvt), w; only w if !vectors
void launch_svd_outputs(int n, const int *perm, const double *Dp, const double *Uq,
                        long long ldq, const double *V, long long ldv, double *Uo, long long ldu,
                        double *VT, long long ldvt, double *w, bool vectors, cudaStream_t st);
void launch_rows_rotate_back(int n, int ncols, const double *cs, const double *sn, double *A,
                             long long lda, cudaStream_t st);

// bsvd.cu: banded SVD divide and conquer (leaves, row coefficients z = V^T b,
// the fold of the null vectors, the deflation of a row append)
size_t bsvd_leaf_smem();
int bsvd_rows_max();
int bsvd_cols_max();
void launch_bsvd_leaf(int nleaf, const int *la, const int *lr, const int *lc, int sb,
                      const double *AB, long long ldab, double *U, long long ldu, double *V,
                      long long ldv, double *Dp, int *perm, int *status, cudaStream_t st);
void launch_bsvd_z(int P, int total, const int *poff, const int *ms, const int *mrow, int sb, int n,
                   const double *AB, long long ldab, const double *V, long long ldv, double *z,
                   cudaStream_t st);
void launch_bsvd_fold(int P, int maxm, const int *ms, const int *mN, const int *mM, const int *mnl,
                      const int *mrow, int sb, int n, const double *AB, long long ldab, double *V,
                      long long ldv, double *z, double *amax, cudaStream_t st);
void launch_bsvd_prepare(int P, int maxn, const int *ms, const int *mrow, const int *mna,
                         const int *mb0, const int *mnb, const double *amax, const double *zslot,
                         double *U, long long ldu, const double *Dp, const int *perm,
                         const LevelScratch &w, int *out, double *onrm, cudaStream_t st);

// driver.cu: set the message hss_last_error() returns
void set_last_error(const std::string &msg);

// band -> tridiagonal reduction (band_sbr.cu): working band in lower storage
// with ldb = 2b diagonals; reflectors (b doubles each) of step j of sweep s
// at roff[s] + j when R is not null.
long long sbr_reflectors(int n, int b, std::vector<long long> *roff);
void launch_sbr_load(int n, int kd, int b, const double *AB, long long ldab, double *LB, int ldb,
                     cudaStream_t st);
int launch_sbr_reduce(int n, int b, double *LB, int ldb, double *R, const long long *droff,
                      double *rtau, cudaStream_t st);
void launch_sbr_tri(int n, const double *LB, int ldb, double *d, double *e, cudaStream_t st);
int launch_sbr_back(int n, int b, const double *R, const long long *droff, const double *rtau,
                    double *Z, long long ldz, cudaStream_t st);

}  // namespace hss
