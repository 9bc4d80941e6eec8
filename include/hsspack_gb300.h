/*
 * hsspack_gb300.h -- C ABI of the GB300 (sm_103a) HSS divide-and-conquer merge.
 *
 * Two layers:
 *  1. Fortran drop-ins with the reference's argument lists (gfortran/ifort ABI:
 *     lower-case name + '_', every argument by reference, a hidden size_t
 *     length after the visible arguments for each CHARACTER argument).  All
 *     arrays are host memory, column-major.  A Fortran caller links
 *     libhsspack_gb300.so in place of libhsspack.a for these routines.
 *  2. Device entry points (hss_*_dev) taking device pointers and a CUDA stream,
 *     for C/C++ callers whose data already lives in HBM.
 *
 * Status convention (LAPACK): 0 = success, -i = bad i-th argument,
 * > 0 = numerical failure; device-side failures are mapped into > 0 ranges and
 * reported through hss_last_error().  Nothing here aborts the process.
 */
#ifndef HSSPACK_GB300_H
#define HSSPACK_GB300_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------ config ---- */
typedef struct hss_config {
  int hss_leaf;   /* HSS leaf block Ni (reference: 200, SRC/mdlaed3.f90:253)        */
  int bsmlz;      /* merges with K >= bsmlz use HSS, else dense (mdlaed2.f90:175)    */
  double tol;     /* HSS low-rank tolerance (reference: 1e-17, CauchyHssEig.f90:2523) */
  int smlsiz;     /* DC leaf size, ILAENV(9) = 25 (mdlaed0.f90:188)                  */
  int precision;  /* 0: FP64 products; 1: split-BF16 tensor-core products           */
  int predictor;  /* secular start: 0 standard; 1 learned (MLP); 2 FP32 pre-solve;
                    3 FP32 pre-solve refined by one float-float step */
  int batched;    /* 1: one launch per stage per DC level; 0: launches per merge    */
  int profile;    /* 1: time every stage with CUDA events (hss_stats.stage_ms)      */
  int sec_terms;  /* secular solver: at most this many lanes' worth of work per  */
                  /* root (lanes <= the power of two covering K / sec_terms); 0: 8 */
  int split_min_log2; /* split-BF16 products for M*N*K >= 2^this and M >=     */
                      /* split_min_m; 0: 15                                    */
  int small_nk;       /* FP64 products with N, K <= this on the element      */
                      /* kernel (thread per output); 0: 128                    */
  int split_min_m;    /* smallest M of a split-BF16 product; 0: 128            */
  int sec_threads;    /* secular solver: fewest lanes per root that give this  */
                      /* many threads per level (and <= 64 terms per lane);    */
                      /* 0: 152 * 256                                          */
  int gemm_path;      /* split-BF16 products: 0 digit planes staged in global  */
                      /* memory, then the TMA-fed kernel (faster on the DC     */
                      /* shapes); 1 operands split inside each CTA             */
  int reserved[2];
} hss_config;

/* stages timed when hss_config.profile = 1 */
enum hss_stage {
  HSS_ST_LEAF = 0, HSS_ST_PREPARE, HSS_ST_GIVENS, HSS_ST_SECULAR, HSS_ST_LOWNER,
  HSS_ST_BUILD_S, HSS_ST_GATHER, HSS_ST_GEMM, HSS_ST_SCATTER, HSS_ST_FINISH,
  HSS_ST_FINAL, HSS_ST_HSS_BUILD, HSS_ST_HSS_MM, HSS_ST_OTHER, HSS_ST_PREDICT,
  HSS_NSTAGE = 16
};

typedef struct hss_stats {
  int n_levels, n_merges, n_hss_merges, n_dense_merges;
  int max_k, max_rank;
  long long total_k;            /* sum of secular sizes                     */
  long long secular_iters;      /* sum over roots of iterations             */
  long long secular_roots;      /* number of roots solved                   */
  long long predictor_fallbacks;/* roots whose learned guess was rejected   */
  long long kernel_launches;    /* kernels launched by the last call        */
  double ms_total;              /* device time of the last call (events)    */
  double stage_ms[16];          /* per hss_stage device time (profile = 1)  */
  long long stage_calls[16];    /* timed launches per stage                 */
  long long stage_bytes[16];    /* algorithmic bytes moved per stage        */
  double stage_flops[16];       /* algorithmic flops per stage              */
  long long host_h2d_bytes;     /* host entries: bytes copied host -> device */
  long long host_d2h_bytes;     /* host entries: bytes copied device -> host */
  int reserved[4];
} hss_stats;

void hss_default_config(hss_config *cfg);
void hss_set_config(const hss_config *cfg);      /* process-wide default */
void hss_get_config(hss_config *cfg);
void hss_get_stats(hss_stats *st);
const char *hss_last_error(void);
int hss_finalize(void);                           /* frees the device pool */

/* ------------------------------------------ Fortran drop-ins (host) ---- */
/* MDSTEDC(COMPZ,N,D,E,Z,LDZ,WORK,LWORK,IWORK,LIWORK,INFO)
 * replaces SRC/mdstedc.f90:139.  COMPZ = 'I' runs the GPU merge; 'N' returns
 * eigenvalues only; 'V' takes in Z the orthogonal matrix that reduced a
 * symmetric matrix to (D, E) and returns Z times the tridiagonal's
 * eigenvectors (the reference's ICOMPQ = 1 path, mdstedc.f90:341-372; here the
 * tridiagonal solve of 'I' followed by the product on the device).
 * LWORK = -1 or LIWORK = -1 is a workspace query returning the reference's
 * sizes (mdstedc.f90:211-229: 'I' 1+4N+N^2 and 3+5N; 'V' 1+3N+2N lg N+4N^2
 * and 6+6N+5N lg N; 2(N-1) and 1 for N <= 25). */
void mdstedc_(const char *compz, const int *n, double *d, double *e, double *z,
              const int *ldz, double *work, const int *lwork, int *iwork,
              const int *liwork, int *info, size_t compz_len);

/* MDBDSDC(UPLO,COMPQ,N,D,E,U,LDU,VT,LDVT,Q,IQ,WORK,IWORK,INFO) replaces
 * SRC/mdbdsdc.f90:1: SVD of the N x N upper (UPLO = 'U') or lower ('L')
 * bidiagonal (D, E); D returns the singular values in decreasing order, U and
 * VT the singular vectors (COMPQ = 'I') or nothing (COMPQ = 'N').  COMPQ = 'P'
 * (compact form) returns INFO = -2.  Argument numbering as the reference
 * (-1, -2, -3, -7, -9); WORK, IWORK, Q, IQ are not touched (the workspace is
 * in device memory); E is destroyed. */
void mdbdsdc_(const char *uplo, const char *compq, const int *n, double *d, double *e,
              double *u, const int *ldu, double *vt, const int *ldvt, double *q, int *iq,
              double *work, int *iwork, int *info, size_t uplo_len, size_t compq_len);

/* MDBDSVD(N,SB,AB,LDAB,A,S,U,LDU,VT,LDVT,SMLSIZ,WORK,LWORK,IWORK,INFO) replaces
 * SRC/mdbdsvd.f90:1: SVD of the N x N upper banded matrix with SB
 * superdiagonals, AB(LDAB, N) in upper band storage (AB(SB+1+I-J, J) =
 * A(I, J)); S returns the singular values in decreasing order, U the left and
 * VT the (transposed) right singular vectors.  Structured banded divide and
 * conquer: dense leaf SVDs, then at every merge the SB center rows appended
 * one at a time.  INFO as the reference (-2: N < 0 or N < SB, -3: SB < 1,
 * -9 / -10: LDU / LDVT < N, -11: SMLSIZ < 3; the later test wins), plus
 * -4 for LDAB < SB + 1 and -3 for SB > 32 (leaves of at most 64 rows and 96
 * columns in one CTA's shared memory).  SMLSIZ is raised to 3 SB when N > SMLSIZ,
 * as MDBDSVDT does; A, WORK, LWORK and IWORK (workspaces) are not touched. */
void mdbdsvd_(const int *n, const int *sb, double *ab, const int *ldab, double *a, double *s,
              double *u, const int *ldu, double *vt, const int *ldvt, int *smlsiz, double *work,
              int *lwork, int *iwork, int *info);

/* CauchyHssMM(D,F,U,V,N,ni,tol,ncol,B,LDB,time) replaces SRC/cauchyhssmm.f90:1:
 * B(1:N, 1:N) <- C * B for the Cauchy-like C(i,j) = U(i) V(j) / (D(i) - F(j)),
 * compressed to HSS with leaf ni and tolerance tol; time(1) / time(2) return
 * the construction / multiplication seconds.  ncol (the reference's panel
 * width) is accepted and ignored: all columns are multiplied in one pass. */
void cauchyhssmm_(const double *D, const double *F, const double *U, const double *V,
                  const int *n, const int *ni, const double *tol, const int *ncol, double *B,
                  const int *ldb, double *time);

/* DHSSMM(A,LDA,M,N,B,LDB,K,tol,prank,ni,ncol,time,info) replaces
 * SRC/DHSSMM.f90:1-125: B(1:N, 1:K) <- A_hss * B, where A_hss is the HSS
 * approximation of the dense N x N matrix A built by truncated SVDs of its
 * block rows and columns (mat2hssvd, SRC/ConstructHssd.f90:371: leaf size ni,
 * singular values above the absolute tolerance tol kept).  M must equal N (the
 * reference assumes LDA = M = N).  A is not modified (the reference uses it as
 * workspace).  prank is accepted and ignored, as by the reference's
 * construction; ncol (the reference's panel width) must be >= 1 and is
 * otherwise ignored (all K columns in one pass).  time(1) / time(2): seconds of
 * construction / multiplication.  INFO = -i for a bad i-th argument,
 * 1000000 / 1000001 for a CUDA / construction failure (hss_last_error()). */
void dhssmm_(const double *A, const int *lda, const int *m, const int *n, double *B,
             const int *ldb, const int *k, const double *tol, const int *prank,
             const int *ni, const int *ncol, double *time, int *info);

/* DHSSMML(...) replaces SRC/DHSSMML.f90:2-122: B(1:K, 1:N) <- B * A_hss
 * (B is K x N, LDB >= K); otherwise as DHSSMM. */
void dhssmml_(const double *A, const int *lda, const int *m, const int *n, double *B,
              const int *ldb, const int *k, const double *tol, const int *prank,
              const int *ni, const int *ncol, double *time, int *info);

/* Largest band half-width of the banded divide and conquer (leaves of up to
 * 2 kd rows are solved by one warp each).  Wider bands, and every
 * eigenvalues-only band call, are reduced to tridiagonal form on the device
 * (Householder bulge chasing, the role of LAPACK DSBTRD in the reference) and
 * solved by the tridiagonal divide and conquer. */
#define HSS_BAND_KD_MAX 32

/* MDSBEVD(COMPZ,UPLO,N,KD,AB,LDAB,D,Q,LDQ,WORK,LWORK,IWORK,LIWORK,INFO)
 * replaces SRC/mdsbevd.f90:183: eigenpairs of the symmetric band matrix in
 * upper band storage AB (the reference reads the upper band whatever UPLO
 * says); COMPZ = 'I' computes Q, 'N' eigenvalues only.  Argument errors and
 * workspace queries as the reference (INFO = -1, -2, -6, -8, -10); KD < 0 or
 * LDAB < KD+1 gives INFO = -4.  KD > HSS_BAND_KD_MAX and COMPZ = 'N' go
 * through the device band-to-tridiagonal reduction. */
void mdsbevd_(const char *compz, const char *uplo, const int *n, const int *kd,
              double *ab, const int *ldab, double *d, double *q, const int *ldq,
              double *work, const int *lwork, int *iwork, const int *liwork,
              int *info, size_t compz_len, size_t uplo_len);

/* MDSBEDC(JOBZ,UPLO,N,KD,AB,LDAB,W,Z,LDZ,WORK,LWORK,IWORK,LIWORK,INFO)
 * replaces SRC/mdsbedc.f90:166: JOBZ = 'V' / 'N', UPLO = 'U' / 'L' (lower
 * storage is converted; the reference passes it on as upper).  Workspace
 * LWMIN = 1+5N+2N^2, LIWMIN = 3+5N (JOBZ = 'V') as mdsbedc.f90:190-201.
 * JOBZ = 'N' (the reference's DSBTRD + DSTERF, mdsbedc.f90:311-318) and
 * KD > HSS_BAND_KD_MAX (its DSBEVD fallback for KD > 16, :274-276) reduce
 * the band to tridiagonal form on the device first. */
void mdsbedc_(const char *jobz, const char *uplo, const int *n, const int *kd,
              double *ab, const int *ldab, double *w, double *z, const int *ldz,
              double *work, const int *lwork, int *iwork, const int *liwork,
              int *info, size_t jobz_len, size_t uplo_len);

/* Cauchylike(A,D,F,u,v,M,N): A(i,j) = u(i) v(j) / (D(i) - F(j)),
 * replaces SRC/Cauchylike.f90:1 (computed on the GPU). */
void cauchylike_(double *A, const double *D, const double *F, const double *u,
                 const double *v, const int *m, const int *n);

/* ------------------------------------------------ device entry points ---- */
/* Whole tridiagonal eigensolve, COMPZ='I' semantics, all pointers in HBM.
 * d(n) in: diagonal, out: eigenvalues ascending; e(n-1) off-diagonal
 * (destroyed); z(ldz, n) out: eigenvectors.  stream may be NULL. */
int hss_mdstedc_dev(int n, double *d, double *e, double *z, int ldz, void *stream);

/* Device MDSTEDC('V') (SRC/mdstedc.f90:139 with COMPZ = 'V'): z (n x n,
 * column-major, leading dimension ldz, device) holds on entry the orthogonal
 * matrix Q0 of a reduction to tridiagonal form and on exit Q0 times the
 * eigenvectors of (d, e); d returns the eigenvalues ascending.  Q0 is applied
 * column group by column group over the supports of the divide-and-conquer
 * eigenvectors (grouped tensor-core products under precision = 1).  Returns
 * as hss_mdstedc_dev. */
int hss_mdstedc_v_dev(int n, double *d, double *e, double *z, int ldz, void *stream);

/* SVD of the upper bidiagonal (d, e) in HBM (the MDBDSDC path, COMPQ = 'I'):
 * d(n) in: diagonal, out: singular values descending; e(n-1) superdiagonal;
 * u(ldu, n), vt(ldvt, n) out.  Returns 0, -i for a bad i-th argument, > 0 on
 * failure. */
int hss_mdbdsdc_dev(int n, double *d, double *e, double *u, int ldu, double *vt, int ldvt,
                    void *stream);

/* SVD of the upper banded n x n matrix in HBM (the MDBDSVD path): ab(ldab, n)
 * upper band storage with 1 <= sb <= min(n, 32) superdiagonals; s(n) singular
 * values descending, u(ldu, n), vt(ldvt, n) out; smlsiz >= 3 as MDBDSVD's
 * (the tree depth before the leaves are cut to 64 rows).  Returns 0, -i for a
 * bad i-th argument, > 0 on failure. */
int hss_mdbdsvd_dev(int n, int sb, const double *ab, int ldab, double *s, double *u, int ldu,
                    double *vt, int ldvt, int smlsiz, void *stream);

/* Symmetric band eigensolve in HBM (the MDSBEVD path): ab(ldab, n) upper band
 * storage, kd >= 0 (band divide and conquer up to HSS_BAND_KD_MAX, device
 * reduction to tridiagonal form above); w(n) eigenvalues ascending, z(ldz, n)
 * eigenvectors.  Returns 0, -i for a bad i-th argument, > 0 on failure. */
int hss_mdsbevd_dev(int n, int kd, const double *ab, int ldab, double *w, double *z,
                    int ldz, void *stream);

/* Many independent tridiagonal eigensolves in one call, each with COMPZ='I'
 * semantics of MDSTEDC (SRC/mdstedc.f90:139); no batched counterpart in the
 * reference, whose drivers take one matrix per call.  n(nprob) on the host;
 * d, e, z in HBM, packed: problem p starts at o_p = n_0 + ... + n_{p-1} in d
 * (eigenvalues out, ascending) and e (its n_p - 1 off-diagonals; entry
 * o_p + n_p - 1 is ignored), and at n_0^2 + ... + n_{p-1}^2 in z (eigenvectors,
 * leading dim n_p).  All problems' DC levels run together.  Returns 0, -1 / -2
 * for a bad nprob / n, or > 0 as hss_mdstedc_dev. */
int hss_mdstedc_batch_dev(int nprob, const int *n, double *d, double *e, double *z,
                          void *stream);

/* K secular roots of 1 + rho * sum_i z_i^2 / (dlamda_i - x) (the DLAED4 loop of
 * SRC/mdlaed3.f90:207-225).  Outputs lam(K), difl(K) = lam_j - dlamda_j,
 * difr(K) = lam_j - dlamda_{j+1} (difr(K-1) = 0), iters(K) (may be NULL).
 * Returns 0 or the 1-based index of the first root that failed. */
int hss_secular_dev(int k, const double *dlamda, const double *z, double rho,
                    double *lam, double *difl, double *difr, int *iters,
                    void *stream);

/* Loewner rebuild of z and the column scalings alpha (SRC/mdlaed3.f90:228-249):
 * z(K) in/out, alpha(K) out. */
int hss_lowner_dev(int k, const double *dlamda, const double *difl,
                   const double *difr, double *z, double *alpha, void *stream);

/* hss_lowner_dev without any device allocation; no counterpart in the
 * reference.  For callers that cannot let a library allocate device memory
 * (all of it reserved by their own allocator, or allocation forbidden after
 * start-up): the scratch is a static device array of 65536 doubles, so
 * k <= 65536 (larger k returns -1 and sets hss_last_error()).  Every call
 * looks the scratch address up in the current context; the first call on a
 * device (and the first after cudaDeviceReset) may also load the module there
 * and should come at set-up, before any stream capture.  All calls share the
 * scratch; calls are serialised and wait for their stream, since overlapping
 * ones would race on it. */
int hss_lowner_noalloc_dev(int k, const double *dlamda, const double *difl,
                           const double *difr, double *z, double *alpha,
                           void *stream);

/* SvdHssUpdat(D,F,Z,V,N0,TOL,ni) replaces SRC/SvdHssUpdat.f90:1: the SVD of
 * A = U diag(F) V^T with one row a^T appended, given F (N0, ascending), Z = V^T a
 * and V (N0 x N0, leading dimension N0, the right singular vectors as ROWS, as
 * the reference's MDLASD20 reads it).  On return D(1:K) holds the K new
 * singular values of the non-deflated problem (ascending) and D(K+1:N0) the
 * deflated ones (the reference leaves D(K+1:N0) undefined), F and Z are as
 * MDLASD20 / MDLASD31 leave them (F(1:K) the poles, F(K+1:N0) the deflated
 * values; Z(1:K) recomputed by Loewner's formula), and the rows of V are the
 * updated right singular vectors in the order of D.  The Cauchy-like matrix of
 * the new vectors is compressed to HSS (leaf ni, tolerance TOL) on the GPU.
 * No INFO argument (as the reference): every call clears hss_last_error() on
 * entry, and a failure leaves the outputs untouched and sets it. */
void svdhssupdat_(double *D, double *F, double *Z, double *V, const int *n0, const double *tol,
                  const int *ni);

/* HssCholSolver(RS,WPCG,A,LDA,b,ni,tol,prank,pp,tau,MaxIt,info) replaces
 * SRC/HssCholSolver.f90:1: solves A x = b for the dense SPD matrix A (N = LDA,
 * as the reference) through an HSS Cholesky factorisation (leaves of ni rows,
 * ni <= 128; singular values of the scaled off-diagonal block columns above
 * tol kept, at most prank per node; RS = 'S' exact singular vectors, 'R' a
 * sketch of prank + pp rows).  WPCG = 'N' returns the factorisation's solve,
 * 'Y' the preconditioned CG solution (relative residual below tau or MaxIt + 1
 * steps).  b (N) is replaced by the solution; A is not modified.  INFO: -1 / -2
 * bad RS / WPCG (as the reference), -4, -6, -8, -9, -11 for LDA, ni, prank, pp,
 * MaxIt; 1 a diagonal block not positive definite, 2 a node of more than 128
 * rows, 1000000 / 1000001 CUDA / construction failures (hss_last_error()). */
void hsscholsolver_(const char *rs, const char *wpcg, double *A, const int *lda, double *b,
                    const int *ni, const double *tol, const int *prank, const int *pp,
                    const double *tau, const int *maxit, int *info, size_t rs_len,
                    size_t wpcg_len);

/* DHSSEVC (SRC/CauchyHssEig.f90:2444): Q(0:nrows, 0:K) <- Q * C where
 * C(i,j) = u_i v_j / (F_i - lam_j), lam_j = F_j + difl_j, compressed to HSS
 * with leaf ni and tolerance tol.  Q is column-major with leading dim ldq. */
int hss_dhssevc_dev(int k, int ni, double tol, const double *F, const double *u,
                    const double *v, const double *difl, const double *difr,
                    double *Q, int ldq, int nrows, void *stream);

/* CauchyHssMM on device arrays: B(n, ncb; ldb) <- C B with
 * C(i,j) = u_i v_j / (D_i - F_j) in HSS form (leaf ni, tolerance tol);
 * times[0..1] (may be NULL) receive construction / multiply milliseconds. */
int hss_cauchyhssmm_dev(int n, const double *D, const double *F, const double *u,
                        const double *v, int ni, double tol, double *B, int ldb, int ncb,
                        float *times, void *stream);

/* DHSSMM / DHSSMML on device arrays: A (n x n, lda) compressed to HSS (leaf
 * ni, tolerance tol; A is read only); side 0: B (n x k, ldb) <- A_hss B,
 * side 1: B (k x n, ldb) <- B A_hss.  times[0..1] (may be NULL): construction
 * / multiply milliseconds; hss_get_stats()->max_rank: the largest HSS rank (n
 * when a node dimension exceeded 128 and A was applied as a dense product).
 * Returns 0, -i for a bad i-th argument, or 1000000 / 1000001. */
int hss_dhssmm_dev(int n, const double *A, int lda, double *B, int ldb, int k, double tol,
                   int ni, int side, float *times, void *stream);

/* SvdHssUpdat on device arrays: d, f, z (n), vt (n x n, ldvt; rows = right
 * singular vectors), as svdhssupdat_; *k (may be NULL) receives K, the order of
 * the secular equation after deflation.  hss_get_stats(): max_rank (the
 * largest HSS rank; K when the product ran as one dense block), stage_ms of
 * HSS_ST_HSS_BUILD / HSS_ST_HSS_MM.  Returns 0, -i for a bad i-th argument, a
 * positive status (a secular root did not converge), or 1000000 / 1000001. */
int hss_svdhssupdat_dev(int n, double *d, double *f, double *z, double *vt, int ldvt,
                        double tol, int ni, int *k, void *stream);

/* MDLASD20's deflation alone (host code; needs no GPU): f, z (n) modified as
 * MDLASD20 leaves them, idxp[j] (n) the original position of new position j;
 * *nrot (may be NULL) the number of deflating rotations.  Returns K. */
int hss_svdupd_deflate(int n, double *f, double *z, int *idxp, int *nrot);

/* The banded SVD's tree (host logic of the MDBDSVD path, no GPU): the leaves of
 * the n-row band with sb superdiagonals, in row order -- first row, rows, and
 * columns (rows + the sb extra columns, none for the last leaf); the arrays hold
 * n entries.  Returns the number of merge levels, -1 for bad arguments, -2 when
 * no tree fits the leaf limit. */
int hss_bsvd_tree(int n, int sb, int smlsiz, int *leaf_start, int *leaf_rows, int *leaf_cols,
                  int *nleaves);

/* HSS Cholesky on device arrays (the pieces of HssCholSolver).  The factor
 * owns its device memory until hss_chol_free.
 * hss_chol_factor_dev: A (n x n, lda; read only); ni leaf rows (<= 128); tol;
 *   prank the largest rank kept per node; ps = 0 exact singular vectors of the
 *   scaled block columns, ps > 0 those of a ps-row uniform [0,1) sketch.
 *   Returns 0 (*out set), -i for a bad i-th argument, 1 / 2 as INFO above.
 * hss_chol_solve_dev: B (n x nrhs, ldb) <- the factorisation's solve.
 * hss_chol_pcg_dev: x <- CG solution of A x = b preconditioned by the factor
 *   (f = NULL: unpreconditioned); *iters, *relres as the loop ends. */
typedef struct hss_chol hss_chol;
int hss_chol_factor_dev(int n, const double *A, int lda, int ni, double tol, int prank, int ps,
                        hss_chol **out, void *stream);
int hss_chol_solve_dev(const hss_chol *f, double *B, int ldb, int nrhs, void *stream);
int hss_chol_pcg_dev(const hss_chol *f, int n, const double *A, int lda, const double *b,
                     double *x, double tau, int maxit, int *iters, double *relres, void *stream);
int hss_chol_info(const hss_chol *f, int *n, int *max_rank, int *levels, int *root,
                  long long *bytes);
void hss_chol_free(hss_chol *f);

/* Dense Cauchy-like eigenvector block C(i,j) = u_i v_j / (F_i - lam_j) through
 * DIFL/DIFR (SRC/CauchyHssEig.f90:1688, CauchylikeEig), k-by-k column-major. */
int hss_cauchy_eig_dev(int k, const double *F, const double *u, const double *v,
                       const double *difl, const double *difr, double *C,
                       void *stream);

/* Diagnostic (no counterpart in the reference): y[i] = 1 / x[i] by the
 * reciprocal the secular pole sums and the eigenvector blocks use instead of
 * a correctly rounded divide (two Newton-Raphson steps from the hardware
 * estimate; within a few ulp for normal x), so its accuracy can be checked. */
int hss_rcp_dev(int n, const double *x, double *y, void *stream);

/* Measurement helper (no counterpart in the reference): the GPU's FP64 FMA
 * rate.  One launch of `blocks` CTAs x 256 threads, each thread running eight
 * independent chains of `iters` FMAs, timed with CUDA events on `stream`
 * after one untimed launch; *ms = its duration, *tflops = 2 flops per FMA
 * over it.  Returns 0, -1 for bad arguments, 1000000 on a CUDA error. */
int hss_fp64_fma_rate(int blocks, int iters, float *ms, double *tflops, void *stream);

/* C(m x n, ldc) = A(m x k, lda) * B(k x n, ldb) [+ C if beta != 0], FP64
 * column-major device arrays; precision 0 = FP64 CUDA cores, 1 = split-BF16
 * tensor cores (7 digit planes, exact integer accumulation; error below
 * 2^-56 of sum |A||B|).  The
 * grouped GEMM behind the dense merge update of LAPACK DLAED3 (called at
 * SRC/mdlaed1.f90:199) and the HSS multiply (SRC/ConstructHssd.f90:1394). */
int hss_gemm_dev(int m, int n, int k, const double *A, int lda, const double *B, int ldb,
                 double *C, int ldc, int beta, int precision, void *stream);

/* ---------------------------------------- learned secular initial iterate ----
 * No reference counterpart: a 3 x 64 MLP (BF16 weights, FP32 math) predicting
 * each root's position inside its pole interval from local features; used as
 * the first iterate of the secular solver when hss_config.predictor = 1.  The
 * FP64 iteration always finishes (and restarts from the standard guess when
 * the learned start fails its residual check). */
int hss_predictor_nparam(void);                 /* parameters (FP32 layout)    */
int hss_predictor_nfeat(void);                  /* features per root           */
/* install weights W[nparam] and feature normalisation norm[2*nfeat] (host) */
int hss_predictor_set(const float *W, const float *norm);
/* training features X[(k-1) x nfeat] and targets T[k-1] for one solved
 * secular problem (device arrays; difl/difr from hss_secular_dev) */
int hss_predictor_features_dev(int k, const double *d, const double *z, double rho,
                               const double *difl, const double *difr, float *X, float *T,
                               void *stream);
/* mean squared error and its gradient G[nparam] over n samples (device) */
int hss_predictor_grad_dev(int n, const float *X, const float *T, const float *norm,
                           const float *W, float *G, float *loss, void *stream);
/* one Adam step on W with moments M, V (device arrays of nparam floats) */
int hss_predictor_adam_dev(const float *G, float *W, float *M, float *V, float lr, int step,
                           void *stream);
/* learned starts guess[k]: +u / -u = distance u <= 1/2 (in units of the pole
 * gap) from the left / right pole of the root's interval; 2 = no prediction */
int hss_predict_dev(int k, const double *d, const double *z, double rho, float *guess,
                    void *stream);

#ifdef __cplusplus
}
#endif
#endif
