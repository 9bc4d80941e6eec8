/*
 * hss_oracle.h -- CPU oracle for the HSS-accelerated divide-and-conquer merge.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker that the CUDA path in
 * hsspack_gb300/ is compared against, and the timed CPU baseline of bench.py.
 * Nothing in the product links it or calls it.
 *
 * It restates HSSPACK's Fortran algorithm (MDSTEDC -> MDLAED0/1/2/3 -> DHSSEVC ->
 * Cauchy2hssEig -> ComprcauchyEig -> rrluCauchyEig{row,col} -> fastHssmmL) in
 * C++, and calls LAPACK (DLAED4, DLAED3, DSTEQR, DLAMRG, DGEMM, DSTEDC) from the
 * OpenBLAS shipped inside SciPy (symbols scipy_<name>_), loaded with dlopen.
 * The reference build pins LAPACK 3.5.0 / MKL 2013; the OpenBLAS build bundles
 * reference LAPACK >= 3.11, whose DLAED4/DLAED3/DSTEQR algorithms are unchanged.
 */
#ifndef HSS_ORACLE_H
#define HSS_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int hss_leaf;      /* Ni: HSS leaf block size (reference: 200, mdlaed3.f90:253) */
  int bsmlz;         /* K threshold for HSS vs LAPACK DLAED3 (mdlaed2.f90:175)    */
  double tol;        /* low-rank tolerance (reference: 1e-17, CauchyHssEig.f90:2523) */
  int smlsiz;        /* DC leaf size (ILAENV(9) = 25)                              */
} hso_config;

/* statistics of the last hso_mdstedc call */
typedef struct {
  int n_merges, n_hss_merges, n_dense_merges;
  int max_k;               /* largest secular size                          */
  int max_rank;            /* largest HSS generator rank seen               */
  long long total_k;       /* sum of K over all merges                      */
  long long n_swaps;       /* strong-RRLU swaps                             */
} hso_stats;

int  hso_init(const char *openblas_path);
void hso_set_threads(int nthreads);
int  hso_get_threads(void);
void hso_default_config(hso_config *cfg);
void hso_get_stats(hso_stats *st);

/* MDSTEDC('I'|'V'|'N', ...) with HSS merges; column-major Z(ldz, n). */
int hso_mdstedc(char compz, int n, double *d, double *e, double *z, int ldz,
                const hso_config *cfg);
/* LAPACK DSTEDC('I') on the same inputs (accuracy oracle). */
int hso_dstedc_lapack(int n, double *d, double *e, double *z, int ldz);

/* All K roots of 1 + rho * sum z_i^2/(d_i - x): lam(K), difl(K) = lam_j - d_j,
 * difr(K) = lam_j - d_{j+1} (difr(K-1) = 0).  Uses LAPACK DLAED4. */
int hso_secular(int k, const double *dlamda, const double *z, double rho,
                double *lam, double *difl, double *difr);
/* Loewner rebuild of z (in place) and column scalings alpha (mdlaed3.f90:207-249). */
int hso_lowner(int k, const double *dlamda, const double *difl,
               const double *difr, double *z, double *alpha);
/* Dense Cauchy-like eigenvector block C(i,j) = u_i v_j / (F_i - D_j) through
 * DIFL/DIFR (CauchyHssEig.f90:1688-1765), C is k-by-k column-major. */
void hso_cauchy_eig_dense(int k, const double *F, const double *u,
                          const double *v, const double *difl,
                          const double *difr, double *C);
/* DHSSEVC: Q(0:nrows, 0:k) <- Q * C with C compressed to HSS (leaf ni, tol).
 * ranks_out (optional) receives the max rank; returns 0 on success. */
int hso_dhssevc(int k, int ni, double tol, const double *F, const double *D,
                const double *u, const double *v, const double *difl,
                const double *difr, double *Q, int ldq, int nrows,
                int *max_rank_out);

/* Generic Cauchy matrix A(i,j) = u_i v_j / (D_i - F_j) (Cauchylike.f90:1-13). */
void hso_cauchylike(double *A, const double *D, const double *F,
                    const double *u, const double *v, int m, int n);

#ifdef __cplusplus
}
#endif
#endif
