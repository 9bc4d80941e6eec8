// hss_oracle.cpp -- CPU oracle (test infrastructure, never shipped).
//
// A C++ restatement of HSSPACK's tridiagonal divide-and-conquer eigensolver with
// HSS-accelerated merges.  Each routine names the Fortran it follows
// (paths relative to the HSSPACK source tree).  LAPACK pieces that the
// reference calls but does not ship (DLAED4, DLAED3, DSTEQR, DLAMRG, DGEMM,
// DSTEDC) come from SciPy's OpenBLAS through dlopen.
//
// Deliberate deviations from the Fortran, all numerical no-ops or bug fixes:
//  * CauchyPivtEig (CauchyHssEig.f90:683-688) reads the local row-pole array
//    F at the global index PL(k) when forming the current pivot; the intended
//    value F_k = FF(PL(k)) is used here.
//  * fastHssmmL_omp returns without multiplying when the HSS tree has fewer
//    than 3 levels (ConstructHssd.f90:1455-1458); this multiply handles every
//    tree depth >= 1.
//  * The multiply runs over all rows of X at once instead of 200-row panels
//    (CauchyHssEig.f90:2585-2592); the arithmetic per entry is the same.
//  * Generator blocks are kept per node instead of in one H array whose order
//    depends on the OpenMP schedule (CauchyHssEig.f90:2385-2401).
#include "hss_oracle.h"

#include <dlfcn.h>
#include <omp.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

namespace {

// ---------------------------------------------------------------- LAPACK ----
typedef void (*fn_dlaed4)(const int *, const int *, const double *,
                          const double *, double *, const double *, double *,
                          int *);
typedef void (*fn_dlaed3)(const int *, const int *, const int *, double *,
                          double *, const int *, const double *, double *,
                          const double *, const int *, const int *, double *,
                          double *, int *);
typedef void (*fn_dsteqr)(const char *, const int *, double *, double *,
                          double *, const int *, double *, int *, size_t);
typedef void (*fn_dlamrg)(const int *, const int *, const double *,
                          const int *, const int *, int *);
typedef void (*fn_dgemm)(const char *, const char *, const int *, const int *,
                         const int *, const double *, const double *,
                         const int *, const double *, const int *,
                         const double *, double *, const int *, size_t,
                         size_t);
typedef void (*fn_dstedc)(const char *, const int *, double *, double *,
                          double *, const int *, double *, const int *, int *,
                          const int *, int *, size_t);
typedef void (*fn_setthreads)(const int *);
typedef int (*fn_getthreads)(void);

struct Lapack {
  void *h = nullptr;
  fn_dlaed4 dlaed4 = nullptr;
  fn_dlaed3 dlaed3 = nullptr;
  fn_dsteqr dsteqr = nullptr;
  fn_dlamrg dlamrg = nullptr;
  fn_dgemm dgemm = nullptr;
  fn_dstedc dstedc = nullptr;
  fn_setthreads set_threads = nullptr;
  fn_getthreads get_threads = nullptr;
} L;

int g_threads = 1;
hso_stats g_stats;

void *sym(const char *base) {
  char name[128];
  const char *pats[] = {"scipy_%s_", "scipy_%s", "%s_", "%s"};
  for (const char *p : pats) {
    snprintf(name, sizeof name, p, base);
    void *f = dlsym(L.h, name);
    if (f) return f;
  }
  return nullptr;
}

const double EPS = 1.1102230246251565e-16;  // DLAMCH('Epsilon') = 2^-53

void dgemm(char ta, char tb, int m, int n, int k, double alpha,
           const double *A, int lda, const double *B, int ldb, double beta,
           double *C, int ldc) {
  if (m <= 0 || n <= 0) return;
  if (k <= 0) {
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < m; ++i)
        C[i + (size_t)j * ldc] = beta == 0.0 ? 0.0 : beta * C[i + (size_t)j * ldc];
    return;
  }
  L.dgemm(&ta, &tb, &m, &n, &k, &alpha, A, &lda, B, &ldb, &beta, C, &ldc, 1, 1);
}

// --------------------------------------------------------------- HSS tree ---
// npart / n2tree / btree / child / hsslevel / GetTreeInfo (aux_hss.f90:238-307,
// :664-827).  Nodes are numbered 1..ltr in post order; parent[root] = 0.
struct Tree {
  int lm = 0, ltr = 0, lvl = 0;
  std::vector<int> m;                  // leaf sizes, leaf order = post order
  std::vector<int> parent, c1, c2;     // size ltr+1
  std::vector<int> depth;              // root depth 0
  std::vector<std::vector<int>> ttr;   // ttr[L] (L = 1..lvl): nodes at depth L
  bool leaf(int i) const { return c1[i] == 0 && c2[i] == 0; }
  int sibling(int i) const {
    int p = parent[i];
    return c1[p] == i ? c2[p] : c1[p];
  }
};

// perfect post-order tree with n = 2^k - 1 nodes, ids offset by `off`
void perfect_tree(int n, int off, std::vector<int> &par) {
  if (n == 1) { par[off + 1] = 0; return; }
  int h = (n - 1) / 2;
  perfect_tree(h, off, par);
  perfect_tree(h, off + h, par);
  par[off + h] = off + n;
  par[off + 2 * h] = off + n;
  par[off + n] = 0;
}

// n2tree: a perfect left subtree of 2^floor(log2 n)-1 nodes, the remainder on
// the right, recursively (aux_hss.f90:737-760).
void n2tree(int n, int off, std::vector<int> &par) {
  if (n == 1) { par[off + 1] = 0; return; }
  int p2 = 1;
  while (p2 * 2 <= n) p2 *= 2;
  int n1 = p2 - 1;
  perfect_tree(n1, off, par);
  n2tree(n - n1 - 1, off + n1, par);
  par[off + n1] = off + n;
  par[off + n - 1] = off + n;
  par[off + n] = 0;
}

// npart (aux_hss.f90:803-827) + GetTreeInfo.
Tree make_tree(int n, int ni) {
  Tree t;
  int lm = n / ni;
  int mr = n % ni;
  if (lm == 0) {  // smaller than one leaf: a single leaf
    lm = 1;
    t.m.assign(1, n);
  } else {
    t.m.assign(lm, ni);
    if (mr >= ni / 2) {
      t.m.push_back(mr);
      ++lm;
    } else {
      t.m[lm - 1] += mr;
    }
  }
  t.lm = lm;
  t.ltr = 2 * lm - 1;
  t.parent.assign(t.ltr + 1, 0);
  n2tree(t.ltr, 0, t.parent);
  t.c1.assign(t.ltr + 1, 0);
  t.c2.assign(t.ltr + 1, 0);
  for (int i = 1; i < t.ltr; ++i) {
    int p = t.parent[i];
    if (t.c1[p] == 0) t.c1[p] = i; else t.c2[p] = i;
  }
  t.depth.assign(t.ltr + 1, 0);
  for (int i = t.ltr - 1; i >= 1; --i) t.depth[i] = t.depth[t.parent[i]] + 1;
  int lvl = 0;
  {  // lvl = ceiling(log2(ltr+1)) - 1  (CauchyHssEig.f90:2561)
    int p = 1;
    while (p < t.ltr + 1) { p *= 2; ++lvl; }
    lvl -= 1;
  }
  t.lvl = lvl;
  t.ttr.assign(lvl + 1, {});
  for (int j = 1; j < t.ltr; ++j) t.ttr[t.depth[j]].push_back(j);
  return t;
}

// --------------------------------------------- pole differences via DIFL/R ---
// computfd / computdd (CauchyHssEig.f90:470-568).  Indices are 0-based into
// FF (old poles), DIFL(j) = lam_j - FF_j > 0, DIFR(j) = lam_j - FF_{j+1} < 0.
struct Poles {
  const double *FF, *DIFL, *DIFR;
  // FF_p - lam_q
  inline double fd(int p, int q) const {
    return p <= q ? (FF[p] - FF[q]) - DIFL[q] : (FF[p] - FF[q + 1]) - DIFR[q];
  }
  // lam_p - lam_q
  inline double dd(int p, int q) const {
    return p < q ? (FF[p + 1] - FF[q]) + DIFR[p] - DIFL[q]
                 : (FF[p] - FF[q + 1]) + DIFL[p] - DIFR[q];
  }
};

// ----------------------------------------------- generators of one HSS ---
struct Gen {
  std::vector<std::vector<double>> D, U, V, B;
  std::vector<int> Dm, Ur, Uc, Vr, Vc, Br, Bc;
  void init(int ltr) {
    D.assign(ltr + 1, {}); U.assign(ltr + 1, {}); V.assign(ltr + 1, {});
    B.assign(ltr + 1, {});
    Dm.assign(ltr + 1, 0); Ur.assign(ltr + 1, 0); Uc.assign(ltr + 1, 0);
    Vr.assign(ltr + 1, 0); Vc.assign(ltr + 1, 0); Br.assign(ltr + 1, 0);
    Bc.assign(ltr + 1, 0);
  }
};

// CauchylikeEig (CauchyHssEig.f90:1688-1765): A(i,j) = u_i v_j / (F_{PL_i} - lam_{PU_j})
void cauchy_block(double *A, int lda, const Poles &P, const double *u,
                  const double *v, const int *PL, const int *PU, int M, int N) {
  for (int j = 0; j < N; ++j)
    for (int i = 0; i < M; ++i)
      A[i + (size_t)j * lda] = u[i] * v[j] / P.fd(PL[i], PU[j]);
}

template <class T>
inline void swp(T *a, int i, int j) { T t = a[i]; a[i] = a[j]; a[j] = t; }

// Structured strong rank-revealing LU on the generators of
//   C(i,j) = A_i V_j / (F_i - lam_j)           (row block of the eigenvector matrix)
// rrluCauchyEigrow (CauchyHssEig.f90:7-212) with the Gu-variant pivoting of
// CauchyPivtEig (:571-680), complete pivoting CauchyPivtEig_CP (:1001-1064) and
// periodic strong swaps searchMax2Eig (:1137-1212).
// Outputs: U (Schur row generators, first Rk unused), W (Rk), PQ, Rk.
int rrlu_row(double *F, double *Dv, double *A, double *V, const Poles &P,
             double tol, double *U, double *W, int *PL, int *PU, int M, int N,
             int *PQ, long long &nswap) {
  const double rho = 1.5;
  const int period = 10;
  for (int i = 0; i < M; ++i) { U[i] = A[i]; PQ[i] = i; }
  int mn = std::min(M, N);
  int Rk = mn;
  double Amax = 0.0;
  // column k of the Schur complement: max_i |U_i / (F_i - lam_k)|, i >= k
  auto colmax = [&](int k, int &arg) {
    double best = -1.0; arg = k;
    for (int i = k; i < M; ++i) {
      double t = std::fabs(U[i] / P.fd(PL[i], PU[k]));
      if (t > best) { best = t; arg = i; }
    }
    return best;
  };
  // row k: max_j |V_j / (F_k - lam_j)|, j >= k
  auto rowmax = [&](int k, int &arg) {
    double best = -1.0; arg = k;
    for (int j = k; j < N; ++j) {
      double t = std::fabs(V[j] / P.fd(PL[k], PU[j]));
      if (t > best) { best = t; arg = j; }
    }
    return best;
  };
  auto swap_row = [&](int a, int b) {
    swp(F, a, b); swp(U, a, b); swp(A, a, b); swp(PL, a, b); swp(PQ, a, b);
  };
  auto swap_col = [&](int a, int b) { swp(Dv, a, b); swp(V, a, b); swp(PU, a, b); };

  for (int k = 0; k < mn; ++k) {
    {  // Gu's variant of complete pivoting
      int jl, ju;
      double jkL = colmax(k, jl) * std::fabs(V[k]);
      double jkU = rowmax(k, ju) * std::fabs(U[k]);
      double piv = std::fabs(U[k] * V[k] / P.fd(PL[k], PU[k]));
      if (!(jkL <= piv && jkU <= piv)) {
        bool fromcol = jkL > jkU;
        for (int guard = 0; guard < 4 * (M + N) + 8; ++guard) {
          if (fromcol) {
            swap_row(k, jl);
            rowmax(k, ju);
            if (ju == k) break;
            fromcol = false;
          }
          swap_col(k, ju);
          colmax(k, jl);
          if (jl == k) break;
          fromcol = true;
        }
      }
    }
    double Ukk = U[k] * V[k] / P.fd(PL[k], PU[k]);
    Amax = std::max(Amax, std::fabs(Ukk));
    if (std::fabs(Ukk) < tol * Amax) {
      // complete pivoting over the whole Schur complement
      double best = -1.0;
      int bi = k, bj = k;
      for (int j = k; j < N; ++j) {
        double cm = -1.0;
        int a = k;
        for (int i = k; i < M; ++i) {
          double t = std::fabs(U[i] / P.fd(PL[i], PU[j]));
          if (t > cm) { cm = t; a = i; }
        }
        double t = std::fabs(cm * V[j]);
        if (j == k || t > best) { best = t; bi = a; bj = j; }
      }
      swap_row(k, bi);
      swap_col(k, bj);
      Ukk = U[k] * V[k] / P.fd(PL[k], PU[k]);
      Amax = std::max(Amax, std::fabs(Ukk));
      if (std::fabs(Ukk) < tol * Amax) { Rk = k; break; }
    }
    // Schur-complement generator updates
    for (int j = k + 1; j < M; ++j) U[j] *= (F[j] - F[k]) / P.fd(PL[j], PU[k]);
    for (int j = k + 1; j < N; ++j)
      V[j] *= P.dd(PU[j], PU[k]) / (-P.fd(PL[k], PU[j]));
    for (int j = 0; j < k; ++j) W[j] *= (-P.fd(PL[j], PU[k])) / (F[k] - F[j]);
    W[k] = P.fd(PL[k], PU[k]) / A[k];
    for (int j = 0; j < k; ++j) W[k] *= (-P.fd(PL[k], PU[j])) / (F[j] - F[k]);
    // strong swaps every `period` steps
    if ((k + 1) % period == 0) {
      for (int guard = 0; guard < M + 8; ++guard) {
        // max |Mat(i,j)| = |U_{k+1+i} W_j / (F_{k+1+i} - F_j)|
        double nmax = -1.0;
        int ii = 0, jj = k + 1;
        for (int j = 0; j <= k; ++j) {
          double cm = -1.0;
          int a = k + 1;
          for (int i = k + 1; i < M; ++i) {
            double t = std::fabs(U[i] / (F[i] - F[j]));
            if (t > cm) { cm = t; a = i; }
          }
          double t = cm * std::fabs(W[j]);
          if (j == 0 || t > nmax) { nmax = t; ii = j; jj = a; }
        }
        if (!(nmax > rho) || jj >= M) break;
        ++nswap;
        for (int j = k + 1; j < N; ++j)
          V[j] *= (-P.fd(PL[ii], PU[j])) / (-P.fd(PL[jj], PU[j]));
        for (int j = k + 1; j < M; ++j)
          if (j != jj) U[j] *= (F[j] - F[jj]) / (F[j] - F[ii]);
        for (int j = 0; j <= k; ++j)
          if (j != ii) W[j] *= (F[j] - F[ii]) / (F[j] - F[jj]);
        double ujj = A[ii] * ((F[ii] - F[jj]) / P.fd(PL[ii], PU[ii]));
        double wii = P.fd(PL[jj], PU[ii]) / A[jj];
        for (int j = 0; j <= k; ++j) {
          if (j == ii) continue;
          ujj *= (F[ii] - F[j]) / P.fd(PL[ii], PU[j]);
          wii *= (-P.fd(PL[jj], PU[j])) / (F[j] - F[jj]);
        }
        U[jj] = ujj;
        W[ii] = wii;
        swp(PL, ii, jj); swp(PQ, ii, jj); swp(F, ii, jj); swp(A, ii, jj);
      }
    }
  }
  return Rk;
}

// Column version: C(i,j) = A_i V_j / (lam_i - F_j), rows are eigenvalue poles.
// rrluCauchyEigcol (CauchyHssEig.f90:215-467), CauchyPivtEigm (:683-792),
// CauchyPivtEigm_CP (:795-1000), searchMax2Eigm (:1215-1286).
// PL: indices into lam for rows, PU: indices into FF for columns.
int rrlu_col(double *Dv, double *F, double *A, double *V, const Poles &P,
             double tol, double *U, double *W, int *PL, int *PU, int M, int N,
             int *PQ, long long &nswap) {
  const double rho = 1.5;
  const int period = 10;
  for (int i = 0; i < M; ++i) { U[i] = A[i]; PQ[i] = i; }
  int mn = std::min(M, N);
  int Rk = mn;
  double Amax = 0.0;
  // lam_{PL_i} - F_{PU_j} = -fd(PU_j, PL_i)
  auto den = [&](int i, int j) { return -P.fd(PU[j], PL[i]); };
  auto colmax = [&](int k, int &arg) {
    double best = -1.0; arg = k;
    for (int i = k; i < M; ++i) {
      double t = std::fabs(U[i] / den(i, k));
      if (t > best) { best = t; arg = i; }
    }
    return best;
  };
  auto rowmax = [&](int k, int &arg) {
    double best = -1.0; arg = k;
    for (int j = k; j < N; ++j) {
      double t = std::fabs(V[j] / den(k, j));
      if (t > best) { best = t; arg = j; }
    }
    return best;
  };
  auto swap_row = [&](int a, int b) {
    swp(Dv, a, b); swp(U, a, b); swp(A, a, b); swp(PL, a, b); swp(PQ, a, b);
  };
  auto swap_col = [&](int a, int b) { swp(F, a, b); swp(V, a, b); swp(PU, a, b); };

  for (int k = 0; k < mn; ++k) {
    {
      int jl, ju;
      double jkL = colmax(k, jl) * std::fabs(V[k]);
      double jkU = rowmax(k, ju) * std::fabs(U[k]);
      double piv = std::fabs(U[k] * V[k] / den(k, k));
      if (!(jkL <= piv && jkU <= piv)) {
        bool fromcol = jkL > jkU;
        for (int guard = 0; guard < 4 * (M + N) + 8; ++guard) {
          if (fromcol) {
            swap_row(k, jl);
            rowmax(k, ju);
            if (ju == k) break;
            fromcol = false;
          }
          swap_col(k, ju);
          colmax(k, jl);
          if (jl == k) break;
          fromcol = true;
        }
      }
    }
    double Ukk = U[k] * V[k] / den(k, k);
    Amax = std::max(Amax, std::fabs(Ukk));
    if (std::fabs(Ukk) < tol * Amax) {
      double best = -1.0;
      int bi = k, bj = k;
      for (int j = k; j < N; ++j) {
        double cm = -1.0;
        int a = k;
        for (int i = k; i < M; ++i) {
          double t = std::fabs(U[i] / den(i, j));
          if (t > cm) { cm = t; a = i; }
        }
        double t = std::fabs(cm * V[j]);
        if (j == k || t > best) { best = t; bi = a; bj = j; }
      }
      swap_row(k, bi);
      swap_col(k, bj);
      Ukk = U[k] * V[k] / den(k, k);
      Amax = std::max(Amax, std::fabs(Ukk));
      if (std::fabs(Ukk) < tol * Amax) { Rk = k; break; }
    }
    for (int j = k + 1; j < M; ++j)
      U[j] *= P.dd(PL[j], PL[k]) / den(j, k);                 // (D_j-D_k)/(D_j-F_k)
    for (int j = k + 1; j < N; ++j)
      V[j] *= (F[j] - F[k]) / P.fd(PU[j], PL[k]);             // (F_j-F_k)/(F_j-D_k)
    for (int j = 0; j < k; ++j)
      W[j] *= P.fd(PU[k], PL[j]) / P.dd(PL[k], PL[j]);        // (F_k-D_j)/(D_k-D_j)
    W[k] = den(k, k) / A[k];
    for (int j = 0; j < k; ++j)
      W[k] *= P.fd(PU[j], PL[k]) / P.dd(PL[j], PL[k]);        // (F_j-D_k)/(D_j-D_k)
    if ((k + 1) % period == 0) {
      for (int guard = 0; guard < M + 8; ++guard) {
        double nmax = -1.0;
        int ii = 0, jj = k + 1;
        for (int j = 0; j <= k; ++j) {
          double cm = -1.0;
          int a = k + 1;
          for (int i = k + 1; i < M; ++i) {
            double t = std::fabs(U[i] / P.dd(PL[i], PL[j]));
            if (t > cm) { cm = t; a = i; }
          }
          double t = cm * std::fabs(W[j]);
          if (j == 0 || t > nmax) { nmax = t; ii = j; jj = a; }
        }
        if (!(nmax > rho) || jj >= M) break;
        ++nswap;
        for (int j = k + 1; j < N; ++j)
          V[j] *= P.fd(PU[j], PL[ii]) / P.fd(PU[j], PL[jj]);
        for (int j = k + 1; j < M; ++j)
          if (j != jj) U[j] *= P.dd(PL[j], PL[jj]) / P.dd(PL[j], PL[ii]);
        for (int j = 0; j <= k; ++j)
          if (j != ii) W[j] *= P.dd(PL[j], PL[ii]) / P.dd(PL[j], PL[jj]);
        double ujj = A[ii] * (P.dd(PL[ii], PL[jj]) / den(ii, ii));
        double wii = -P.fd(PU[ii], PL[jj]) / A[jj];
        for (int j = 0; j <= k; ++j) {
          if (j == ii) continue;
          ujj *= P.dd(PL[ii], PL[j]) / (-P.fd(PU[j], PL[ii]));
          wii *= P.fd(PU[j], PL[jj]) / P.dd(PL[j], PL[jj]);
        }
        U[jj] = ujj;
        W[ii] = wii;
        swp(PL, ii, jj); swp(PQ, ii, jj); swp(Dv, ii, jj); swp(A, ii, jj);
      }
    }
  }
  return Rk;
}

// ComprcauchyEig (CauchyHssEig.f90:2253-2440), row case: returns the
// interpolation generator U_node (M x Rk, column-major) in the node's original
// row order; the node's row generators A and PL are permuted in place so that
// the first Rk are the skeleton rows.
int compress_rows(double *Fi, double *Di, double *A, double *Vi, const Poles &P,
                  int *PL, int *PUi, double tol, int M, int N,
                  std::vector<double> &Ug, long long &nswap) {
  int mn = std::min(M, N);
  std::vector<double> Z(M, 0.0), W(std::max(mn, 1), 0.0);
  std::vector<int> PQ(M);
  int Rk = rrlu_row(Fi, Di, A, Vi, P, tol, Z.data(), W.data(), PL, PUi, M, N,
                    PQ.data(), nswap);
  // PQ[i] = original row now at position i;  inverse: pos of original row r
  std::vector<int> inv(M);
  for (int i = 0; i < M; ++i) inv[PQ[i]] = i;
  if (Rk < mn) {
    Ug.assign((size_t)M * Rk, 0.0);
    // row r of result = row inv[r] of [I; Mat]
    for (int r = 0; r < M; ++r) {
      int p = inv[r];
      for (int j = 0; j < Rk; ++j) {
        double v;
        if (p < Rk) v = (p == j) ? 1.0 : 0.0;
        else v = Z[p] * W[j] / (Fi[p] - Fi[j]);   // CauchylikeEigQ (:1872-1942)
        Ug[r + (size_t)j * M] = v;
      }
    }
  } else {
    Rk = M;
    Ug.assign((size_t)M * M, 0.0);
    for (int r = 0; r < M; ++r) Ug[r + (size_t)inv[r] * M] = 1.0;
  }
  return Rk;
}

// ComprcauchyEig, column case: V_node (Rk x N) in the node's original column order.
int compress_cols(double *Fi, double *Dn, double *Ui, double *Vn, const Poles &P,
                  int *PLi, int *PUn, double tol, int M, int N,
                  std::vector<double> &Vg, long long &nswap) {
  int mn = std::min(M, N);
  std::vector<double> Z(N, 0.0), W(std::max(mn, 1), 0.0);
  std::vector<int> PQ(N);
  // transpose view: rows = node columns (lam poles), columns = other rows (F poles)
  int Rk = rrlu_col(Dn, Fi, Vn, Ui, P, tol, Z.data(), W.data(), PUn, PLi, N, M,
                    PQ.data(), nswap);
  std::vector<int> inv(N);
  for (int i = 0; i < N; ++i) inv[PQ[i]] = i;
  if (Rk < mn) {
    Vg.assign((size_t)Rk * N, 0.0);
    for (int c = 0; c < N; ++c) {
      int p = inv[c];
      for (int i = 0; i < Rk; ++i) {
        double v;
        if (p < Rk) v = (p == i) ? 1.0 : 0.0;
        else v = -W[i] * Z[p] / P.dd(PUn[i], PUn[p]);  // CauchylikeEigQ2 (:1768-1869)
        Vg[i + (size_t)c * Rk] = v;
      }
    }
  } else {
    Rk = N;
    Vg.assign((size_t)N * N, 0.0);
    for (int c = 0; c < N; ++c) Vg[inv[c] + (size_t)c * N] = 1.0;
  }
  return Rk;
}

// Cauchy2hssEig_omp (CauchyHssEig.f90:1945-2250): HSS generators of
// C(i,j) = u_i v_j / (F_i - lam_j), K x K.
void cauchy2hss_eig(const Tree &t, int K, const Poles &P, const double *u0,
                    const double *v0, double tol, Gen &g, long long &nswap) {
  g.init(t.ltr);
  std::vector<double> U(u0, u0 + K), V(v0, v0 + K), D(K);
  std::vector<int> PL(K), PU(K);
  for (int i = 0; i < K; ++i) { PL[i] = i; PU[i] = i; }
  // D holds lam values only for bookkeeping (never used in arithmetic)
  for (int i = 0; i < K; ++i) D[i] = P.FF[i] + P.DIFL[i];
  std::vector<int> lr0(t.ltr + 1), lr1(t.ltr + 1), lc0, lc1;
  {
    int lt = 0, it = 0;
    for (int i = 1; i <= t.ltr; ++i) {
      if (t.leaf(i)) { lr0[i] = lt; lr1[i] = lt + t.m[it] - 1; lt += t.m[it]; ++it; }
      else { lr0[i] = lr0[t.c1[i]]; lr1[i] = lr1[t.c2[i]]; }
    }
  }
  lc0 = lr0; lc1 = lr1;
  // leaf diagonal blocks
  for (int i = 1; i <= t.ltr; ++i) {
    if (!t.leaf(i)) continue;
    int mi = lr1[i] - lr0[i] + 1;
    g.D[i].assign((size_t)mi * mi, 0.0);
    g.Dm[i] = mi;
    cauchy_block(g.D[i].data(), mi, P, &U[lr0[i]], &V[lr0[i]], &PL[lr0[i]],
                 &PU[lr0[i]], mi, mi);
  }
  int lda = K, lca = K;
  for (int LL = t.lvl; LL >= 1; --LL) {
    const std::vector<int> &nodes = t.ttr[LL];
    const int nn = (int)nodes.size();
    for (int nodi : nodes)
      if (!t.leaf(nodi)) {
        lr0[nodi] = lr0[t.c1[nodi]]; lr1[nodi] = lr1[t.c2[nodi]];
        lc0[nodi] = lc0[t.c1[nodi]]; lc1[nodi] = lc1[t.c2[nodi]];
      }
    // ---- row compression (each node against all other current columns)
    std::vector<long long> sw(nn, 0);
#pragma omp parallel for schedule(dynamic) num_threads(g_threads)
    for (int a = 0; a < nn; ++a) {
      int nodi = nodes[a];
      int mi = lr1[nodi] - lr0[nodi] + 1;
      int ncol = lc1[nodi] - lc0[nodi] + 1;
      int nt = lca - ncol;
      std::vector<int> PUi(nt);
      std::vector<double> Vi(nt), Di(nt), Fi(mi);
      int q = 0;
      for (int j = 0; j < lca; ++j)
        if (j < lc0[nodi] || j > lc1[nodi]) { PUi[q] = PU[j]; Vi[q] = V[j]; Di[q] = D[j]; ++q; }
      for (int i = 0; i < mi; ++i) Fi[i] = P.FF[PL[lr0[nodi] + i]];
      int Rk = compress_rows(Fi.data(), Di.data(), &U[lr0[nodi]], Vi.data(), P,
                             &PL[lr0[nodi]], PUi.data(), tol, mi, nt, g.U[nodi], sw[a]);
      g.Ur[nodi] = mi;
      g.Uc[nodi] = Rk;
    }
    for (long long s : sw) nswap += s;
    // ---- compact rows: skeletons of this level, then untouched leaves above
    {
      std::vector<double> Un; std::vector<int> PLn;
      for (int nodi : nodes) {
        int Rk = g.Uc[nodi], b = lr0[nodi];
        lr0[nodi] = (int)Un.size(); lr1[nodi] = lr0[nodi] + Rk - 1;
        for (int i = 0; i < Rk; ++i) { Un.push_back(U[b + i]); PLn.push_back(PL[b + i]); }
      }
      for (int LLt = LL - 1; LLt >= 1; --LLt)
        for (int nodi : t.ttr[LLt])
          if (t.leaf(nodi)) {
            int mi = lr1[nodi] - lr0[nodi] + 1, b = lr0[nodi];
            lr0[nodi] = (int)Un.size(); lr1[nodi] = lr0[nodi] + mi - 1;
            for (int i = 0; i < mi; ++i) { Un.push_back(U[b + i]); PLn.push_back(PL[b + i]); }
          }
      lda = (int)Un.size();
      std::copy(Un.begin(), Un.end(), U.begin());
      std::copy(PLn.begin(), PLn.end(), PL.begin());
    }
    // ---- column compression (each node against all other current rows)
#pragma omp parallel for schedule(dynamic) num_threads(g_threads)
    for (int a = 0; a < nn; ++a) {
      int nodi = nodes[a];
      int mc = lc1[nodi] - lc0[nodi] + 1;
      int nr = lr1[nodi] - lr0[nodi] + 1;
      int nt = lda - nr;
      std::vector<int> PLi(nt);
      std::vector<double> Ui(nt), Fi(nt);
      int q = 0;
      for (int i = 0; i < lda; ++i)
        if (i < lr0[nodi] || i > lr1[nodi]) { PLi[q] = PL[i]; Ui[q] = U[i]; Fi[q] = P.FF[PL[i]]; ++q; }
      long long s = 0;
      int Rk = compress_cols(Fi.data(), &D[lc0[nodi]], Ui.data(), &V[lc0[nodi]], P,
                             PLi.data(), &PU[lc0[nodi]], tol, nt, mc, g.V[nodi], s);
      sw[a] = s;
      g.Vr[nodi] = Rk;
      g.Vc[nodi] = mc;
    }
    for (long long s : sw) nswap += s;
    {
      std::vector<double> Vn, Dn; std::vector<int> PUn;
      for (int nodi : nodes) {
        int Rk = g.Vr[nodi], b = lc0[nodi];
        lc0[nodi] = (int)Vn.size(); lc1[nodi] = lc0[nodi] + Rk - 1;
        for (int i = 0; i < Rk; ++i) { Vn.push_back(V[b + i]); Dn.push_back(D[b + i]); PUn.push_back(PU[b + i]); }
      }
      for (int LLt = LL - 1; LLt >= 1; --LLt)
        for (int nodi : t.ttr[LLt])
          if (t.leaf(nodi)) {
            int mc = lc1[nodi] - lc0[nodi] + 1, b = lc0[nodi];
            lc0[nodi] = (int)Vn.size(); lc1[nodi] = lc0[nodi] + mc - 1;
            for (int i = 0; i < mc; ++i) { Vn.push_back(V[b + i]); Dn.push_back(D[b + i]); PUn.push_back(PU[b + i]); }
          }
      lca = (int)Vn.size();
      std::copy(Vn.begin(), Vn.end(), V.begin());
      std::copy(Dn.begin(), Dn.end(), D.begin());
      std::copy(PUn.begin(), PUn.end(), PU.begin());
    }
    // ---- B generators: skeleton rows of nodi x skeleton columns of its sibling
    for (int nodi : nodes) {
      int nodj = t.sibling(nodi);
      int mi = lr1[nodi] - lr0[nodi] + 1;
      int nj = lc1[nodj] - lc0[nodj] + 1;
      g.B[nodi].assign((size_t)std::max(mi, 0) * std::max(nj, 0), 0.0);
      g.Br[nodi] = mi;
      g.Bc[nodi] = nj;
      if (mi > 0 && nj > 0)
        cauchy_block(g.B[nodi].data(), mi, P, &U[lr0[nodi]], &V[lc0[nodj]],
                     &PL[lr0[nodi]], &PU[lc0[nodj]], mi, nj);
    }
  }
}

// fastHssmmL_omp (ConstructHssd.f90:1394-1630): X (nrows x K, ld ldx) <- X * H.
void hss_mm_left(const Tree &t, const Gen &g, double *X, int ldx, int nrows) {
  if (nrows <= 0) return;
  const int ltr = t.ltr;
  std::vector<int> lx(ltr + 1, 0), lg(ltr + 1, 0), lf(ltr + 1, 0);
  {
    int lt = 0, it = 0;
    for (int i = 1; i <= ltr; ++i)
      if (t.leaf(i)) { lx[i] = lt; lt += t.m[it++]; }
  }
  if (t.lm == 1) {  // single leaf: X <- X * D
    std::vector<double> T((size_t)nrows * g.Dm[ltr]);
    int m = g.Dm[ltr];
    dgemm('N', 'N', nrows, m, m, 1.0, X, ldx, g.D[ltr].data(), m, 0.0, T.data(), nrows);
    for (int j = 0; j < m; ++j)
      std::memcpy(X + (size_t)j * ldx, T.data() + (size_t)j * nrows, sizeof(double) * nrows);
    return;
  }
  int ncg = 0;
  for (int LL = t.lvl; LL >= 1; --LL)
    for (int ni : t.ttr[LL]) { lg[ni] = ncg; ncg += g.Uc[ni]; }
  int ncf = 0;
  for (int LL = 1; LL <= t.lvl; ++LL)
    for (int ni : t.ttr[LL]) { lf[ni] = ncf; ncf += g.Bc[t.sibling(ni)]; }
  std::vector<double> G((size_t)nrows * std::max(ncg, 1), 0.0),
      F((size_t)nrows * std::max(ncf, 1), 0.0);
  // upsweep: G_i = X_i U_i (leaf), G_p = [G_c1 G_c2] U_p
  for (int LL = t.lvl; LL >= 1; --LL)
    for (int ni : t.ttr[LL]) {
      if (t.leaf(ni))
        dgemm('N', 'N', nrows, g.Uc[ni], g.Ur[ni], 1.0, X + (size_t)lx[ni] * ldx, ldx,
              g.U[ni].data(), g.Ur[ni], 0.0, G.data() + (size_t)lg[ni] * nrows, nrows);
      else
        dgemm('N', 'N', nrows, g.Uc[ni], g.Ur[ni], 1.0,
              G.data() + (size_t)lg[t.c1[ni]] * nrows, nrows, g.U[ni].data(),
              g.Ur[ni], 0.0, G.data() + (size_t)lg[ni] * nrows, nrows);
    }
  // downsweep: F_i (+)= G_j B_j (j = sibling), F_children = F_i V_i
  for (int LL = 1; LL <= t.lvl; ++LL)
    for (int ni : t.ttr[LL]) {
      int nj = t.sibling(ni);
      dgemm('N', 'N', nrows, g.Bc[nj], g.Br[nj], 1.0, G.data() + (size_t)lg[nj] * nrows,
            nrows, g.B[nj].data(), std::max(g.Br[nj], 1), LL == 1 ? 0.0 : 1.0,
            F.data() + (size_t)lf[ni] * nrows, nrows);
      if (!t.leaf(ni))
        dgemm('N', 'N', nrows, g.Vc[ni], g.Vr[ni], 1.0, F.data() + (size_t)lf[ni] * nrows,
              nrows, g.V[ni].data(), std::max(g.Vr[ni], 1), 0.0,
              F.data() + (size_t)lf[t.c1[ni]] * nrows, nrows);
    }
  // leaves: X_i <- F_i V_i + X_i D_i
  std::vector<double> T;
  for (int ni = 1; ni < ltr; ++ni) {
    if (!t.leaf(ni)) continue;
    int m = g.Dm[ni];
    T.assign((size_t)nrows * m, 0.0);
    dgemm('N', 'N', nrows, g.Vc[ni], g.Vr[ni], 1.0, F.data() + (size_t)lf[ni] * nrows,
          nrows, g.V[ni].data(), std::max(g.Vr[ni], 1), 0.0, T.data(), nrows);
    dgemm('N', 'N', nrows, m, m, 1.0, X + (size_t)lx[ni] * ldx, ldx, g.D[ni].data(), m,
          1.0, T.data(), nrows);
    for (int j = 0; j < m; ++j)
      std::memcpy(X + (size_t)(lx[ni] + j) * ldx, T.data() + (size_t)j * nrows,
                  sizeof(double) * nrows);
  }
}

int max_rank(const Tree &t, const Gen &g) {
  int r = 0;
  for (int i = 1; i < t.ltr; ++i) r = std::max(r, std::max(g.Uc[i], g.Vr[i]));
  return r;
}

// DHSSEVC (CauchyHssEig.f90:2444-2598)
int dhssevc(int K, int ni, double tol, const double *F, const double *u,
            const double *v, const double *difl, const double *difr, double *Q,
            int ldq, int nrows, int *mr) {
  Poles P{F, difl, difr};
  Tree t = make_tree(K, ni);
  Gen g;
  long long sw = 0;
  cauchy2hss_eig(t, K, P, u, v, tol, g, sw);
  g_stats.n_swaps += sw;
  hss_mm_left(t, g, Q, ldq, nrows);
  int r = max_rank(t, g);
  g_stats.max_rank = std::max(g_stats.max_rank, r);
  if (mr) *mr = r;
  return 0;
}

// ------------------------------------------------------- secular + Loewner ---
// MDLAED3 steps 1-2 (mdlaed3.f90:196-249).
int secular_lowner(int K, const double *dlamda, double *z, double rho,
                   double *lam, double *difl, double *difr, double *alpha) {
  std::vector<double> prod(K, 1.0);
  int err = 0;
#pragma omp parallel num_threads(g_threads)
  {
    std::vector<double> delta(K + 1), lprod(K, 1.0);
#pragma omp for schedule(static)
    for (int j = 0; j < K; ++j) {
      int jj = j + 1, info = 0;
      L.dlaed4(&K, &jj, dlamda, z, delta.data(), &rho, &lam[j], &info);
      if (info != 0) {
#pragma omp atomic write
        err = jj;
      }
      if (K > 2) {
        difl[j] = -delta[j];
        difr[j] = (j + 1 < K) ? -delta[j + 1] : 0.0;
      } else {
        // for N <= 2 LAPACK's DELTA holds eigenvector data, not d_i - lam
        difl[j] = lam[j] - dlamda[j];
        difr[j] = (j + 1 < K) ? lam[j] - dlamda[j + 1] : 0.0;
      }
      lprod[j] *= delta[j];
      for (int i = 0; i < K; ++i)
        if (i != j) lprod[i] *= delta[i] / (dlamda[i] - dlamda[j]);
    }
#pragma omp critical
    for (int i = 0; i < K; ++i) prod[i] *= lprod[i];
  }
  if (err) return err;
  for (int i = 0; i < K; ++i) z[i] = std::copysign(std::sqrt(std::fabs(prod[i])), z[i]);
  if (alpha) {
    Poles P{dlamda, difl, difr};
#pragma omp parallel for schedule(static) num_threads(g_threads)
    for (int j = 0; j < K; ++j) {
      double s = 0.0;
      for (int i = 0; i < K; ++i) {
        double w = z[i] / P.fd(i, j);
        s += w * w;
      }
      alpha[j] = 1.0 / std::sqrt(s);
    }
  }
  return 0;
}

// ---------------------------------------------------------- DC merge ------
struct Ws {
  hso_config cfg;
};

// DLAMRG (via LAPACK)
void lamrg(int n1, int n2, const double *a, int s1, int s2, int *idx) {
  L.dlamrg(&n1, &n2, a, &s1, &s2, idx);
}

// MDLAED2 (mdlaed2.f90:149-528) + MDLAED3 / DLAED3, i.e. one MDLAED1 merge
// (mdlaed1.f90:109-233).  Arrays are local to the merge: D(n), Q(ldq, n) block,
// indxq(n) 1-based LAPACK permutation (as DLAMRG produces).
int merge(int n, int n1, double *D, double *Q, int ldq, int *indxq, double rho,
          const hso_config &cfg) {
  const int n2 = n - n1;
  std::vector<double> z(n), dlamda(n), w(n);
  std::vector<int> indx(n), indxc(n), indxp(n), coltyp(n);
  // z: last row of Q1 and first row of Q2 (mdlaed1.f90:178-180)
  for (int j = 0; j < n1; ++j) z[j] = Q[(n1 - 1) + (size_t)j * ldq];
  for (int j = n1; j < n; ++j) z[j] = Q[n1 + (size_t)j * ldq];
  g_stats.n_merges++;
  // ---- MDLAED2
  if (rho < 0.0) for (int j = n1; j < n; ++j) z[j] = -z[j];
  const double t0 = 1.0 / std::sqrt(2.0);
  for (int j = 0; j < n; ++j) z[j] *= t0;
  rho = std::fabs(2.0 * rho);
  for (int i = n1; i < n; ++i) indxq[i] += n1;
  for (int i = 0; i < n; ++i) dlamda[i] = D[indxq[i] - 1];
  lamrg(n1, n2, dlamda.data(), 1, 1, indxc.data());
  for (int i = 0; i < n; ++i) indx[i] = indxq[indxc[i] - 1] - 1;  // 0-based
  double zmax = 0.0, dmax = 0.0;
  for (int i = 0; i < n; ++i) { zmax = std::max(zmax, std::fabs(z[i])); dmax = std::max(dmax, std::fabs(D[i])); }
  const double tol = 8.0 * EPS * std::max(dmax, zmax);
  int K = 0;
  std::vector<double> Q2;
  if (rho * zmax <= tol) {
    // nothing to merge: reorder columns by indx
    Q2.assign((size_t)n * n, 0.0);
    for (int j = 0; j < n; ++j) {
      int c = indx[j];
      for (int i = 0; i < n; ++i) Q2[i + (size_t)j * n] = Q[i + (size_t)c * ldq];
      dlamda[j] = D[c];
    }
    for (int j = 0; j < n; ++j) {
      for (int i = 0; i < n; ++i) Q[i + (size_t)j * ldq] = Q2[i + (size_t)j * n];
      D[j] = dlamda[j];
    }
    for (int i = 0; i < n; ++i) indxq[i] = i + 1;
    return 0;
  }
  for (int i = 0; i < n; ++i) coltyp[i] = i < n1 ? 1 : 3;
  int k2 = n;  // deflated entries fill indxp[k2..n-1] from the back
  int j = 0, pj = -1;
  for (; j < n; ++j) {
    int nj = indx[j];
    if (rho * std::fabs(z[nj]) <= tol) { coltyp[nj] = 4; indxp[--k2] = nj; }
    else { pj = nj; break; }
  }
  for (++j; j < n; ++j) {
    int nj = indx[j];
    if (rho * std::fabs(z[nj]) <= tol) { coltyp[nj] = 4; indxp[--k2] = nj; continue; }
    double s = z[pj], c = z[nj];
    double tau = std::hypot(c, s);
    double t = D[nj] - D[pj];
    c /= tau; s = -s / tau;
    if (std::fabs(t * c * s) <= tol) {
      // deflation by a Givens rotation of columns pj, nj
      z[nj] = tau; z[pj] = 0.0;
      if (coltyp[nj] != coltyp[pj]) coltyp[nj] = 2;
      coltyp[pj] = 4;
      double *x = Q + (size_t)pj * ldq, *y = Q + (size_t)nj * ldq;
      for (int i = 0; i < n; ++i) {
        double xi = x[i], yi = y[i];
        x[i] = c * xi + s * yi;
        y[i] = c * yi - s * xi;
      }
      double tt = D[pj] * c * c + D[nj] * s * s;
      D[nj] = D[pj] * s * s + D[nj] * c * c;
      D[pj] = tt;
      --k2;
      int i = k2;
      while (i + 1 < n && D[pj] < D[indxp[i + 1]]) { indxp[i] = indxp[i + 1]; ++i; }
      indxp[i] = pj;
      pj = nj;
    } else {
      dlamda[K] = D[pj]; w[K] = z[pj]; indxp[K] = pj; ++K;
      pj = nj;
    }
  }
  if (pj < 0) return -100;  // unreachable: rho*max|z| > tol keeps one pole
  dlamda[K] = D[pj]; w[K] = z[pj]; indxp[K] = pj; ++K;
  int ctot[5] = {0, 0, 0, 0, 0};
  for (int i = 0; i < n; ++i) ctot[coltyp[i]]++;
  K = n - ctot[4];
  g_stats.max_k = std::max(g_stats.max_k, K);
  g_stats.total_k += K;
  std::vector<double> zt(n);
  const bool hflag = K < cfg.bsmlz;
  if (hflag) {
    // group columns by type 1,2,3,4 (mdlaed2.f90:469-508)
    int psm[5];
    psm[1] = 0; psm[2] = ctot[1]; psm[3] = psm[2] + ctot[2]; psm[4] = psm[3] + ctot[3];
    for (int jj = 0; jj < n; ++jj) {
      int js = indxp[jj], ct = coltyp[js];
      indx[psm[ct]] = js;
      indxc[psm[ct]] = jj + 1;
      psm[ct]++;
    }
    Q2.assign((size_t)n * n + 1, 0.0);
    size_t iq1 = 0, iq2 = (size_t)(ctot[1] + ctot[2]) * n1;
    int i = 0;
    for (int a = 0; a < ctot[1]; ++a, ++i) {
      int js = indx[i];
      std::memcpy(&Q2[iq1], Q + (size_t)js * ldq, sizeof(double) * n1); iq1 += n1;
      zt[i] = D[js];
    }
    for (int a = 0; a < ctot[2]; ++a, ++i) {
      int js = indx[i];
      std::memcpy(&Q2[iq1], Q + (size_t)js * ldq, sizeof(double) * n1); iq1 += n1;
      std::memcpy(&Q2[iq2], Q + n1 + (size_t)js * ldq, sizeof(double) * n2); iq2 += n2;
      zt[i] = D[js];
    }
    for (int a = 0; a < ctot[3]; ++a, ++i) {
      int js = indx[i];
      std::memcpy(&Q2[iq2], Q + n1 + (size_t)js * ldq, sizeof(double) * n2); iq2 += n2;
      zt[i] = D[js];
    }
    size_t iqd = iq2;
    for (int a = 0; a < ctot[4]; ++a, ++i) {
      int js = indx[i];
      std::memcpy(&Q2[iq2], Q + (size_t)js * ldq, sizeof(double) * n); iq2 += n;
      zt[i] = D[js];
    }
    for (int a = 0; a < ctot[4]; ++a)
      std::memcpy(Q + (size_t)(K + a) * ldq, &Q2[iqd + (size_t)a * n], sizeof(double) * n);
    for (int a = K; a < n; ++a) D[a] = zt[a];
    if (K > 0) {
      g_stats.n_dense_merges++;
      int info = 0;
      int ctot4[4] = {ctot[1], ctot[2], ctot[3], ctot[4]};
      std::vector<double> S((size_t)std::max(n1, n2) * K + (size_t)K * K + 16);
      L.dlaed3(&K, &n, &n1, D, Q, &ldq, &rho, dlamda.data(), Q2.data(), indxc.data(),
               ctot4, w.data(), S.data(), &info);
      if (info) return info;
    }
  } else {
    // HSS path: full columns, nondeflated first (mdlaed2.f90:456-499)
    Q2.assign((size_t)n * n, 0.0);
    for (int jj = 0; jj < n; ++jj) {
      int js = indxp[jj];
      std::memcpy(&Q2[(size_t)jj * n], Q + (size_t)js * ldq, sizeof(double) * n);
      zt[jj] = D[js];
    }
    for (int jj = 0; jj < n; ++jj)
      std::memcpy(Q + (size_t)jj * ldq, &Q2[(size_t)jj * n], sizeof(double) * n);
    for (int a = K; a < n; ++a) D[a] = zt[a];
    g_stats.n_hss_merges++;
    // ---- MDLAED3 (mdlaed3.f90:124-261)
    std::vector<double> difl(K), difr(K), alpha(K), zz(w.begin(), w.begin() + K);
    int info = secular_lowner(K, dlamda.data(), zz.data(), rho, D, difl.data(),
                              difr.data(), alpha.data());
    if (info) return info;
    int mr = 0;
    dhssevc(K, cfg.hss_leaf, cfg.tol, dlamda.data(), zz.data(), alpha.data(),
            difl.data(), difr.data(), Q2.data(), n, n, &mr);
    for (int jj = 0; jj < K; ++jj)
      std::memcpy(Q + (size_t)jj * ldq, &Q2[(size_t)jj * n], sizeof(double) * n);
  }
  // INDXQ for the merged list (mdlaed1.f90:221)
  lamrg(K, n - K, D, 1, -1, indxq);
  return 0;
}

// MDLAED0 with ICOMPQ = 2 (mdlaed0.f90:121-380): eigen-decomposition of the
// unreduced tridiagonal (d, e) of size n into Q (ldq).
int laed0(int n, double *d, double *e, double *Q, int ldq, const hso_config &cfg) {
  // halving tree (mdlaed0.f90:192-208): split every block until the last
  // (largest, since right halves take the ceiling) is at most SMLSIZ
  std::vector<int> sz(1, n);
  while (sz.back() > cfg.smlsiz) {
    std::vector<int> nx;
    for (int s : sz) { nx.push_back(s / 2); nx.push_back((s + 1) / 2); }
    sz.swap(nx);
  }
  int subpbs = (int)sz.size();
  std::vector<int> endp(subpbs);
  for (int j = 0, acc = 0; j < subpbs; ++j) { acc += sz[j]; endp[j] = acc; }
  // rank-one cuts (mdlaed0.f90:213-219)
  for (int i = 0; i + 1 < subpbs; ++i) {
    int sm1 = endp[i] - 1;  // 0-based last row of block i
    d[sm1] -= std::fabs(e[sm1]);
    d[sm1 + 1] -= std::fabs(e[sm1]);
  }
  std::vector<int> indxq(n);
  std::vector<double> work(std::max(1, 2 * cfg.smlsiz + 2));
  for (int i = 0; i < subpbs; ++i) {
    int s = i == 0 ? 0 : endp[i - 1];
    int m = endp[i] - s;
    int info = 0;
    char cz = 'I';
    work.resize(std::max<size_t>(work.size(), 2 * (size_t)m + 2));
    L.dsteqr(&cz, &m, d + s, e + s, Q + s + (size_t)s * ldq, &ldq, work.data(), &info, 1);
    if (info) return (s + 1) * (n + 1) + s + m;
    for (int j = 0; j < m; ++j) indxq[s + j] = j + 1;
  }
  // merge levels (mdlaed0.f90:294-341)
  std::vector<int> ends(endp);
  while ((int)ends.size() > 1) {
    std::vector<int> nx;
    for (size_t i = 0; i + 1 < ends.size(); i += 2) {
      int s = i == 0 ? 0 : ends[i - 1];
      int matsiz = ends[i + 1] - s;
      int msd2 = i == 0 ? ends[0] : matsiz / 2;
      int info = merge(matsiz, msd2, d + s, Q + s + (size_t)s * ldq, ldq, &indxq[s],
                       e[s + msd2 - 1], cfg);
      if (info) return (s + 1) * (n + 1) + s + matsiz;
      nx.push_back(ends[i + 1]);
    }
    ends.swap(nx);
  }
  // final permutation (mdlaed0.f90:355-362)
  std::vector<double> dw(n), qw((size_t)n * n);
  for (int i = 0; i < n; ++i) {
    int jx = indxq[i] - 1;
    dw[i] = d[jx];
    std::memcpy(&qw[(size_t)i * n], Q + (size_t)jx * ldq, sizeof(double) * n);
  }
  std::memcpy(d, dw.data(), sizeof(double) * n);
  for (int i = 0; i < n; ++i)
    std::memcpy(Q + (size_t)i * ldq, &qw[(size_t)i * n], sizeof(double) * n);
  return 0;
}

// ---------------------------------------------- generic Cauchy HSS (VP2) ---
// Module CauchyHss_VP2 (SRC/CauchyHss_VP2.f90) for C(i,j) = u_i v_j / (D_i - F_j)
// with plain pole differences (no DIFL/DIFR), as SRC/cauchyhssmm.f90 uses it.
// Indices are 0-based; k below is the 0-based step (Fortran k - 1).

// CauchyMax (:166-185): largest |u_i / (D_i - F)|, i < n, first index on ties.
void vp2_cmax(const double *D, double F, const double *u, int n, double &junk, int &jj) {
  junk = -1.0;
  jj = 0;
  for (int i = 0; i < n; ++i) {
    const double t = std::fabs(u[i] / (D[i] - F));
    if (t > junk) { junk = t; jj = i; }
  }
}

// CauchyPivtG (:187-236): alternate row / column maxima until the pivot is
// the largest entry of its row and its column.  Fortran's `continue` after the
// row swap is a no-op, so a row swap is always followed by a column swap.
void vp2_pivt(double *D, double *F, double *u, double *v, int *PL, int *PU, int k, double *A,
              int M, int N) {
  double junkL, junkU;
  int jjL, jjU;
  vp2_cmax(D + k, F[k], u + k, M - k, junkL, jjL);
  vp2_cmax(F + k, D[k], v + k, N - k, junkU, jjU);
  junkL *= std::fabs(v[k]);
  junkU *= std::fabs(u[k]);
  const double piv = std::fabs(u[k] * v[k] / (D[k] - F[k]));
  if (junkL <= piv && junkU <= piv) return;
  bool flg = junkL > junkU;
  for (int guard = 0; guard < 4 * (M + N) + 8; ++guard) {  // the Fortran loop is unbounded
    if (flg) {
      const int jj = jjL;
      swp(D, k, jj + k); swp(u, k, jj + k); swp(A, k, jj + k); swp(PL, k, jj + k);
      vp2_cmax(F + k, D[k], v + k, N - k, junkU, jjU);
      if (jjU == 0) return;
    }
    const int jj = jjU;
    swp(F, k, jj + k); swp(v, k, jj + k); swp(PU, k, jj + k);
    vp2_cmax(D + k, F[k], u + k, M - k, junkL, jjL);
    if (jjL == 0) return;
    flg = true;
  }
}

// CauchyPivtG_CP (:239-290): complete pivoting over the Schur complement.
void vp2_pivt_cp(double *D, double *F, double *u, double *v, int *PL, int *PU, int k, double *A,
                 int M, int N) {
  double best = -1.0;
  int ii = 0, jj = 0;
  for (int j = 0; j < N - k; ++j) {
    double t;
    int a;
    vp2_cmax(D + k, F[k + j], u + k, M - k, t, a);
    t = std::fabs(t * v[k + j]);
    if (j == 0 || t > best) { best = t; ii = a; jj = j; }
  }
  swp(D, k, ii + k); swp(u, k, ii + k); swp(A, k, ii + k); swp(PL, k, ii + k);
  swp(F, k, jj + k); swp(v, k, jj + k); swp(PU, k, jj + k);
}

// searchMax2 (:135-163): the largest |U2_i W_j / (D2_i - D1_j)| over i < ldu,
// j < ldw; ii = column j, jj = row i (relative to U2/D2).
void vp2_search(const double *U2, const double *W, const double *D2, const double *D1, int ldu,
                int ldw, int &ii, int &jj, double &nmax) {
  double junk;
  int jjl;
  vp2_cmax(D2, D1[0], U2, ldu, junk, jjl);
  nmax = junk * std::fabs(W[0]);
  ii = 0;
  jj = jjl;
  for (int j = 1; j < ldw; ++j) {
    vp2_cmax(D2, D1[j], U2, ldu, junk, jjl);
    junk *= std::fabs(W[j]);
    if (junk > nmax) { nmax = junk; ii = j; jj = jjl; }
  }
}

// rrluCauchy (:7-134): structured strong RRLU with rho = 1.02, swaps checked
// every 10 steps.  A (row generators) and D are permuted in place; U receives
// the Schur row generators (last M - Rk used), W the first Rk column
// generators of Mat_N; PL / PU the row / column permutations.
int vp2_rrlu(double *D, double *F, double *A, double *V, double tol, double *U, double *W,
             int *PL, int *PU, int M, int N, long long &nswap) {
  for (int i = 0; i < M; ++i) { U[i] = A[i]; PL[i] = i; }
  for (int j = 0; j < N; ++j) PU[j] = j;
  int Rk = std::min(M, N);
  const int mn = Rk;
  double Amax = 0.0;
  const double rho = 1.02;
  const int prd = 10;
  for (int k = 0; k < mn; ++k) {
    vp2_pivt(D, F, U, V, PL, PU, k, A, M, N);
    double Ukk = U[k] * V[k] / (D[k] - F[k]);
    Amax = std::max(Amax, std::fabs(Ukk));
    if (std::fabs(Ukk) < tol * Amax) {
      vp2_pivt_cp(D, F, U, V, PL, PU, k, A, M, N);
      Ukk = U[k] * V[k] / (D[k] - F[k]);
      Amax = std::max(Amax, std::fabs(Ukk));
      if (std::fabs(Ukk) < tol * Amax) { Rk = k; break; }
    }
    for (int i = k + 1; i < M; ++i) U[i] = U[i] * (D[i] - D[k]) / (D[i] - F[k]);
    for (int j = k + 1; j < N; ++j) V[j] = V[j] * (F[j] - F[k]) / (F[j] - D[k]);
    for (int j = 0; j < k; ++j) W[j] = W[j] * ((F[k] - D[j]) / (D[k] - D[j]));
    W[k] = (D[k] - F[k]) / A[k];
    for (int j = 0; j < k; ++j) W[k] = W[k] * (F[j] - D[k]) / (D[j] - D[k]);
    bool again = ((k + 1) % prd) == 0;
    while (again) {
      again = false;
      int ii, jj;
      double nmax;
      vp2_search(U + k + 1, W, D + k + 1, D, M - k - 1, k + 1, ii, jj, nmax);
      if (M - k - 1 > 0 && nmax > rho) {
        ++nswap;
        again = true;
        jj += k + 1;
        for (int j = k + 1; j < N; ++j) V[j] = V[j] * ((F[j] - D[ii]) / (F[j] - D[jj]));
        for (int i = k + 1; i < jj; ++i) U[i] = U[i] * ((D[i] - D[jj]) / (D[i] - D[ii]));
        for (int i = jj + 1; i < M; ++i) U[i] = U[i] * ((D[i] - D[jj]) / (D[i] - D[ii]));
        for (int j = 0; j < ii; ++j) W[j] = W[j] * ((D[j] - D[ii]) / (D[j] - D[jj]));
        for (int j = ii + 1; j <= k; ++j) W[j] = W[j] * ((D[j] - D[ii]) / (D[j] - D[jj]));
        U[jj] = A[ii] * ((D[ii] - D[jj]) / (D[ii] - F[ii]));
        W[ii] = (D[jj] - F[ii]) / A[jj];
        for (int j = 0; j <= k; ++j) {
          if (j == ii) continue;
          U[jj] = U[jj] * ((D[ii] - D[j]) / (D[ii] - F[j]));
          W[ii] = W[ii] * ((F[j] - D[jj]) / (D[j] - D[jj]));
        }
        swp(PL, ii, jj); swp(D, ii, jj); swp(A, ii, jj);
      }
    }
  }
  return Rk;
}

// comprcauchy (:616-725) + Cauchylike2 (:743-778).  Row case: the node's rows
// (poles Dn, generators Un, M of them) against the other columns (Fo, Vo, N):
// returns U_node (M x Rk) in the node's original row order; Dn / Un permuted
// so that their first Rk entries are the skeleton.  Column case: the node's
// columns (poles Fn, generators Vn, M) against the other rows (Do, Uo, N):
// returns V_node (Rk x M) in the node's original column order.
int vp2_compress(bool row, double *Pn, double *Gn, double *Po, double *Go, double tol, int M,
                 int N, std::vector<double> &Q, long long &nswap) {
  std::vector<double> Z(M, 0.0), W(std::max(std::min(M, N), 1), 0.0);
  std::vector<int> PL(M), PU(std::max(N, 1)), inv(M);
  // row: rrluCauchy(D, F, U, V); column: rrluCauchy(F, D, V, U)
  const int Rk = vp2_rrlu(Pn, Po, Gn, Go, tol, Z.data(), W.data(), PL.data(), PU.data(), M, N,
                          nswap);
  for (int i = 0; i < M; ++i) inv[PL[i]] = i;
  if (Rk < M) {
    Q.assign((size_t)M * Rk, 0.0);
    for (int r = 0; r < M; ++r) {
      const int p = inv[r];
      for (int j = 0; j < Rk; ++j) {
        const double v = p < Rk ? (p == j ? 1.0 : 0.0) : Z[p] * W[j] / (Pn[p] - Pn[j]);
        // Cauchylike2's two branches (:763-775) give the same entry
        // Z_p W_j / (P_p - P_j); the column case stores it transposed (Rk x M)
        if (row) Q[r + (size_t)j * M] = v;
        else Q[j + (size_t)r * Rk] = v;
      }
    }
  } else {
    Q.assign((size_t)M * M, 0.0);
    for (int r = 0; r < M; ++r) {
      if (row) Q[r + (size_t)inv[r] * M] = 1.0;
      else Q[inv[r] + (size_t)r * M] = 1.0;
    }
  }
  return Rk;
}

// cauchy2hss (:387-613): post-order traversal with a stack of compressed
// skeletons; every node's rows are compressed against the skeleton columns
// of the nodes to its left and the full columns to its right, then its
// columns likewise.  D, F, U, V are overwritten (as in the Fortran).
void cauchy2hss_vp2(const Tree &t, int n, double *D, double *F, double *U, double *V, double tol,
                    Gen &g, long long &nswap) {
  g.init(t.ltr);
  const int ltr = t.ltr;
  std::vector<int> l0(ltr + 1), l1(ltr + 1);
  for (int i = 1, lt = 0, it = 0; i <= ltr; ++i) {
    if (t.leaf(i)) { l0[i] = lt; l1[i] = lt + t.m[it] - 1; lt = l1[i] + 1; ++it; }
    else { l0[i] = l0[t.c1[i]]; l1[i] = l1[t.c2[i]]; }
  }
  std::vector<int> lsr(t.lvl + 3, 0), lsc(t.lvl + 3, 0);
  int ns = 0;  // stack depth; lsr[ns] / lsc[ns]: next free skeleton position
  std::vector<double> Di, Fi, Ui, Vi;
  auto row_compress = [&](int node, int r0, int mi, int ncolL) {
    // rows D/U[r0 .. r0+mi) against skeleton columns [0, ncolL) and columns right of the node
    const int ni = n - (l1[node] + 1);
    const int nt = ncolL + ni;
    Di.assign(D + r0, D + r0 + mi); Ui.assign(U + r0, U + r0 + mi);
    Fi.resize(std::max(nt, 1)); Vi.resize(std::max(nt, 1));
    for (int j = 0; j < ncolL; ++j) { Fi[j] = F[j]; Vi[j] = V[j]; }
    for (int j = 0; j < ni; ++j) { Fi[ncolL + j] = F[l1[node] + 1 + j]; Vi[ncolL + j] = V[l1[node] + 1 + j]; }
    const int Rk = vp2_compress(true, Di.data(), Ui.data(), Fi.data(), Vi.data(), tol, mi, nt,
                                g.U[node], nswap);
    g.Ur[node] = mi; g.Uc[node] = Rk;
    return Rk;
  };
  auto col_compress = [&](int node, int c0, int mi, int nrowL) {
    const int ni = n - (l1[node] + 1);
    const int nt = nrowL + ni;
    Fi.assign(F + c0, F + c0 + mi); Vi.assign(V + c0, V + c0 + mi);
    Di.resize(std::max(nt, 1)); Ui.resize(std::max(nt, 1));
    for (int j = 0; j < nrowL; ++j) { Di[j] = D[j]; Ui[j] = U[j]; }
    for (int j = 0; j < ni; ++j) { Di[nrowL + j] = D[l1[node] + 1 + j]; Ui[nrowL + j] = U[l1[node] + 1 + j]; }
    const int Rk = vp2_compress(false, Fi.data(), Vi.data(), Di.data(), Ui.data(), tol, mi, nt,
                                g.V[node], nswap);
    g.Vr[node] = Rk; g.Vc[node] = mi;
    return Rk;
  };
  for (int i = 1; i <= ltr; ++i) {
    if (t.leaf(i)) {
      const int mi = l1[i] - l0[i] + 1;
      g.Dm[i] = mi;
      g.D[i].assign((size_t)mi * mi, 0.0);
      for (int c = 0; c < mi; ++c)
        for (int r = 0; r < mi; ++r)
          g.D[i][r + (size_t)c * mi] = U[l0[i] + r] * V[l0[i] + c] / (D[l0[i] + r] - F[l0[i] + c]);
      if (i == ltr) break;  // a single leaf: no off-diagonal blocks
      int Rk = row_compress(i, l0[i], mi, lsc[ns]);
      for (int j = 0; j < Rk; ++j) { D[lsr[ns] + j] = Di[j]; U[lsr[ns] + j] = Ui[j]; }
      lsr[ns + 1] = lsr[ns] + Rk;
      Rk = col_compress(i, l0[i], mi, lsr[ns]);
      for (int j = 0; j < Rk; ++j) { F[lsc[ns] + j] = Fi[j]; V[lsc[ns] + j] = Vi[j]; }
      lsc[ns + 1] = lsc[ns] + Rk;
      ++ns;
    } else {
      // B generators between the two children (top two stack entries)
      const int c1 = t.c1[i], c2 = t.c2[i];
      const int r1 = lsr[ns - 1] - lsr[ns - 2], r2 = lsr[ns] - lsr[ns - 1];
      const int k1 = lsc[ns - 1] - lsc[ns - 2], k2 = lsc[ns] - lsc[ns - 1];
      g.Br[c1] = r1; g.Bc[c1] = k2;
      g.B[c1].assign((size_t)std::max(r1 * k2, 1), 0.0);
      for (int c = 0; c < k2; ++c)
        for (int r = 0; r < r1; ++r)
          g.B[c1][r + (size_t)c * r1] = U[lsr[ns - 2] + r] * V[lsc[ns - 1] + c] /
                                        (D[lsr[ns - 2] + r] - F[lsc[ns - 1] + c]);
      g.Br[c2] = r2; g.Bc[c2] = k1;
      g.B[c2].assign((size_t)std::max(r2 * k1, 1), 0.0);
      for (int c = 0; c < k1; ++c)
        for (int r = 0; r < r2; ++r)
          g.B[c2][r + (size_t)c * r2] = U[lsr[ns - 1] + r] * V[lsc[ns - 2] + c] /
                                        (D[lsr[ns - 1] + r] - F[lsc[ns - 2] + c]);
      if (i == ltr) break;
      // the children's skeleton rows (then columns) merged and compressed again
      int mi = lsr[ns] - lsr[ns - 2];
      int Rk = row_compress(i, lsr[ns - 2], mi, lsc[ns - 2]);
      for (int j = 0; j < Rk; ++j) { D[lsr[ns - 2] + j] = Di[j]; U[lsr[ns - 2] + j] = Ui[j]; }
      lsr[ns - 1] = lsr[ns - 2] + Rk;
      mi = lsc[ns] - lsc[ns - 2];
      Rk = col_compress(i, lsc[ns - 2], mi, lsr[ns - 2]);
      for (int j = 0; j < Rk; ++j) { F[lsc[ns - 2] + j] = Fi[j]; V[lsc[ns - 2] + j] = Vi[j]; }
      lsc[ns - 1] = lsc[ns - 2] + Rk;
      --ns;
    }
  }
}

// The generators of C^T from those of C: U <-> V^T, D^T, and B of a node is
// the transposed B of its sibling (C^T(rows i, cols j) = (U_j B_j V_i)^T).
void transpose_gen(const Tree &t, const Gen &g, Gen &h) {
  h.init(t.ltr);
  auto tr = [](const std::vector<double> &a, int r, int c) {
    std::vector<double> b((size_t)std::max(r * c, 1), 0.0);
    for (int j = 0; j < c; ++j)
      for (int i = 0; i < r; ++i) b[j + (size_t)i * c] = a[i + (size_t)j * r];
    return b;
  };
  for (int i = 1; i <= t.ltr; ++i) {
    if (t.leaf(i) && g.Dm[i] > 0) { h.Dm[i] = g.Dm[i]; h.D[i] = tr(g.D[i], g.Dm[i], g.Dm[i]); }
    if (i == t.ltr) continue;
    h.Ur[i] = g.Vc[i]; h.Uc[i] = g.Vr[i]; h.U[i] = tr(g.V[i], g.Vr[i], g.Vc[i]);
    h.Vr[i] = g.Uc[i]; h.Vc[i] = g.Ur[i]; h.V[i] = tr(g.U[i], g.Ur[i], g.Uc[i]);
    const int s = t.sibling(i);
    h.Br[i] = g.Bc[s]; h.Bc[i] = g.Br[s]; h.B[i] = tr(g.B[s], g.Br[s], g.Bc[s]);
  }
}

}  // namespace

// =================================================================== C API ==
extern "C" {

int hso_init(const char *path) {
  if (L.h) return 0;
  L.h = dlopen(path, RTLD_NOW | RTLD_LOCAL);
  if (!L.h) { fprintf(stderr, "hso_init: %s\n", dlerror()); return -1; }
  L.dlaed4 = (fn_dlaed4)sym("dlaed4");
  L.dlaed3 = (fn_dlaed3)sym("dlaed3");
  L.dsteqr = (fn_dsteqr)sym("dsteqr");
  L.dlamrg = (fn_dlamrg)sym("dlamrg");
  L.dgemm = (fn_dgemm)sym("dgemm");
  L.dstedc = (fn_dstedc)sym("dstedc");
  L.set_threads = (fn_setthreads)sym("openblas_set_num_threads");
  if (!L.dlaed4 || !L.dlaed3 || !L.dsteqr || !L.dlamrg || !L.dgemm || !L.dstedc) {
    fprintf(stderr, "hso_init: missing LAPACK symbols in %s\n", path);
    return -2;
  }
  hso_set_threads(1);
  return 0;
}

void hso_set_threads(int nt) {
  g_threads = std::max(1, nt);
  if (L.set_threads) L.set_threads(&g_threads);
}
int hso_get_threads(void) { return g_threads; }

void hso_default_config(hso_config *c) {
  c->hss_leaf = 200;
  c->bsmlz = 1500;
  c->tol = 1e-17;
  c->smlsiz = 25;
}

void hso_get_stats(hso_stats *st) { *st = g_stats; }

int hso_mdstedc(char compz, int n, double *d, double *e, double *z, int ldz,
                const hso_config *cfgp) {
  hso_config cfg;
  if (cfgp) cfg = *cfgp; else hso_default_config(&cfg);
  std::memset(&g_stats, 0, sizeof g_stats);
  int icompz = (compz == 'N' || compz == 'n') ? 0 : (compz == 'V' || compz == 'v') ? 1
               : (compz == 'I' || compz == 'i') ? 2 : -1;
  if (icompz < 0) return -1;
  if (n < 0) return -2;
  if (ldz < 1 || (icompz > 0 && ldz < std::max(1, n))) return -6;
  if (icompz != 2) return -1;  // only COMPZ='I' is on the HSS path
  if (n == 0) return 0;
  if (n == 1) { z[0] = 1.0; return 0; }
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) z[i + (size_t)j * ldz] = (i == j) ? 1.0 : 0.0;
  std::vector<double> work(2 * (size_t)n + 2);
  if (n <= cfg.smlsiz) {
    int info = 0; char cz = 'I';
    L.dsteqr(&cz, &n, d, e, z, &ldz, work.data(), &info, 1);
    return info;
  }
  double orgnrm = 0.0;
  for (int i = 0; i < n; ++i) orgnrm = std::max(orgnrm, std::fabs(d[i]));
  for (int i = 0; i + 1 < n; ++i) orgnrm = std::max(orgnrm, std::fabs(e[i]));
  if (orgnrm == 0.0) return 0;
  int start = 0, m = n;
  while (start < n) {
    int finish = start;
    while (finish < n - 1) {
      double tiny = EPS * std::sqrt(std::fabs(d[finish])) * std::sqrt(std::fabs(d[finish + 1]));
      if (std::fabs(e[finish]) > tiny) ++finish; else break;
    }
    m = finish - start + 1;
    if (m == 1) { start = finish + 1; continue; }
    if (m > cfg.smlsiz) {
      double nrm = 0.0;
      for (int i = start; i <= finish; ++i) nrm = std::max(nrm, std::fabs(d[i]));
      for (int i = start; i < finish; ++i) nrm = std::max(nrm, std::fabs(e[i]));
      const double mul = 1.0 / nrm;  // DLASCL multiplies by CTO/CFROM
      for (int i = start; i <= finish; ++i) d[i] *= mul;
      for (int i = start; i < finish; ++i) e[i] *= mul;
      int info = laed0(m, d + start, e + start, z + start + (size_t)start * ldz, ldz, cfg);
      if (info) return (info / (m + 1) + start) * (n + 1) + info % (m + 1) + start;
      for (int i = start; i <= finish; ++i) d[i] *= nrm;
    } else {
      int info = 0; char cz = 'I';
      work.resize(std::max<size_t>(work.size(), 2 * (size_t)m));
      L.dsteqr(&cz, &m, d + start, e + start, z + start + (size_t)start * ldz, &ldz,
               work.data(), &info, 1);
      if (info) return (start + 1) * (n + 1) + finish + 1;
    }
    start = finish + 1;
  }
  if (m != n) {  // selection sort (mdstedc.f90:408-423)
    for (int i = 0; i + 1 < n; ++i) {
      int k = i; double p = d[i];
      for (int j = i + 1; j < n; ++j) if (d[j] < p) { k = j; p = d[j]; }
      if (k != i) {
        d[k] = d[i]; d[i] = p;
        for (int r = 0; r < n; ++r) std::swap(z[r + (size_t)i * ldz], z[r + (size_t)k * ldz]);
      }
    }
  }
  return 0;
}

int hso_dstedc_lapack(int n, double *d, double *e, double *z, int ldz) {
  char cz = 'I';
  int lwork = -1, liwork = -1, info = 0, iq = 0;
  double wq = 0;
  L.dstedc(&cz, &n, d, e, z, &ldz, &wq, &lwork, &iq, &liwork, &info, 1);
  lwork = (int)wq; liwork = iq;
  std::vector<double> work(std::max(lwork, 1));
  std::vector<int> iwork(std::max(liwork, 1));
  L.dstedc(&cz, &n, d, e, z, &ldz, work.data(), &lwork, iwork.data(), &liwork, &info, 1);
  return info;
}

int hso_secular(int k, const double *dlamda, const double *z, double rho,
                double *lam, double *difl, double *difr) {
  std::vector<double> zz(z, z + k);
  return secular_lowner(k, dlamda, zz.data(), rho, lam, difl, difr, nullptr);
}

int hso_lowner(int k, const double *dlamda, const double *difl, const double *difr,
               double *z, double *alpha) {
  // z_hat_i^2 = prod_j (d_i - lam_j) / prod_{j != i} (d_i - d_j), with
  // d_i - lam_j = -fd(i, j) formed from DIFL/DIFR (mdlaed3.f90:217-230)
  Poles P{dlamda, difl, difr};
  std::vector<double> prod(k, 1.0);
  for (int j = 0; j < k; ++j) {
    prod[j] *= P.fd(j, j);
    for (int i = 0; i < k; ++i)
      if (i != j) prod[i] *= P.fd(i, j) / (dlamda[i] - dlamda[j]);
  }
  for (int i = 0; i < k; ++i) z[i] = std::copysign(std::sqrt(std::fabs(prod[i])), z[i]);
  for (int j = 0; j < k; ++j) {
    double s = 0.0;
    for (int i = 0; i < k; ++i) { double w = z[i] / P.fd(i, j); s += w * w; }
    alpha[j] = 1.0 / std::sqrt(s);
  }
  return 0;
}

void hso_cauchy_eig_dense(int k, const double *F, const double *u, const double *v,
                          const double *difl, const double *difr, double *C) {
  Poles P{F, difl, difr};
  for (int j = 0; j < k; ++j)
    for (int i = 0; i < k; ++i) C[i + (size_t)j * k] = u[i] * v[j] / P.fd(i, j);
}

int hso_dhssevc(int k, int ni, double tol, const double *F, const double * /*D*/,
                const double *u, const double *v, const double *difl,
                const double *difr, double *Q, int ldq, int nrows, int *mr) {
  return dhssevc(k, ni, tol, F, u, v, difl, difr, Q, ldq, nrows, mr);
}

// CauchyHssMM (SRC/cauchyhssmm.f90:1-123): B (n x ncb, ldb) <- C B with
// C(i,j) = U_i V_j / (D_i - F_j) compressed by the VP2 module (leaf ni, tol);
// the product is (B^T C^T)^T through fastHssmmL's restatement.  D, F, U, V are
// overwritten as in the Fortran.  Returns the largest generator rank.
int hso_cauchyhssmm(int n, double *D, double *F, double *U, double *V, int ni, double tol,
                    double *B, int ldb, int ncb) {
  Tree t = make_tree(n, ni);
  Gen g, h;
  long long sw = 0;
  cauchy2hss_vp2(t, n, D, F, U, V, tol, g, sw);
  g_stats.n_swaps += sw;
  transpose_gen(t, g, h);
  std::vector<double> X((size_t)ncb * n);
  for (int c = 0; c < n; ++c)
    for (int r = 0; r < ncb; ++r) X[r + (size_t)c * ncb] = B[c + (size_t)r * ldb];
  hss_mm_left(t, h, X.data(), ncb, ncb);
  for (int c = 0; c < n; ++c)
    for (int r = 0; r < ncb; ++r) B[c + (size_t)r * ldb] = X[r + (size_t)c * ncb];
  int r = 0;
  for (int i = 1; i < t.ltr; ++i) r = std::max(r, std::max(g.Uc[i], g.Vr[i]));
  g_stats.max_rank = std::max(g_stats.max_rank, r);
  return r;
}

void hso_cauchylike(double *A, const double *D, const double *F, const double *u,
                    const double *v, int m, int n) {
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < m; ++i) A[i + (size_t)j * m] = u[i] * v[j] / (D[i] - F[j]);
}

}  // extern "C"
