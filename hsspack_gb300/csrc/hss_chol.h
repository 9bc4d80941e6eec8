// hss_chol.h -- HSS Cholesky factor of a dense SPD matrix (hsschol.cu): the
// host description of every level and the device arrays it owns.
#pragma once
#include <cuda_runtime.h>

#include <vector>

namespace hss {

constexpr int CH_MAXM = 128;  // largest node dimension (shared-memory Cholesky / QL)

// One active node of a level: range [o, o + m) of the level's reduced matrix,
// range [o2, o2 + rk) of the next one; ir = m - rk variables eliminated here
// (0: passed through unchanged); f: offset of its factors Qt, Lt (m x m each).
struct ChNode {
  int o, m, o2, rk, ir;
  int slot;  // scratch slot of a node factored at this level (-1: none)
  long long f;
};

struct ChLevel {
  int Nc = 0, Nc2 = 0;
  std::vector<ChNode> nodes;  // every active node, left to right
  ChNode *d_nodes = nullptr;  // device copy
  double *fac = nullptr;      // Qt, Lt of the level's compressed nodes
};

struct CholFactor {
  int n = 0, max_rank = 0, Nroot = 0;
  std::vector<ChLevel> lv;
  double *root = nullptr;     // the root's Cholesky factor (Nroot x Nroot)
  long long fac_bytes = 0;
  std::vector<void *> allocs;
  CholFactor() = default;
  CholFactor(const CholFactor &) = delete;
  CholFactor &operator=(const CholFactor &) = delete;
  ~CholFactor() {
    for (void *p : allocs) cudaFree(p);
  }
};

// Factor A (n x n, lda, device, read only); see hsschol.cu.  Returns 0 or a
// status: 1 not positive definite, 2 a node of more than CH_MAXM rows.
int hss_chol_factor_core(int n, const double *A, long long lda, int ni, double tol, int ncol,
                         int ps, unsigned long long seed, CholFactor &F, cudaStream_t st);
// B (n x nrhs, ldb, device) <- the factor's solve of B
void hss_chol_solve_core(const CholFactor &F, double *B, long long ldb, int nrhs, cudaStream_t st);
// preconditioned CG (F may be null: plain CG); returns the steps taken
int hss_chol_pcg_core(const CholFactor *F, int n, const double *A, long long lda, const double *b,
                      double *x, double tau, int maxit, double *relres, cudaStream_t st);

}  // namespace hss
