"""HSS Cholesky solver (HssCholSolver, SRC/HssCholSolver.f90:1).

The reference's test (TEST/testhsschol.f90) factors an SPD matrix with leaves
of 20 rows, tol = 1e-8 and at most prank = 10 kept per node (the randomised
variant, 5 oversampling rows), solves A x = A 1 directly ('N', "low accuracy")
and by preconditioned CG to tau = 1e-13 within 30 steps ('Y').  Its matrix file
is not shipped; a Gaussian kernel on sorted points plus a nugget (numerically
low-rank off-diagonal blocks, SPD) stands in for it.

CPU: the numpy restatement (oracle/hsschol_ref.py, the reference's node order)
is pinned against numpy's dense solve (no truncation: exact to rounding) and
against its own CG.  GPU: the Fortran entry point and the device API against
the dense solve (untruncated, 1e-9), the reference test's settings (CG
converges below 1e-12 relative residual, both variants), the truncated direct
solve against the restatement's quality (its relative residual within a factor
of 10 of the restatement's: the GPU compresses the nodes of one tree height
together, the reference one node after another, so their kept subspaces agree
to the truncation level, not bit for bit), ranks within 2 of the
restatement's, several right-hand sides, and INFO for a matrix that is not
positive definite."""
import numpy as np
import pytest

import hsspack_gb300 as hp
from oracle import hsschol_ref as ref


def _problem(n, length, seed=0):
    A = ref.kernel_matrix(n, length, 1e-2, seed)
    x0 = np.ones(n)
    return A, x0, A @ x0


def _relres(A, x, b):
    return np.linalg.norm(A @ x - b) / np.linalg.norm(b)


# ------------------------------------------------------------------ CPU ----
def test_oracle_exact_without_truncation():
    A, x0, b = _problem(600, 0.1)
    F = ref.factor(A, 20, 1e-12, 128)
    x = ref.solve(F, b)
    assert F["max_rank"] > 0  # nodes were compressed
    assert _relres(A, x, b) <= 1e-13
    assert np.linalg.norm(x - np.linalg.solve(A, b)) <= 1e-9 * np.linalg.norm(x0)


def test_oracle_truncated_preconditioner():
    A, x0, b = _problem(600, 0.1)
    F = ref.factor(A, 20, 1e-8, 10)
    x = ref.solve(F, b)
    r = _relres(A, x, b)
    assert 1e-12 < r < 1e-3  # an approximate factorisation
    xc, it, res = ref.cg(A, b, 1e-13, 30, F)
    assert res < 1e-13 and it <= 10
    _, it0, res0 = ref.cg(A, b, 1e-13, 30, None)
    assert res0 > 1e-13  # plain CG does not get there in 30 steps


def test_oracle_tree_matches_npart():
    sizes, par = ref.npart_tree(1000, 20)
    assert sizes == [20] * 50 and len(par) - 1 == 99 and par[99] == 0


# ------------------------------------------------------------------ GPU ----
@pytest.mark.gpu
def test_fortran_entry_exact():
    A, x0, b = _problem(800, 0.08, seed=1)
    x, info = hp.hsscholsolver("S", "N", A, b, 20, 1e-12, 128)
    assert info == 0
    assert np.linalg.norm(x - np.linalg.solve(A, b)) <= 1e-9 * np.linalg.norm(x0)
    assert hp.get_stats()["max_rank"] > 0


@pytest.mark.gpu
@pytest.mark.parametrize("rs", ["S", "R"])
def test_reference_settings_pcg(rs):
    A, x0, b = _problem(1000, 0.05, seed=2)
    x, info = hp.hsscholsolver(rs, "Y", A, b, 20, 1e-8, 10, pp=5, tau=1e-13, maxit=30)
    assert info == 0
    assert _relres(A, x, b) <= 1e-12
    assert hp.get_stats()["secular_iters"] <= 30  # CG steps taken


@pytest.mark.gpu
def test_truncated_direct_solve_vs_oracle():
    A, x0, b = _problem(1000, 0.05, seed=3)
    x, info = hp.hsscholsolver("S", "N", A, b, 20, 1e-8, 10)
    assert info == 0
    F = ref.factor(A, 20, 1e-8, 10)
    r_ref = _relres(A, ref.solve(F, b), b)
    r_gpu = _relres(A, x, b)
    assert r_gpu <= 10 * r_ref + 1e-14, (r_gpu, r_ref)


@pytest.mark.gpu
def test_device_api_ranks_and_several_rhs():
    import torch
    n = 1200
    A, x0, b = _problem(n, 0.05, seed=4)
    At = torch.tensor(np.asfortranarray(A).ravel(order="F"), device="cuda")
    f = hp.HssChol(At, 24, 1e-10, 128)
    info = f.info()
    F = ref.factor(A, 24, 1e-10, 128)
    assert abs(info["max_rank"] - F["max_rank"]) <= 2, (info, F["max_rank"])
    rng = np.random.default_rng(5)
    X0 = rng.standard_normal((n, 3))
    B = A @ X0
    Bt = torch.tensor(np.asfortranarray(B).ravel(order="F"), device="cuda")
    f.solve(Bt)
    X = Bt.cpu().numpy().reshape(n, 3, order="F")
    assert np.linalg.norm(A @ X - B) / np.linalg.norm(B) <= 1e-8
    bt = torch.tensor(B[:, 0], device="cuda")
    xt = torch.zeros(n, dtype=torch.float64, device="cuda")
    it, rr = f.pcg(At, bt, xt, 1e-13, 30)
    assert rr < 1e-13 and it <= 5
    assert _relres(A, xt.cpu().numpy(), B[:, 0]) <= 1e-12
    f.free()


@pytest.mark.gpu
def test_not_positive_definite_returns_info():
    A, x0, b = _problem(400, 0.1, seed=6)
    A[5, 5] = -1.0  # a leaf's diagonal block is indefinite
    x, info = hp.hsscholsolver("S", "N", A, b, 20, 1e-10, 64)
    assert info == 1
