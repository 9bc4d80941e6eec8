"""CPU tests of the oracle (the checker): pinned against LAPACK DSTEDC, the
closed-form spectrum of TEST/Testedc.f90 (D = 2, E = 1), 50-digit secular
roots and the committed golden fixtures."""
import os

import numpy as np
import pytest

import oracle
from helpers import (eig_metrics, interlace_grid, rand_tridiag, secular_problem, toeplitz_eigs,
                     toeplitz_tridiag)

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
EV_TOL, RES_TOL, ORTH_TOL = 1e-13, 1e-12, 1e-12


@pytest.mark.parametrize("n,bsmlz,leaf", [(30, 1500, 200), (300, 1500, 200), (700, 60, 32),
                                          (1024, 100, 64)])
def test_oracle_vs_lapack_random(n, bsmlz, leaf):
    d, e = rand_tridiag(n, seed=n)
    w, Q = oracle.eigh_tridiagonal(d, e, hss_leaf=leaf, bsmlz=bsmlz, tol=1e-14)
    wl, _ = oracle.dstedc_lapack(d, e)
    ev, res, orth = eig_metrics(d, e, w, Q, wl)
    assert ev <= EV_TOL and res <= RES_TOL and orth <= ORTH_TOL, (ev, res, orth)


@pytest.mark.parametrize("n,bsmlz", [(500, 1500), (1000, 200), (2048, 600)])
def test_oracle_toeplitz_closed_form(n, bsmlz):
    d, e = toeplitz_tridiag(n)
    w, Q = oracle.eigh_tridiagonal(d, e, hss_leaf=64, bsmlz=bsmlz, tol=1e-14)
    assert np.max(np.abs(w - toeplitz_eigs(n))) <= 4 * EV_TOL
    ev, res, orth = eig_metrics(d, e, w, Q, toeplitz_eigs(n))
    assert res <= RES_TOL and orth <= ORTH_TOL
    if bsmlz < n // 2:
        assert oracle.stats()["n_hss_merges"] > 0


def test_oracle_secular_vs_mp_roots():
    g = np.load(os.path.join(GOLD, "secular_mp.npz"))
    for k in (3, 40, 200):
        d, z, rho = g["k%d_d" % k], g["k%d_z" % k], float(g["k%d_rho" % k])
        lam, difl, difr = oracle.secular(d, z, rho)
        assert np.max(np.abs(lam - g["k%d_lam" % k])) <= 1e-13
        assert np.max(np.abs(difl - g["k%d_difl" % k]) / np.abs(g["k%d_difl" % k])) <= 1e-10


def test_oracle_secular_vs_mp_roots_nearly_deflatable():
    # a pole of weight 1e-7 or 3e-14 sitting on a root of the other poles'
    # equation (the merges of glued matrices): LAPACK DLAED4, which the GPU
    # pole-on-a-root tests compare with, stays within its 1e-13 on every root
    g = np.load(os.path.join(GOLD, "secular_edge_mp.npz"))
    for where in ("last", "middle", "first"):
        for w in ("w7", "w14"):
            key = "%s_%s" % (where, w)
            d, z, rho = g[key + "_d"], g[key + "_z"], float(g[key + "_rho"])
            lam, difl, difr = oracle.secular(d, z, rho)
            assert np.max(np.abs(lam - g[key + "_lam"])) <= 1e-13, key


def test_oracle_secular_vs_mp_roots_merge8192():
    # the n = 8192 Cauchy-merge problem: LAPACK DLAED4 within 1e-13 of the
    # 50-digit roots except the last, which it leaves 1.5e-13 off (its stopping
    # test for the root beyond the last pole is looser); the GPU parity test
    # pins that root to the 50-digit value instead
    g = np.load(os.path.join(GOLD, "merge8192_mp.npz"))
    n = 8192
    rng = np.random.default_rng(0)
    d = np.sort(rng.uniform(0.0, 1.0, n))
    z = rng.standard_normal(n) / np.sqrt(n)
    lam, difl, difr = oracle.secular(d, z, 1.0)
    i = g["idx"]
    err = np.abs(lam[i] - g["lam"])
    assert np.max(err[i < n - 1]) <= 1e-13
    assert 1e-14 < err[i == n - 1][0] <= 1e-12


def test_oracle_glued_wilkinson():
    # Wilkinson-type blocks glued by 1e-8: every merge has nearly deflatable
    # poles; the restated MDSTEDC (HSS merges from K >= 40) holds the bar
    m, nb = 21, 60
    d = np.tile(np.abs(np.arange(m) - (m - 1) / 2.0), nb)
    e = np.ones(m * nb - 1)
    e[m - 1::m] = 1e-8
    w, Q = oracle.eigh_tridiagonal(d, e, hss_leaf=64, bsmlz=40, tol=1e-14)
    wl, _ = oracle.dstedc_lapack(d, e)
    ev, res, orth = eig_metrics(d, e, w, Q, wl)
    assert ev <= 1e-13 and res <= 1e-12 and orth <= 1e-12, (ev, res, orth)


def test_oracle_matches_golden_dc():
    g = np.load(os.path.join(GOLD, "dc_small.npz"))
    for name in ("rand64", "rand200", "rand512", "toep100"):
        d, e = g[name + "_d"], g[name + "_e"]
        w, Q = oracle.eigh_tridiagonal(d, e, hss_leaf=64, bsmlz=40, tol=1e-14)
        assert np.max(np.abs(w - g[name + "_w"])) <= 1e-13
        if name + "_Q" in g:
            # eigenvectors up to sign
            Qg = g[name + "_Q"]
            s = np.sign(np.sum(Q * Qg, axis=0))
            assert np.max(np.abs(Q * s - Qg)) <= 1e-12


@pytest.mark.parametrize("k,ni,tol", [(600, 64, 1e-14), (1500, 128, 1e-17), (2000, 200, 1e-17)])
def test_oracle_dhssevc_vs_dense(k, ni, tol):
    d, z, rho = secular_problem(k, seed=k)
    lam, difl, difr = oracle.secular(d, z, rho)
    zh, alpha = oracle.lowner(d, difl, difr, z)
    C = oracle.cauchy_eig_dense(d, zh, alpha, difl, difr)
    assert np.linalg.norm(C.T @ C - np.eye(k)) / k <= 1e-14
    rng = np.random.default_rng(k)
    X = np.asfortranarray(rng.standard_normal((97, k)))
    Y, rank = oracle.dhssevc(d, zh, alpha, difl, difr, X, ni=ni, tol=tol)
    err = np.max(np.abs(Y - X @ C)) / np.max(np.abs(X @ C))
    assert err <= 1e-12, err
    assert 0 < rank <= 2 * ni  # parents compress the union of two child skeletons


def test_cauchylike_grid_fixture():
    g = np.load(os.path.join(GOLD, "hss_grid.npz"))
    A = np.zeros((len(g["D"]), len(g["F"])))
    F, D = interlace_grid(len(g["F"]))
    assert np.array_equal(F, g["F"]) and np.array_equal(D, g["D"])
    C = g["u"][:, None] * g["v"][None, :] / (g["D"][:, None] - g["F"][None, :])
    assert np.allclose(C @ g["B"], g["CB"], rtol=1e-13, atol=0)
    del A


@pytest.mark.parametrize("n,kd", [(64, 2), (100, 4), (257, 3), (300, 8)])
def test_band_restatement_matches_lapack(n, kd):
    # the banded DC restatement (split by cut SVDs, leaf solves, kd rank-one
    # updates with Z carried along) against LAPACK DSBEVD
    from oracle import band_ref
    rng = np.random.default_rng(n + kd)
    ab = rng.uniform(-1.0, 1.0, (kd + 1, n))
    A = band_ref.band_to_dense(ab)
    w, Q = band_ref.band_dc(A, kd)
    wl, _ = band_ref.eig_banded_lapack(ab)
    na = np.abs(A).sum(axis=1).max()
    assert np.max(np.abs(w - wl)) <= 1e-13 * na
    assert np.linalg.norm(A @ Q - Q * w) / (n * na) <= 1e-14
    assert np.linalg.norm(Q.T @ Q - np.eye(n)) / n <= 1e-14


def test_hssmm_oracle_tree_and_accuracy():
    # npart leaf sizes (SRC/aux_hss.f90:807-818) and the reference test's error
    # level: DHSSMM / DHSSMML products within 2e-11 of the dense ones at
    # tol = 1e-11, ni = 64 (TEST/testfmm.f90 prints this absolute error)
    from oracle import hssmm_ref
    assert hssmm_ref.leaf_sizes(2000, 64) == [64] * 30 + [80]
    assert hssmm_ref.leaf_sizes(1100, 64) == [64] * 16 + [76]
    assert hssmm_ref.leaf_sizes(100, 64) == [64, 36]
    assert hssmm_ref.leaf_sizes(40, 64) == [40]
    ltr, par, ch = hssmm_ref.post_order_tree(3)
    assert ltr == 5 and par[1:] == [3, 3, 5, 5, 0]
    n = 700
    A = hssmm_ref.fmm_test_matrix(n)
    B = np.random.default_rng(2).uniform(size=(n, 60))
    Y, rank = hssmm_ref.dhssmm(A, B, 64, 1e-11)
    assert np.abs(Y - A @ B).max() <= 2e-11 and 20 <= rank <= 45
    Y2, _ = hssmm_ref.dhssmml(A, B.T, 64, 1e-11)
    assert np.abs(Y2 - B.T @ A).max() <= 2e-11


@pytest.mark.parametrize("n,ni,tol", [(300, 32, 1e-14), (1024, 64, 1e-14), (2000, 64, 1e-11)])
def test_oracle_cauchyhssmm_vp2_vs_dense(n, ni, tol):
    # CauchyHssMM restated with the VP2 module (post-order cauchy2hss, rrluCauchy
    # with rho = 1.02) on the interlacing grid of TEST/testCauchyHss_serial.f90:
    # the HSS product agrees with the dense one to the compression tolerance
    from helpers import interlace_grid
    F, D = interlace_grid(n)
    rng = np.random.default_rng(n)
    u, v = rng.standard_normal(n), rng.standard_normal(n)
    B = rng.standard_normal((n, 64))
    C = u[:, None] * v[None, :] / (D[:, None] - F[None, :])
    ref = C @ B
    out, r = oracle.cauchyhssmm(D, F, u, v, B, ni, tol)
    assert np.linalg.norm(out - ref) / np.linalg.norm(ref) <= 100 * tol
    assert 0 < r < n // 4
