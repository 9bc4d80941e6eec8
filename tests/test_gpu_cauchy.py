"""Cauchy-like HSS products on the GPU: CauchyHssMM (generic Cauchy matrix,
SRC/cauchyhssmm.f90) against the dense product, and the n = 8192 Cauchy merge
(secular roots, Loewner z, HSS compression of the eigenvector matrix, product
with a dense orthogonal Q) against the oracle: roots, DIFL/DIFR against
LAPACK DLAED4, the Loewner vectors and the dense eigenvector block against the
restated MDLAED3/CauchylikeEig.

Tolerances: the HSS products within 1e-11 (relative Frobenius) of the dense
products at HSS tolerance 1e-14; orthogonality of Q C within 1e-12 * n."""
import os

import numpy as np
import pytest
import torch

import oracle
import hsspack_gb300 as hp
from helpers import interlace_grid

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _dev(a):
    return torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


@pytest.mark.parametrize("n,ni", [(1024, 64), (3000, 128)])
@pytest.mark.parametrize("precision", [0, 1])
def test_cauchyhssmm_interlacing_grid(n, ni, precision):
    # the grid of TEST/testCauchyHss_serial.f90:46-52
    F, D = interlace_grid(n)
    rng = np.random.default_rng(n)
    u, v = rng.standard_normal(n), rng.standard_normal(n)
    B = rng.standard_normal((n, n))
    C = u[:, None] * v[None, :] / (D[:, None] - F[None, :])
    ref = C @ B
    Bd = _dev(B.T)  # tensor memory = column-major B
    old = hp.set_config(precision=precision)
    try:
        t_build, t_mult = hp.cauchyhssmm_dev(_dev(D), _dev(F), _dev(u), _dev(v), Bd, ni, 1e-14)
    finally:
        hp.restore_config(old)
    out = Bd.cpu().numpy().T
    err = np.linalg.norm(out - ref) / np.linalg.norm(ref)
    assert err <= 1e-11, err
    assert t_build > 0 and t_mult > 0
    assert hp.get_stats()["max_rank"] < n // 4  # the grid's blocks are low rank


@pytest.mark.parametrize("n,ni,tol", [(1024, 64, 1e-14), (3000, 128, 1e-14), (2000, 64, 1e-11)])
def test_cauchyhssmm_ranks_vs_vp2_oracle(n, ni, tol):
    # the same compression rule as the reference's generic Cauchy module
    # (rrluCauchy, rho = 1.02, CauchyHss_VP2.f90:7-134): the GPU's level-batched
    # construction against the oracle's restated post-order cauchy2hss.  The
    # skeleton sets differ (levels vs the post-order stack), so ranks are
    # compared within a few units, the products to the tolerance.
    F, D = interlace_grid(n)
    rng = np.random.default_rng(n + 1)
    u, v = rng.standard_normal(n), rng.standard_normal(n)
    B = rng.standard_normal((n, 256))
    ref, r_o = oracle.cauchyhssmm(D, F, u, v, B, ni, tol)
    Bd = _dev(B.T)
    hp.cauchyhssmm_dev(_dev(D), _dev(F), _dev(u), _dev(v), Bd, ni, tol)
    r_g = hp.get_stats()["max_rank"]
    out = Bd.cpu().numpy().T
    assert abs(r_g - r_o) <= 4, (r_g, r_o)
    C = u[:, None] * v[None, :] / (D[:, None] - F[None, :])
    dense = C @ B
    nrm = np.linalg.norm(dense)
    assert np.linalg.norm(out - dense) / nrm <= 100 * tol
    assert np.linalg.norm(out - ref) / nrm <= 200 * tol


def test_cauchyhssmm_fortran_entry():
    n = 800
    F, D = interlace_grid(n, 0.3, 5.0)
    rng = np.random.default_rng(1)
    u, v = rng.standard_normal(n), rng.standard_normal(n)
    B = np.asfortranarray(rng.standard_normal((n, n)))
    ref = (u[:, None] * v[None, :] / (D[:, None] - F[None, :])) @ B
    t = hp.cauchyhssmm(D, F, u, v, B, 64, 1e-14, ncol=100)
    assert np.linalg.norm(B - ref) / np.linalg.norm(ref) <= 1e-11
    assert t[0] > 0 and t[1] > 0


@pytest.fixture(scope="module")
def merge_8192():
    """The Cauchy merge workload: d sorted U[0,1], z ~ N(0,1)/sqrt(n), rho = 1
    (seed 0), n = 8192; the GPU's roots, DIFL/DIFR, z-hat and alpha, checked
    against the oracle (LAPACK DLAED4 per root and the restated MDLAED3 steps,
    SRC/mdlaed3.f90:207-249) before any product uses them."""
    n = 8192
    rng = np.random.default_rng(0)
    d = np.sort(rng.uniform(0.0, 1.0, n))
    z = rng.standard_normal(n) / np.sqrt(n)
    dd, zz = _dev(d), _dev(z)
    lam, difl, difr = (torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(3))
    hp.secular_dev(dd, zz, 1.0, lam, difl, difr)
    zh, al = zz.clone(), torch.zeros(n, dtype=torch.float64, device="cuda")
    hp.lowner_dev(dd, difl, difr, zh, al)
    return n, d, z, dd, lam, difl, difr, zh, al


def test_cauchy_merge_8192_secular_vs_dlaed4(merge_8192):
    n, d, z, dd, lam, difl, difr, zh, al = merge_8192
    lam_o, difl_o, difr_o = oracle.secular(d, z, 1.0)
    lam_g, difl_g, difr_g = (t.cpu().numpy() for t in (lam, difl, difr))
    # the secular tests' bar: roots within 1e-13 * max|d|, gaps to 1e-11; the
    # last root against 50 digits instead (DLAED4's is 1.5e-13 off there)
    assert np.max(np.abs(lam_g[:-1] - lam_o[:-1])) <= 1e-13 * max(1.0, np.abs(d).max())
    assert np.max(np.abs(difl_g[:-1] - difl_o[:-1]) / np.abs(difl_o[:-1])) <= 1e-11
    assert np.max(np.abs(difr_g[:-1] - difr_o[:-1]) / np.abs(difr_o[:-1])) <= 1e-11
    g = np.load(os.path.join(GOLD, "merge8192_mp.npz"))
    i = g["idx"]
    assert np.max(np.abs(lam_g[i] - g["lam"])) <= 1e-15 * max(1.0, np.abs(g["lam"]).max())
    assert np.max(np.abs(difl_g[i] - g["difl"]) / np.abs(g["difl"])) <= 1e-13
    m = i < n - 1
    assert np.max(np.abs(difr_g[i[m]] - g["difr"][m]) / np.abs(g["difr"][m])) <= 1e-13
    # Loewner z-hat and alpha from the oracle's roots (the restated MDLAED3):
    # each z-hat is a product of 2k - 1 = 16383 factors, so the two orders of
    # multiplication differ by up to ~k eps relative (1.6e-12 measured); bar 1e-11
    zh_o, al_o = oracle.lowner(d, difl_o, difr_o, z)
    assert np.max(np.abs(zh.cpu().numpy() - zh_o) / np.abs(zh_o)) <= 1e-11
    assert np.max(np.abs(al.cpu().numpy() - al_o) / np.abs(al_o)) <= 1e-11


@pytest.mark.parametrize("precision", [0, 1])
def test_cauchy_merge_8192(merge_8192, precision):
    # HSS leaf 128, tol 1e-14, times a dense random orthogonal Q (8192 x 8192);
    # reference: the oracle's dense eigenvector block (CauchylikeEig restated,
    # SRC/CauchyHssEig.f90:1688-1765) from the oracle's own roots and Loewner
    # vectors, multiplied in FP64 on the host on 512 rows of Q
    n, d, z, dd, lam, difl, difr, zh, al = merge_8192
    lam_o, difl_o, difr_o = oracle.secular(d, z, 1.0)
    zh_o, al_o = oracle.lowner(d, difl_o, difr_o, z)
    C_o = oracle.cauchy_eig_dense(d, zh_o, al_o, difl_o, difr_o)
    gen = torch.Generator(device="cuda").manual_seed(1)
    Qf, _ = torch.linalg.qr(torch.randn(n, n, dtype=torch.float64, device="cuda", generator=gen))
    rows = np.random.default_rng(3).choice(n, 512, replace=False)
    ref = Qf[torch.tensor(rows, device="cuda")].cpu().numpy() @ C_o
    Q = Qf.T.contiguous()  # memory = column-major Qf
    old = hp.set_config(precision=precision)
    try:
        hp.dhssevc_dev(dd, zh, al, difl, difr, Q, n, n, ni=128, tol=1e-14)
    finally:
        hp.restore_config(old)
    out = Q.T  # Q C
    got = out[torch.tensor(rows, device="cuda")].cpu().numpy()
    err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    assert err <= 1e-11, err
    g = torch.randn(n, 8, dtype=torch.float64, device="cuda", generator=gen)
    y = out.T @ (out @ g) - g
    assert float(torch.sqrt(torch.sum(y * y) / 8)) / n <= 1e-12
