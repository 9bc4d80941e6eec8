"""Bidiagonal SVD divide and conquer (MDBDSDC path) on the GPU against LAPACK
(numpy's SVD of the dense bidiagonal) and the numpy restatement of the
reference algorithm.

Tolerances as the acceptance bar: singular values within 1e-13 * ||B||,
||B - U S VT||_F / (n ||B||) <= 1e-12, ||U^T U - I||_F / n and
||VT VT^T - I||_F / n <= 1e-12."""
import numpy as np
import pytest
import torch

import hsspack_gb300 as hp
from oracle import svd_ref

SV_TOL, RES_TOL, ORTH_TOL = 1e-13, 1e-12, 1e-12

pytestmark = pytest.mark.gpu


def _bidiag(n, seed, lo=0.0, hi=1.0):
    rng = np.random.default_rng(seed)
    return rng.uniform(lo, hi, n), rng.uniform(lo, hi, max(n - 1, 0))


def _check(d, e, s, U, VT, lower=False):
    n = len(d)
    B = svd_ref.bidiag(d, e)
    if lower:
        B = B.T
    nb = max(np.abs(B).sum(axis=1).max(), 1e-300)
    sref = np.linalg.svd(B, compute_uv=False)
    assert np.all(np.diff(s) <= 0), "singular values not descending"
    ev = np.max(np.abs(s - sref)) / nb
    res = np.linalg.norm(B - (U * s) @ VT) / (n * nb)
    ou = np.linalg.norm(U.T @ U - np.eye(n)) / n
    ov = np.linalg.norm(VT @ VT.T - np.eye(n)) / n
    assert ev <= SV_TOL and res <= RES_TOL and ou <= ORTH_TOL and ov <= ORTH_TOL, \
        (n, ev, res, ou, ov)


@pytest.mark.parametrize("n", [1, 2, 3, 7, 25, 26, 64, 100, 257, 1000, 2048])
@pytest.mark.parametrize("precision", [0, 1])
def test_svd_random(n, precision):
    d, e = _bidiag(n, seed=n)
    old = hp.set_config(precision=precision)
    try:
        s, U, VT = hp.svd_bidiagonal(d, e)
    finally:
        hp.restore_config(old)
    _check(d, e, s, U, VT)


def test_svd_lower_signed_graded_and_restatement():
    n = 300
    d, e = _bidiag(n, seed=7, lo=-1.0, hi=1.0)
    s, U, VT = hp.svd_bidiagonal(d, e, lower=True)
    _check(d, e, s, U, VT, lower=True)
    dg, eg = d * np.logspace(0, -12, n), e * np.logspace(0, -12, n - 1)
    _check(dg, eg, *hp.svd_bidiagonal(dg, eg))
    sr, _, _ = svd_ref.bdsdc(*_bidiag(200, seed=3))
    s2, _, _ = hp.svd_bidiagonal(*_bidiag(200, seed=3))
    assert np.max(np.abs(sr - s2)) <= SV_TOL * 2.0


@pytest.mark.parametrize("pred", [2, 3])
@pytest.mark.parametrize("n", [100, 1000, 4000])
def test_svd_fp32_presolved_starts(n, pred):
    # predictor = 2 / 3: the secular iteration starts from an FP32 pre-solve in
    # squared mode (3: refined by one float-float step); random, graded and
    # deflating cases
    old = hp.set_config(predictor=pred, precision=1)
    try:
        d, e = _bidiag(n, seed=100 + n)
        _check(d, e, *hp.svd_bidiagonal(d, e))
        dg, eg = d * np.logspace(0, -10, n), e * np.logspace(0, -10, n - 1)
        _check(dg, eg, *hp.svd_bidiagonal(dg, eg))
        d2, e2 = d.copy(), e.copy()
        d2[::7] = 0.0
        d2[10:50] = 0.5
        e2[10:50] = 0.0
        _check(d2, e2, *hp.svd_bidiagonal(d2, e2))
        assert hp.get_stats()["secular_iters"] > 0
    finally:
        hp.restore_config(old)


def test_svd_deflation_cases():
    # repeated and zero entries: small z, equal singular values, zero diagonals
    n = 400
    d, e = _bidiag(n, seed=11)
    d[::7] = 0.0
    e[::5] = 1e-30
    d[100:140] = 0.5
    e[100:140] = 0.0
    _check(d, e, *hp.svd_bidiagonal(d, e))
    ones = np.ones(n)
    _check(ones, ones[:-1], *hp.svd_bidiagonal(ones, ones[:-1]))


def test_svd_plain_mode_and_values_only():
    d, e = _bidiag(700, seed=5)
    old = hp.set_config(batched=0)
    try:
        s1, U1, VT1 = hp.svd_bidiagonal(d, e)
    finally:
        hp.restore_config(old)
    _check(d, e, s1, U1, VT1)
    dd, ee = d.copy(), np.concatenate([e, [0.0]])
    one, ione = np.zeros(1), np.zeros(1, dtype=np.int32)
    u = np.zeros((1, 1), order="F")
    assert hp.mdbdsdc("U", "N", len(d), dd, ee, u, 1, u.copy(order="F"), 1, one, ione, one,
                      ione) == 0
    assert np.max(np.abs(dd - s1)) <= SV_TOL


def test_svd_16384_full_size():
    # the bidiagonal workload: n = 16384, d, e iid U(0, 1]
    n = 16384
    rng = np.random.default_rng(0)
    d = 1.0 - rng.uniform(0.0, 1.0, n)   # (0, 1]
    e = 1.0 - rng.uniform(0.0, 1.0, n - 1)
    dd = torch.tensor(d, device="cuda")
    ee = torch.tensor(e, device="cuda")
    u = torch.empty(n * n, dtype=torch.float64, device="cuda")
    vt = torch.empty(n * n, dtype=torch.float64, device="cuda")
    hp.mdbdsdc_dev(dd, ee, u, vt)
    s = dd
    U = u.view(n, n).T      # U[:, j]
    VT = vt.view(n, n).T    # VT[i, :]
    dt, et = torch.tensor(d, device="cuda"), torch.tensor(e, device="cuda")
    # B V = U S  with  (B x)_i = d_i x_i + e_i x_{i+1}
    V = VT.T
    BV = dt[:, None] * V
    BV[:-1] += et[:, None] * V[1:]
    nb = float(np.max(np.abs(d) + np.concatenate([np.abs(e), [0.0]])))
    res = float(torch.linalg.norm(BV - U * s[None, :])) / (n * nb)
    assert res <= RES_TOL, res
    g = torch.randn(n, 8, dtype=torch.float64, device="cuda",
                    generator=torch.Generator(device="cuda").manual_seed(1))
    for Q in (U, V):
        y = Q.T @ (Q @ g) - g
        assert float(torch.sqrt(torch.sum(y * y) / 8)) / n <= ORTH_TOL
    sc = s.cpu().numpy()
    assert np.all(np.diff(sc) <= 0)
    from scipy.linalg import eigvalsh_tridiagonal
    # singular values from the Golub-Kahan tridiagonal (zero diagonal,
    # off-diagonal d1, e1, d2, ...): its positive eigenvalues
    gk = np.empty(2 * n - 1)
    gk[0::2] = d
    gk[1::2] = e
    lam = eigvalsh_tridiagonal(np.zeros(2 * n), gk)
    sref = np.sort(lam[n:])[::-1]
    assert float(np.max(np.abs(sc - sref))) / nb <= SV_TOL


@pytest.mark.parametrize("kind", ["ones", "random"])
@pytest.mark.parametrize("precision", [0, 1])
def test_svd_hss_merges(kind, precision):
    # merges with K >= bsmlz go through two HSS products (DHSSVCS); HSS leaf 64,
    # tolerance 1e-14 as the acceptance bar states
    n = 2048
    if kind == "ones":
        d, e = np.ones(n), np.ones(n - 1)
    else:
        d, e = _bidiag(n, seed=21)
    old = hp.set_config(bsmlz=48, hss_leaf=64, tol=1e-14, precision=precision)
    try:
        s, U, VT = hp.svd_bidiagonal(d, e)
        st = hp.get_stats()
    finally:
        hp.restore_config(old)
    assert st["n_hss_merges"] > 0
    _check(d, e, s, U, VT)
