"""Banded divide and conquer (MDSBEDC / MDSBEVD path) on the GPU against LAPACK
DSBEVD and the numpy restatement of the reference algorithm.

Tolerances as for the tridiagonal solver: eigenvalues within 1e-13 * ||A||,
||AQ - QW||_F / (n ||A||) <= 1e-12, ||Q^T Q - I||_F / n <= 1e-12."""
import numpy as np
import pytest
import torch

import hsspack_gb300 as hp
from oracle import band_ref

EV_TOL, RES_TOL, ORTH_TOL = 1e-13, 1e-12, 1e-12

pytestmark = pytest.mark.gpu


def _band(n, kd, seed):
    rng = np.random.default_rng(seed)
    return np.asfortranarray(rng.uniform(-1.0, 1.0, (kd + 1, n)))


def _rowsum(ab):
    """max_i sum_j |A(i, j)| of the band matrix (upper storage), >= ||A||_2."""
    kd, n = ab.shape[0] - 1, ab.shape[1]
    r = np.abs(ab[kd]).copy()
    for o in range(1, kd + 1):
        a = np.abs(ab[kd - o, o:])
        r[:-o] += a
        r[o:] += a
    return r.max()


def _check(ab, w, Q, lower=False):
    A = band_ref.band_to_dense(ab, lower=lower)
    n = A.shape[0]
    na = max(np.abs(A).sum(axis=1).max(), 1e-300)
    wl, _ = band_ref.eig_banded_lapack(ab, lower=lower)
    assert np.all(np.diff(w) >= 0)
    ev = np.max(np.abs(w - wl)) / na
    res = np.linalg.norm(A @ Q - Q * w[None, :]) / (n * na)
    orth = np.linalg.norm(Q.T @ Q - np.eye(n)) / n
    assert ev <= EV_TOL and res <= RES_TOL and orth <= ORTH_TOL, (n, ev, res, orth)


@pytest.mark.parametrize("n,kd", [(30, 2), (100, 4), (257, 3), (700, 4), (1000, 8), (2048, 4),
                                  (300, 16), (400, 32), (65, 5)])
@pytest.mark.parametrize("precision", [0, 1])
def test_band_random(n, kd, precision):
    ab = _band(n, kd, seed=n + kd)
    old = hp.set_config(precision=precision)
    try:
        w, Q = hp.eigh_banded(ab)
    finally:
        hp.restore_config(old)
    _check(ab, w, Q)


def test_band_lower_storage_and_restatement():
    n, kd = 500, 4
    ab = _band(n, kd, seed=5)
    A = band_ref.band_to_dense(ab)
    abl = np.zeros_like(ab)
    for j in range(n):
        for i in range(j, min(n, j + kd + 1)):
            abl[i - j, j] = A[i, j]
    w1, Q1 = hp.eigh_banded(ab)
    w2, Q2 = hp.eigh_banded(np.asfortranarray(abl), lower=True)
    assert np.max(np.abs(w1 - w2)) <= 1e-14 * np.max(np.abs(w1))
    _check(abl, w2, Q2, lower=True)
    wr, _ = band_ref.band_dc(A, kd)
    assert np.max(np.abs(w1 - wr)) <= EV_TOL * np.abs(A).sum(axis=1).max()


@pytest.mark.parametrize("kd", [0, 1])
def test_band_narrow_goes_tridiagonal(kd):
    ab = _band(300, kd, seed=kd)
    w, Q = hp.eigh_banded(ab)
    _check(ab, w, Q)


def test_band_structured_and_batched_modes():
    # a graded band (entries spanning 8 orders) and the per-merge launch mode
    n, kd = 600, 4
    ab = _band(n, kd, seed=9) * np.logspace(0, -8, n)[None, :]
    _check(np.asfortranarray(ab), *hp.eigh_banded(np.asfortranarray(ab)))
    old = hp.set_config(batched=0)
    try:
        ab2 = _band(400, 3, seed=10)
        _check(ab2, *hp.eigh_banded(ab2))
    finally:
        hp.restore_config(old)


def test_mdsbevd_fortran_entry():
    n, kd = 200, 4
    ab = _band(n, kd, seed=3)
    d = np.zeros(n)
    q = np.zeros((n, n), order="F")
    work, iwork = np.zeros(1), np.zeros(1, dtype=np.int32)
    assert hp.mdsbevd("I", "U", n, kd, ab.copy(order="F"), kd + 1, d, q, n, work, -1, iwork,
                      -1) == 0
    assert work[0] == 1 + 4 * n + n * n and iwork[0] == 3 + 5 * n
    info = hp.mdsbevd("I", "U", n, kd, ab.copy(order="F"), kd + 1, d, q, n, work, int(work[0]),
                      iwork, int(iwork[0]))
    assert info == 0
    _check(ab, d, q)


def test_band_16384_kd4_full_size():
    # the banded workload: n = 16384, bandwidth 4, entries iid U[-1, 1]
    n, kd = 16384, 4
    rng = np.random.default_rng(0)
    ab = rng.uniform(-1.0, 1.0, (kd + 1, n))
    abd = torch.tensor(np.ascontiguousarray(ab.T), device="cuda")  # memory = column-major ab
    w = torch.empty(n, dtype=torch.float64, device="cuda")
    z = torch.empty(n * n, dtype=torch.float64, device="cuda")
    hp.mdsbevd_dev(kd, abd, w, z)
    Q = z.view(n, n).T  # Q[:, j] = eigenvector j
    # A Q on the device from the band: A[i, i+o] = ab[kd - o, i + o]
    abt = torch.tensor(ab, device="cuda")
    AQ = abt[kd][:, None] * Q
    for o in range(1, kd + 1):
        a = abt[kd - o, o:]  # A[i, i + o], i = 0 .. n-o-1
        AQ[:-o] += a[:, None] * Q[o:]
        AQ[o:] += a[:, None] * Q[:-o]
    na = _rowsum(ab)
    res = float(torch.linalg.norm(AQ - Q * w[None, :])) / (n * na)
    assert res <= RES_TOL, res
    g = torch.randn(n, 8, dtype=torch.float64, device="cuda",
                    generator=torch.Generator(device="cuda").manual_seed(1))
    y = Q.T @ (Q @ g) - g
    orth = float(torch.sqrt(torch.sum(y * y) / 8)) / n
    assert orth <= ORTH_TOL, orth
    from scipy.linalg import eig_banded
    wl = eig_banded(ab, eigvals_only=True)
    assert float(np.max(np.abs(w.cpu().numpy() - wl))) / na <= EV_TOL


# Bandwidths above the band divide and conquer's limit and eigenvalue-only
# calls go through the device reduction to tridiagonal form (Householder
# bulge chasing; the reference's LAPACK DSBTRD route, SRC/mdsbedc.f90:274-276
# and :311-318): same acceptance bar against LAPACK DSBEVD.


@pytest.mark.parametrize("n,kd", [(50, 33), (300, 40), (700, 64), (257, 100), (40, 39),
                                  (30, 45)])
@pytest.mark.parametrize("lower", [False, True])
def test_band_wide_reduction(n, kd, lower):
    ab = _band(n, kd, seed=n + 3 * kd)
    if lower:  # the same matrix in lower storage
        A = band_ref.band_to_dense(ab)
        ab = np.zeros_like(ab)
        for j in range(n):
            for i in range(j, min(n, j + kd + 1)):
                ab[i - j, j] = A[i, j]
        ab = np.asfortranarray(ab)
    w, Q = hp.eigh_banded(ab, lower=lower)
    _check(ab, w, Q, lower=lower)


@pytest.mark.parametrize("n,kd", [(300, 2), (1000, 4), (500, 16), (600, 48), (2048, 4)])
def test_band_eigenvalues_only_reduction(n, kd):
    ab = _band(n, kd, seed=2 * n + kd)
    w = np.zeros(n)
    z = np.zeros((1, 1), order="F")
    work, iwork = np.zeros(1), np.zeros(1, dtype=np.int32)
    info = hp.mdsbedc("N", "U", n, kd, ab.copy(order="F"), kd + 1, w, z, 1, work, -1, iwork, -1)
    assert info == 0 and work[0] == 2 * n and iwork[0] == 1
    info = hp.mdsbedc("N", "U", n, kd, ab.copy(order="F"), kd + 1, w, z, 1, work, 2 * n, iwork, 1)
    assert info == 0
    wl, _ = band_ref.eig_banded_lapack(ab)
    na = np.abs(band_ref.band_to_dense(ab)).sum(axis=1).max()
    assert np.all(np.diff(w) >= 0)
    assert np.max(np.abs(w - wl)) / na <= EV_TOL
    # the eigenvalues-only path of MDSBEVD as well
    d = np.zeros(n)
    info = hp.mdsbevd("N", "U", n, kd, ab.copy(order="F"), kd + 1, d, z, 1, work, 1, iwork, 1)
    assert info == 0 and np.array_equal(d, w)


def test_band_wide_device_entry():
    n, kd = 900, 50
    ab = _band(n, kd, seed=77)
    abd = torch.tensor(np.ascontiguousarray(ab.T), device="cuda")
    w = torch.empty(n, dtype=torch.float64, device="cuda")
    z = torch.empty(n * n, dtype=torch.float64, device="cuda")
    hp.mdsbevd_dev(kd, abd, w, z)
    _check(ab, w.cpu().numpy(), z.cpu().numpy().reshape(n, n).T)
