"""SVD updating (SvdHssUpdat, SRC/SvdHssUpdat.f90:1).

CPU: the numpy restatement (oracle/svdupd_ref.py) is pinned against a dense SVD
of the updated matrix, and the library's host deflation (MDLASD20) must equal
the restatement's decisions bit for bit.  GPU: the Fortran entry point against
the restatement on the reference's own test case (TEST/testUpsvdCauchy.f90:
F evenly spaced in (0.1, 9), Z uniform with Z(10) = 1e-16 and Z(200) = 1e-17,
V = I, ni = 50, tol = 1e-15; N = 299 and 1000), plus a random orthogonal V,
close poles (deflating rotations), a small K (one dense block) and the device
entry point.  Tolerances: singular values 1e-13 relative to the largest;
vectors 1e-11 (the HSS tolerance times the products' growth); orthogonality of
the new V^T 1e-12."""
import numpy as np
import pytest

import hsspack_gb300 as hp
from oracle import svdupd_ref as ref


def _reference_case(n, seed):
    """TEST/testUpsvdCauchy.f90:55-78 with a seeded generator."""
    rng = np.random.default_rng(seed)
    sa, sb = 0.1, 9.0
    gap = (sb - sa) / (2 * n)
    f = sa + (2 * np.arange(1, n + 1) - 1) * gap
    z = rng.uniform(0.0, 1.0, n)
    z[9] = 1e-16
    if n > 199:
        z[199] = 1e-17
    return f, z


def _close_pole_case(n, seed):
    rng = np.random.default_rng(seed)
    f = np.sort(rng.uniform(0.1, 5.0, n))
    for j in range(5, n - 1, 37):  # pairs of equal poles: rotations
        f[j + 1] = f[j]
    z = rng.uniform(-1.0, 1.0, n)
    z[::53] = 1e-18
    return f, z


def _orthogonal(n, seed):
    rng = np.random.default_rng(seed)
    q, r = np.linalg.qr(rng.standard_normal((n, n)))
    return q * np.sign(np.diag(r))


# ------------------------------------------------------------------ CPU ----
@pytest.mark.parametrize("case", ["reference", "close"])
def test_oracle_matches_dense_svd(case):
    n = 160
    f, z = _reference_case(n, 3) if case == "reference" else _close_pole_case(n, 4)
    VT = _orthogonal(n, 5).T
    K, sig, fo, zo, VTn = ref.svdhssupdat(f, z, VT)
    M = np.vstack([np.diag(f), z[None, :]]) @ VT  # [A; a^T] up to the left factor
    s_dense = np.sort(np.linalg.svd(M, compute_uv=False))
    s_ours = np.sort(np.concatenate([sig, fo[K:]]))
    assert np.max(np.abs(s_ours - s_dense)) <= 1e-13 * s_dense[-1]
    # every row of the new V^T is a right singular vector: |M v| = sigma
    vals = np.concatenate([sig, fo[K:]])
    assert np.max(np.abs(np.linalg.norm(M @ VTn.T, axis=0) - vals)) <= 1e-12 * s_dense[-1]
    assert np.max(np.abs(VTn @ VTn.T - np.eye(n))) <= 1e-13
    assert K < n  # the planted tiny z entries deflate


@pytest.mark.parametrize("case", ["reference", "close"])
def test_host_deflation_matches_oracle(case):
    n = 1000
    f, z = _reference_case(n, 7) if case == "reference" else _close_pole_case(n, 8)
    K, fo, zo, idxp, nrot = hp.svdupd_deflate(f, z)
    K2, fo2, zo2, idxp2, rots = ref.deflate(f, z)
    assert K == K2 and nrot == len(rots)
    assert np.array_equal(idxp, idxp2)
    assert np.array_equal(fo, fo2) and np.array_equal(zo, zo2)
    if case == "close":
        assert nrot > 0


def test_host_deflation_all_small():
    f = np.linspace(1.0, 2.0, 8)
    z = np.full(8, 1e-20)
    K, fo, zo, idxp, nrot = hp.svdupd_deflate(f, z)
    K2, fo2, zo2, idxp2, _ = ref.deflate(f, z)
    assert K == K2 == 0
    assert np.array_equal(idxp, idxp2) and np.array_equal(fo, fo2) and np.array_equal(zo, zo2)


# ------------------------------------------------------------------ GPU ----
def _check(f, z, VT, ni=50, tol=1e-15):
    n = len(f)
    V = np.asfortranarray(VT.copy())
    D, Fo, Zo = hp.svdhssupdat(f, z, V, tol, ni)
    K, sig, fo, zo, VTn = ref.svdhssupdat(f, z, VT)
    smax = max(np.max(np.abs(f)), 1.0)
    assert np.max(np.abs(D[:K] - sig)) <= 1e-13 * smax
    assert np.array_equal(D[K:], fo[K:])
    assert np.array_equal(Fo, fo)
    assert np.max(np.abs(Zo[:K] - zo[:K])) <= 1e-12 * np.max(np.abs(zo[:K]))
    assert np.max(np.abs(V - VTn)) <= 1e-11
    G = V @ V.T
    assert np.max(np.abs(G - np.eye(n))) <= 1e-12
    return K


@pytest.mark.gpu
@pytest.mark.parametrize("n", [299, 1000])
def test_reference_case_identity_v(n):
    f, z = _reference_case(n, 11)
    K = _check(f, z, np.eye(n))
    assert K == n - (2 if n > 199 else 1)
    st = hp.get_stats()
    assert 0 < st["max_rank"] < K


@pytest.mark.gpu
def test_random_orthogonal_v_and_close_poles():
    n = 1200
    f, z = _close_pole_case(n, 12)
    _check(f, z, _orthogonal(n, 13).T, ni=64, tol=1e-14)


@pytest.mark.gpu
def test_small_k_dense_block():
    n = 300
    f, z = _reference_case(n, 14)
    z[40:] = 1e-19  # K = 39 < 2 ni: one dense block
    K = _check(f, z, _orthogonal(n, 15).T, ni=50)
    assert K == 39


@pytest.mark.gpu
def test_device_entry_point():
    import torch
    n = 2048
    f, z = _reference_case(n, 16)
    VT = _orthogonal(n, 17).T
    d_t = torch.zeros(n, dtype=torch.float64, device="cuda")
    f_t = torch.tensor(f, device="cuda")
    z_t = torch.tensor(z, device="cuda")
    vt_t = torch.tensor(np.asfortranarray(VT).ravel(order="F"), device="cuda")
    K = hp.svdhssupdat_dev(d_t, f_t, z_t, vt_t, 1e-14, 64)
    K2, sig, fo, zo, VTn = ref.svdhssupdat(f, z, VT)
    assert K == K2
    assert np.max(np.abs(d_t.cpu().numpy()[:K] - sig)) <= 1e-13 * np.max(f)
    Vn = vt_t.cpu().numpy().reshape(n, n, order="F")
    assert np.max(np.abs(Vn - VTn)) <= 1e-11
