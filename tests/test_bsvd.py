"""Banded SVD by structured banded divide and conquer (MDBDSVD,
SRC/mdbdsvd.f90:1).

The reference's test (TEST/test_bdc1.f90) fills AB (LDAB = SB + 1, N = 5000,
SB = 5) with uniform [0, 1) numbers, runs MDBDSVD with SMLSIZ = 75 and prints
the largest difference of its singular values from LAPACK DGESDD's.  Here:

CPU: the numpy restatement (oracle/bsvd_ref.py: the reference's tree, QR / RZ
of the inserted rows, the first row then SB - 1 updates) against LAPACK's
singular values, residual and orthogonality; its tree against MDBDSVDT's
shape; the Fortran entry point's argument checks.
GPU: the Fortran entry point and the device API against LAPACK (singular
values within 1e-13 ||B||, ||B - U S V^T||_F / (n ||B||) and the
orthogonality of U and V, ||Q^T Q - I||_F / n, at most 1e-12) and against the
restatement, on the reference's case at full size, several semibandwidths (1,
the widest supported 32), a single-leaf matrix, a Toeplitz band (clustered
singular values: rotations in the deflation) and a band with zero rows (zero
singular values: rank-deficient leaves and equal poles)."""
import numpy as np
import pytest
import scipy.linalg as sla

import hsspack_gb300 as hp
from oracle import bsvd_ref as ref


def _band(n, sb, seed, kind="uniform"):
    rng = np.random.default_rng(seed)
    if kind == "uniform":  # TEST/test_bdc1.f90: random_number(AB)
        ab = rng.uniform(0.0, 1.0, (sb + 1, n))
    elif kind == "normal":
        ab = rng.standard_normal((sb + 1, n))
    elif kind == "toeplitz":
        ab = np.repeat(rng.uniform(0.5, 1.0, (sb + 1, 1)), n, axis=1)
    elif kind == "zero_rows":
        ab = rng.standard_normal((sb + 1, n))
        for i in range(7, n, 97):  # row i of B: AB(sb + i - j, j), j = i .. i + sb
            for j in range(i, min(n, i + sb + 1)):
                ab[sb + i - j, j] = 0.0
    return np.asfortranarray(ab)


def _check(B, s, U, VT, sl=None, sval_tol=1e-13, tol=1e-12):
    n = B.shape[0]
    if sl is None:
        sl = sla.svdvals(B)
    nb = sl[0]
    assert np.all(np.diff(s) <= 0)
    assert np.max(np.abs(s - sl)) <= sval_tol * nb, np.max(np.abs(s - sl)) / nb
    res = np.linalg.norm(B - (U * s) @ VT) / (n * nb)
    ou = np.linalg.norm(U.T @ U - np.eye(n)) / n
    ov = np.linalg.norm(VT @ VT.T - np.eye(n)) / n
    assert res <= tol and ou <= tol and ov <= tol, (res, ou, ov)


# ------------------------------------------------------------------ CPU ----
@pytest.mark.parametrize("n,sb,sml,kind", [(300, 5, 25, "uniform"), (640, 3, 25, "normal"),
                                           (500, 1, 10, "normal"), (450, 12, 25, "uniform"),
                                           (400, 4, 25, "toeplitz"), (500, 6, 25, "zero_rows")])
def test_oracle_vs_lapack(n, sb, sml, kind):
    ab = _band(n, sb, n + sb, kind)
    s, U, VT = ref.mdbdsvd(ab, sb, sml)
    _check(ref.band_to_dense(ab, sb), s, U, VT)


def test_oracle_tree_is_mdbdsvdt():
    # the reference's test: N = 5000, SB = 5, SMLSIZ = 75 -> 6 levels, 64 nodes
    # at the bottom, 128 leaves; leaves plus center rows tile the rows
    levels, leaves = ref.tree(5000, 5, 75)
    assert len(levels) == 6 and len(levels[-1]) == 32 and len(leaves) == 64
    rows = sum(r for _, r, _ in leaves) + 5 * sum(len(lv) for lv in levels)
    assert rows == 5000
    assert leaves[-1][2] == leaves[-1][1]  # the last leaf has no extra columns
    assert all(c == r + 5 for _, r, c in leaves[:-1])


@pytest.mark.parametrize("sb", [1, 2, 5, 8, 12, 16, 20, 31, 32])
def test_library_tree_tiles_the_band(sb):
    # the library's cut of the band (host logic): leaves in row order separated
    # by exactly one center block of sb rows, 2^depth leaves, extra columns on
    # all but the last, at most 64 rows (32 whenever the band allows it); where
    # MDBDSVDT's own tree is valid and its leaves already have at most 32 rows,
    # the library's leaves are exactly MDBDSVDT's
    for n in [sb, sb + 1, 33, 64, 65, 100, 257, 1000, 1500, 5000, 16384]:
        if n < sb:
            continue
        depth, leaves = hp.bsvd_tree(n, sb, 25)
        assert len(leaves) == 2 ** depth
        pos = 0
        for i, (a, r, c) in enumerate(leaves):
            assert a == pos and r >= 1
            assert c == r + (sb if i < len(leaves) - 1 else 0)
            assert r <= 64
            pos = a + r + sb
        assert pos - sb == n
        if sb <= 16:
            assert max(r for _, r, _ in leaves) <= 32, (n, sb)
        if n > 32:
            try:
                _, ref_leaves = ref.tree(n, sb, 25)
            except AssertionError:  # the reference's halving leaves a side empty
                continue
            if max(r for _, r, _ in ref_leaves) <= 32:
                assert [(a, r, c) for a, r, c in ref_leaves] == leaves


def test_library_tree_rejects_bad_arguments():
    for args in [(0, 1), (10, 0), (10, 11), (100, 33)]:
        with pytest.raises(hp.HssError):
            hp.bsvd_tree(*args)


def _call(n, sb, ldab, ldu, ldvt, smlsiz):
    ab = np.zeros((max(ldab, 1), max(n, 1)), order="F")
    u = np.zeros((max(ldu, 1), max(n, 1)), order="F")
    vt = np.zeros((max(ldvt, 1), max(n, 1)), order="F")
    one = np.zeros(1)
    return hp.mdbdsvd(n, sb, ab, ldab, one, np.zeros(max(n, 1)), u, ldu, vt, ldvt, smlsiz, one, 1,
                      np.zeros(1, dtype=np.int32))


def test_fortran_argument_checks():
    # SRC/mdbdsvd.f90:120-137: -2 (N < 0 or N < SB), -3 (SB < 1), then -9 / -10
    # / -11 override; -4 (LDAB) and -3 for SB > 32 are this library's
    assert _call(3, 5, 6, 3, 3, 25)[0] == -2
    assert _call(-1, 1, 2, 1, 1, 25)[0] == -2
    assert _call(100, 0, 2, 100, 100, 25)[0] == -3
    assert _call(100, 5, 6, 99, 100, 25)[0] == -9
    assert _call(3, 5, 6, 2, 3, 25)[0] == -9  # the second group wins
    assert _call(100, 5, 6, 100, 99, 25)[0] == -10
    assert _call(100, 5, 6, 100, 100, 2)[0] == -11
    assert _call(100, 5, 5, 100, 100, 25)[0] == -4
    assert _call(100, 33, 34, 100, 100, 25)[0] == -3
    assert _call(0, 0, 1, 1, 1, 25)[0] == -3
    assert _call(0, 1, 2, 1, 1, 25)[0] == -2  # N < SB


# ------------------------------------------------------------------ GPU ----
@pytest.mark.gpu
def test_reference_case_full_size():
    # TEST/test_bdc1.f90: N = 5000, SB = 5, AB uniform [0, 1), SMLSIZ = 75
    import torch
    n, sb = 5000, 5
    ab = _band(n, sb, 2013)
    s, U, VT = hp.svd_banded(ab, sb, 75)
    B = ref.band_to_dense(ab, sb)
    sl = sla.svdvals(B)
    assert np.all(np.diff(s) <= 0)
    assert np.max(np.abs(s - sl)) <= 1e-13 * sl[0]
    Bt = torch.tensor(B, device="cuda")
    Ut = torch.tensor(U, device="cuda")
    Vt = torch.tensor(VT, device="cuda")
    st = torch.tensor(s, device="cuda")
    res = float(torch.linalg.norm(Bt - (Ut * st) @ Vt)) / (n * sl[0])
    eye = torch.eye(n, dtype=torch.float64, device="cuda")
    ou = float(torch.linalg.norm(Ut.T @ Ut - eye)) / n
    ov = float(torch.linalg.norm(Vt @ Vt.T - eye)) / n
    assert res <= 1e-12 and ou <= 1e-12 and ov <= 1e-12, (res, ou, ov)
    assert hp.get_stats()["n_levels"] >= 6


@pytest.mark.gpu
@pytest.mark.parametrize("n,sb,kind", [(1000, 1, "normal"), (1200, 3, "uniform"),
                                       (1500, 32, "normal"), (50, 5, "normal"),
                                       (2000, 4, "toeplitz"), (1600, 6, "zero_rows"),
                                       (2048, 8, "uniform")])
def test_vs_lapack(n, sb, kind):
    ab = _band(n, sb, 7 * n + sb, kind)
    s, U, VT = hp.svd_banded(ab, sb, 25)
    _check(ref.band_to_dense(ab, sb), s, U, VT)


@pytest.mark.gpu
@pytest.mark.parametrize("pred", [2, 3])
@pytest.mark.parametrize("n,sb,kind", [(3000, 5, "uniform"), (1600, 6, "zero_rows"),
                                       (2000, 4, "toeplitz"), (1500, 32, "normal")])
def test_fp32_presolved_starts(n, sb, kind, pred):
    # predictor = 2 / 3: every append's secular equation starts from the FP32
    # pre-solve in squared mode (3: refined by one float-float step)
    old = hp.set_config(predictor=pred, precision=1)
    try:
        ab = _band(n, sb, 3 * n + sb, kind)
        s, U, VT = hp.svd_banded(ab, sb, 25)
    finally:
        hp.restore_config(old)
    _check(ref.band_to_dense(ab, sb), s, U, VT)


@pytest.mark.gpu
@pytest.mark.parametrize("n,sb", [(1, 1), (2, 1), (2, 2), (7, 3), (7, 7), (64, 32), (65, 32),
                                  (66, 32), (97, 31)])
def test_small_and_edge_shapes(n, sb):
    # a single element, sb = n, the widest band as one leaf (n = 64, sb = 32:
    # 64 x 64) and the smallest trees with a one-row leaf (n = 65, 66)
    ab = _band(n, sb, 100 * n + sb, "normal")
    s, U, VT = hp.svd_banded(ab, sb, 25)
    _check(ref.band_to_dense(ab, sb), s, U, VT)


@pytest.mark.gpu
@pytest.mark.parametrize("sb", [2, 7])
def test_vs_oracle(sb):
    n = 700
    ab = _band(n, sb, 11 + sb, "normal")
    s, U, VT = hp.svd_banded(ab, sb, 25)
    so, Uo, VTo = ref.mdbdsvd(ab, sb, 25)
    assert np.max(np.abs(s - so)) <= 1e-13 * so[0]
    # singular subspaces agree: clusters of singular values closer than
    # 1e-7 ||B|| (localised vectors of a random band can be nearly degenerate)
    # span the same spaces, i.e. W = Uo^T U is orthogonal and block diagonal
    cut = np.flatnonzero(so[:-1] - so[1:] > 1e-7 * so[0]) + 1
    lab = np.zeros(n, dtype=np.int64)
    lab[cut] = 1
    lab = np.cumsum(lab)
    for A, Ao in ((U, Uo), (VT.T, VTo.T)):
        W = Ao.T @ A
        off = np.where(lab[:, None] != lab[None, :], W, 0.0)
        assert np.max(np.abs(off)) <= 1e-8
        assert np.linalg.norm(W.T @ W - np.eye(n)) <= 1e-11 * n


@pytest.mark.gpu
def test_device_api_and_lower_level_sizes():
    import torch
    n, sb = 3000, 6
    ab = _band(n, sb, 5, "normal")
    abt = torch.tensor(ab.ravel(order="F"), device="cuda")
    s = torch.empty(n, dtype=torch.float64, device="cuda")
    u = torch.empty(n * n, dtype=torch.float64, device="cuda")
    vt = torch.empty(n * n, dtype=torch.float64, device="cuda")
    hp.mdbdsvd_dev(sb, abt, s, u, vt, smlsiz=25)
    torch.cuda.synchronize()
    B = ref.band_to_dense(ab, sb)
    U = u.cpu().numpy().reshape(n, n, order="F")
    VT = vt.cpu().numpy().reshape(n, n, order="F")
    _check(B, s.cpu().numpy(), U, VT)
    st = hp.get_stats()
    assert st["n_merges"] > 0 and st["secular_roots"] > 0
