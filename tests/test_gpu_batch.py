"""Batched uneven tridiagonal eigensolves (hss_mdstedc_batch_dev) against
LAPACK DSTEDC per problem and against one hss_mdstedc_dev call per problem.

Tolerances as for the single solves: eigenvalues within 1e-13 * ||T||,
||TQ - QW||_F/(n||T||) <= 1e-12, ||Q^T Q - I||_F / n <= 1e-12."""
import numpy as np
import pytest
import torch

import oracle
import hsspack_gb300 as hp
from helpers import eig_metrics, rand_tridiag, toeplitz_eigs, toeplitz_tridiag

EV_TOL, RES_TOL, ORTH_TOL = 1e-13, 1e-12, 1e-12

pytestmark = pytest.mark.gpu


def _check(d, e, w, Q):
    wl, _ = oracle.dstedc_lapack(d, e)
    ev, res, orth = eig_metrics(d, e, w, Q, wl)
    assert np.all(np.diff(w) >= 0)
    assert ev <= EV_TOL and res <= RES_TOL and orth <= ORTH_TOL, (len(d), ev, res, orth)


def _edge_problems():
    probs = []
    for n, seed in [(1, 1), (2, 2), (5, 3), (12, 4), (25, 5), (26, 6), (100, 7), (333, 8),
                    (700, 9)]:
        probs.append(rand_tridiag(n, seed))
    probs.append(toeplitz_tridiag(300))
    # an exact split: tiny coupling in the middle gives two unreduced blocks
    d, e = rand_tridiag(400, 10)
    e[199] = 1e-300
    probs.append((d, e))
    # graded entries (scaling per block)
    d, e = rand_tridiag(257, 11)
    probs.append((d * 1e6, e * 1e6))
    probs.append((np.zeros(40), np.zeros(39)))  # zero matrix: everything deflates
    return probs


@pytest.mark.parametrize("precision", [0, 1])
def test_batch_edge_cases(precision):
    probs = _edge_problems()
    old = hp.set_config(precision=precision)
    try:
        out = hp.eigh_tridiagonal_batch(probs)
    finally:
        hp.restore_config(old)
    for (d, e), (w, Q) in zip(probs, out):
        _check(d, e, w, Q)
    w_t = out[9][0]
    assert np.max(np.abs(w_t - toeplitz_eigs(300))) <= 4 * EV_TOL


def test_batch_matches_single_calls():
    rng = np.random.default_rng(5)
    sizes = np.round(np.exp(rng.uniform(np.log(30), np.log(900), 24))).astype(int)
    probs = [rand_tridiag(int(n), 100 + i) for i, n in enumerate(sizes)]
    out = hp.eigh_tridiagonal_batch(probs)
    for (d, e), (w, Q) in zip(probs, out):
        w1, Q1 = hp.eigh_tridiagonal(d, e)
        assert np.max(np.abs(w - w1)) <= 1e-14 * max(1.0, np.max(np.abs(w1)))
        _check(d, e, w, Q)


def test_batch_empty_and_bad_sizes():
    assert hp.load().hss_mdstedc_batch_dev(0, None, None, None, None, None) == 0
    bad = np.array([3, -1], dtype=np.int32)
    rc = hp.load().hss_mdstedc_batch_dev(2, bad.ctypes.data, None, None, None, None)
    assert rc == -2
    out = hp.eigh_tridiagonal_batch([(np.zeros(0), np.zeros(0)), rand_tridiag(50, 1)])
    assert out[0][0].size == 0
    _check(*rand_tridiag(50, 1), *out[1])


def _residuals_on_device(sizes, D, E, w, z):
    """Per-problem ||TQ - QW||_F / (n ||T||) and eigenvalue sortedness, on the GPU."""
    o, oz = hp.batch_offsets(sizes)
    res = []
    for p, n in enumerate(sizes):
        n = int(n)
        Q = z[oz[p]:oz[p + 1]].view(n, n).T  # column-major block
        d = D[o[p]:o[p + 1]]
        e = E[o[p]:o[p + 1] - 1]
        R = d[:, None] * Q - Q * w[o[p]:o[p + 1]][None, :]
        R[:-1] += e[:, None] * Q[1:]
        R[1:] += e[:, None] * Q[:-1]
        a = d.abs().clone()
        a[:-1] += e.abs()
        a[1:] += e.abs()
        res.append(float(torch.linalg.norm(R)) / (n * float(a.max())))
    return np.array(res)


def test_batch_512_uneven_full_size():
    # the batch workload: 512 problems, n log-uniform in [256, 4096] (seed 2)
    rng = np.random.default_rng(2)
    sizes = np.round(np.exp(rng.uniform(np.log(256), np.log(4096), 512))).astype(np.int32)
    probs = [rand_tridiag(int(n), 1000 + i) for i, n in enumerate(sizes)]
    _, D, E = hp.pack_batch(probs)
    o, oz = hp.batch_offsets(sizes)
    d = torch.tensor(D, device="cuda")
    e = torch.tensor(E, device="cuda")
    z = torch.empty(int(oz[-1]), dtype=torch.float64, device="cuda")
    hp.mdstedc_batch_dev(sizes, d, e, z)
    Dd, Ed = torch.tensor(D, device="cuda"), torch.tensor(E, device="cuda")
    res = _residuals_on_device(sizes, Dd, Ed, d, z)
    assert res.max() <= RES_TOL, res.max()
    w = d.cpu().numpy()
    for p in range(len(sizes)):
        assert np.all(np.diff(w[o[p]:o[p + 1]]) >= 0)
    # eigenvalues against LAPACK and orthogonality on a seeded sample
    for p in np.random.default_rng(3).choice(len(sizes), 6, replace=False):
        n = int(sizes[p])
        Q = z[oz[p]:oz[p + 1]].view(n, n).T
        orth = float(torch.linalg.norm(Q.T @ Q - torch.eye(n, dtype=torch.float64,
                                                             device="cuda"))) / n
        assert orth <= ORTH_TOL, orth
        dp, ep = probs[p]
        wl, _ = oracle.dstedc_lapack(dp, ep)
        nt = max(np.abs(dp).max() + 2 * np.abs(ep).max(), 1e-300)
        assert np.max(np.abs(w[o[p]:o[p + 1]] - wl)) / nt <= EV_TOL
