"""GPU HSS compression + multiply (DHSSEVC) against the dense Cauchy-like
product and the oracle's structured RRLU, and HSS merges inside the DC solve."""
import numpy as np
import pytest
import torch

import oracle
import hsspack_gb300 as hp
from helpers import eig_metrics, secular_problem, toeplitz_eigs, toeplitz_tridiag

pytestmark = pytest.mark.gpu


def _dev(a):
    return torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


def _problem(k, seed):
    d, z, rho = secular_problem(k, seed=seed, normalize=False)
    lam, difl, difr = oracle.secular(d, z, rho)
    zh, alpha = oracle.lowner(d, difl, difr, z)
    return d, zh, alpha, difl, difr


@pytest.mark.parametrize("k,ni,tol,nrows", [(600, 64, 1e-14, 97), (2000, 200, 1e-17, 300),
                                            (4096, 128, 1e-14, 256), (1000, 2000, 1e-14, 64)])
@pytest.mark.parametrize("precision", [0, 1])
def test_dhssevc_vs_dense(k, ni, tol, nrows, precision):
    d, zh, alpha, difl, difr = _problem(k, k)
    C = oracle.cauchy_eig_dense(d, zh, alpha, difl, difr)
    X = np.random.default_rng(k).standard_normal((nrows, k))
    Xd = _dev(np.asfortranarray(X).T.copy())  # rows of the tensor = columns of X
    old = hp.set_config(precision=precision)
    try:
        hp.dhssevc_dev(_dev(d), _dev(zh), _dev(alpha), _dev(difl), _dev(difr), Xd, nrows, nrows,
                       ni=ni, tol=tol)
    finally:
        hp.restore_config(old)
    Y = Xd.cpu().numpy().T
    ref = X @ C
    err = np.max(np.abs(Y - ref)) / np.max(np.abs(ref))
    assert err <= 1e-12, err
    _, r_or = oracle.dhssevc(d, zh, alpha, difl, difr, np.asfortranarray(X), ni=ni, tol=tol)
    r_gpu = hp.get_stats()["max_rank"]
    if ni < k:
        assert abs(r_gpu - r_or) <= 8, (r_gpu, r_or)


@pytest.mark.parametrize("n,bsmlz,leaf,tol", [(2048, 200, 64, 1e-14), (3000, 500, 200, 1e-17)])
@pytest.mark.parametrize("precision", [0, 1])
def test_dc_with_hss_merges(n, bsmlz, leaf, tol, precision):
    d, e = toeplitz_tridiag(n)
    old = hp.set_config(bsmlz=bsmlz, hss_leaf=leaf, tol=tol, precision=precision)
    try:
        w, Q = hp.eigh_tridiagonal(d, e)
        st = hp.get_stats()
    finally:
        hp.restore_config(old)
    assert st["n_hss_merges"] > 0 and 0 < st["max_rank"] < st["max_k"]
    ev, res, orth = eig_metrics(d, e, w, Q, toeplitz_eigs(n))
    assert ev <= 4e-13 and res <= 1e-12 and orth <= 1e-12, (ev, res, orth)
