"""Cauchy-like HSS products on the GPU: CauchyHssMM (generic Cauchy matrix,
SRC/cauchyhssmm.f90) against the dense product, and the n = 8192 Cauchy merge
(secular roots, Loewner z, HSS compression of the eigenvector matrix, product
with a dense orthogonal Q) against the dense eigenvector matrix.

Tolerances: the HSS products within 1e-11 (relative Frobenius) of the dense
products at HSS tolerance 1e-14; orthogonality of Q C within 1e-12 * n."""
import numpy as np
import pytest
import torch

import hsspack_gb300 as hp
from helpers import interlace_grid

pytestmark = pytest.mark.gpu


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


@pytest.mark.parametrize("precision", [0, 1])
def test_cauchy_merge_8192(precision):
    # the Cauchy merge workload: d sorted U[0,1], z ~ N(0,1)/sqrt(n), rho = 1;
    # C_ij = zhat_i alpha_j / (d_i - lambda_j), HSS leaf 128, tol 1e-14, times a
    # dense random orthogonal Q (8192 x 8192)
    n = 8192
    rng = np.random.default_rng(0)
    d = np.sort(rng.uniform(0.0, 1.0, n))
    z = rng.standard_normal(n) / np.sqrt(n)
    dd, zz = _dev(d), _dev(z)
    lam, difl, difr = (torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(3))
    hp.secular_dev(dd, zz, 1.0, lam, difl, difr)
    zh, al = zz.clone(), torch.zeros(n, dtype=torch.float64, device="cuda")
    hp.lowner_dev(dd, difl, difr, zh, al)
    gen = torch.Generator(device="cuda").manual_seed(1)
    Qf, _ = torch.linalg.qr(torch.randn(n, n, dtype=torch.float64, device="cuda", generator=gen))
    Q = Qf.T.contiguous()  # memory = column-major Qf
    C = torch.zeros(n * n, dtype=torch.float64, device="cuda")
    hp.cauchy_eig_dev(dd, zh, al, difl, difr, C)
    Cm = C.view(n, n).T  # C[i, j]
    ref = Qf @ Cm
    old = hp.set_config(precision=precision)
    try:
        hp.dhssevc_dev(dd, zh, al, difl, difr, Q, n, n, ni=128, tol=1e-14)
    finally:
        hp.restore_config(old)
    out = Q.T  # Q C
    err = float(torch.linalg.norm(out - ref) / torch.linalg.norm(ref))
    assert err <= 1e-11, err
    g = torch.randn(n, 8, dtype=torch.float64, device="cuda", generator=gen)
    y = out.T @ (out @ g) - g
    assert float(torch.sqrt(torch.sum(y * y) / 8)) / n <= 1e-12
