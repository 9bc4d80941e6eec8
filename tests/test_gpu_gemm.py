"""Grouped GEMM: FP64 CUDA-core path and the split-BF16 tensor-core path
(7 digit planes, exact integer accumulation) against numpy FP64 products and,
on a small case, against the exact rational product.  Tolerances for the
split path: |C - AB| <= 2^-44 (|A| |B|)_ij against numpy (whose own rounding
dominates at large k), <= 2^-50 (|A| |B|)_ij against the exact product (the
digits keep 56 bits relative to each row's / column's largest entry)."""
from fractions import Fraction

import numpy as np
import pytest
import torch

import hsspack_gb300 as hp

pytestmark = pytest.mark.gpu


def _colmajor(a):
    """device buffer holding a in column-major order"""
    return torch.tensor(np.asfortranarray(a).T.copy(), dtype=torch.float64, device="cuda")


def _run(A, B, C0=None, beta=0, precision=1):
    m, k = A.shape
    n = B.shape[1]
    dA, dB = _colmajor(A), _colmajor(B)
    dC = _colmajor(C0 if C0 is not None else np.zeros((m, n)))
    hp.gemm_dev(dA, dB, dC, m, n, k, m, k, m, beta=beta, precision=precision)
    return dC.cpu().numpy().T


@pytest.mark.parametrize("m,n,k", [(128, 64, 64), (300, 70, 150), (1000, 115, 60), (257, 33, 257),
                                   (64, 200, 700), (5, 3, 1), (2000, 40, 37), (700, 129, 300)])
@pytest.mark.parametrize("precision,path", [(0, 0), (1, 0), (1, 1)])  # path 1: fused split
def test_gemm_vs_numpy(m, n, k, precision, path):
    rng = np.random.default_rng(m * 7 + n * 3 + k)
    A = rng.standard_normal((m, k))
    B = rng.standard_normal((k, n))
    # thresholds at their minimum: every precision-1 product takes the split path
    old = hp.set_config(gemm_path=path, split_min_m=1, split_min_log2=1)
    try:
        C = _run(A, B, precision=precision)
    finally:
        hp.restore_config(old)
    ref = A @ B
    bound = np.abs(A) @ np.abs(B)
    tol = 2.0 ** -44 if precision == 1 else 1e-15 * k
    assert np.max(np.abs(C - ref) / bound) <= tol, np.max(np.abs(C - ref) / bound)


@pytest.mark.parametrize("path", [0, 1])
def test_split_row_col_scales_and_beta(path):
    rng = np.random.default_rng(5)
    m, n, k = 384, 128, 200
    A = rng.standard_normal((m, k)) * (2.0 ** rng.integers(-40, 40, size=(m, 1)))
    B = rng.standard_normal((k, n)) * (2.0 ** rng.integers(-40, 40, size=(1, n)))
    A[3, :] = 0.0  # an all-zero row
    C0 = rng.standard_normal((m, n))
    old = hp.set_config(gemm_path=path)
    try:
        C = _run(A, B, C0=C0, beta=1, precision=1)
    finally:
        hp.restore_config(old)
    ref = C0 + A @ B
    # FP64 rounding of C0 + AB itself is 2^-53 |C0|: allow 2^-52 |C0| on top
    bound = np.abs(A) @ np.abs(B) + np.abs(C0) * 2.0 ** -8
    assert np.max(np.abs(C - ref) / bound) <= 2.0 ** -44


@pytest.mark.parametrize("path", [0, 1])
def test_split_orthogonal_update_accuracy(path):
    # the use in the eigensolver: Q (orthogonal) times an orthogonal S
    rng = np.random.default_rng(9)
    Q, _ = np.linalg.qr(rng.standard_normal((512, 512)))
    S, _ = np.linalg.qr(rng.standard_normal((512, 512)))
    old = hp.set_config(gemm_path=path)
    try:
        C = _run(Q, S, precision=1)
    finally:
        hp.restore_config(old)
    assert np.linalg.norm(C.T @ C - np.eye(512)) / 512 <= 1e-14


@pytest.mark.parametrize("path", [0, 1])
def test_split_gemm_against_exact_product(path):
    rng = np.random.default_rng(17)
    m, n, k = 24, 12, 300  # three K windows of 128
    A = rng.standard_normal((m, k)) * np.exp(rng.uniform(-3, 3, (m, 1)))
    B = rng.standard_normal((k, n))
    old = hp.set_config(gemm_path=path, split_min_m=1, split_min_log2=1)
    try:
        C = _run(A, B, precision=1)
    finally:
        hp.restore_config(old)
    Af = [[Fraction(float(x)) for x in row] for row in A]
    Bf = [[Fraction(float(B[p, j])) for p in range(k)] for j in range(n)]
    bound = np.abs(A) @ np.abs(B)
    worst = 0.0
    for i in range(m):
        for j in range(n):
            exact = sum(a * b for a, b in zip(Af[i], Bf[j]))
            worst = max(worst, abs(float(Fraction(float(C[i, j])) - exact)) / bound[i, j])
    assert worst <= 2.0 ** -50, worst
