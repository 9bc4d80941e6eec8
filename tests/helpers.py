"""Shared problem generators and error metrics for the tests (seeded, numpy)."""
import numpy as np


def rand_tridiag(n, seed=0, lo=-1.0, hi=1.0):
    rng = np.random.default_rng(seed)
    return rng.uniform(lo, hi, n), rng.uniform(lo, hi, max(n - 1, 0))


def toeplitz_tridiag(n):
    """D = 2, E = 1: the closed-form case of TEST/Testedc.f90:34-37."""
    return np.full(n, 2.0), np.ones(max(n - 1, 0))


def toeplitz_eigs(n):
    k = np.arange(1, n + 1)
    return np.sort(2.0 + 2.0 * np.cos(k * np.pi / (n + 1)))


def tmatvec(d, e, Q):
    """T @ Q for the symmetric tridiagonal (d, e) without forming T."""
    R = d[:, None] * Q
    if len(e):
        R[:-1] += e[:, None] * Q[1:]
        R[1:] += e[:, None] * Q[:-1]
    return R


def tnorm(d, e):
    """An upper bound of ||T||_2 (max row sum)."""
    a = np.abs(d).copy()
    if len(e):
        a[:-1] += np.abs(e)
        a[1:] += np.abs(e)
    return a.max()


def eig_metrics(d, e, w, Q, w_ref):
    """max|w - w_ref|/||T||, ||TQ - QW||_F/(n||T||), ||Q^T Q - I||_F/n."""
    n = len(d)
    nt = max(tnorm(d, e), 1e-300)
    ev = float(np.max(np.abs(np.sort(w) - np.sort(w_ref)))) / nt
    res = float(np.linalg.norm(tmatvec(d, e, Q) - Q * w[None, :])) / (n * nt)
    orth = float(np.linalg.norm(Q.T @ Q - np.eye(n))) / n
    return ev, res, orth


def secular_problem(k, seed=0, normalize=True):
    """Poles sorted U[0,1], weights N(0,1)/sqrt(k), rho = 1 (the Cauchy-merge
    configuration); optionally |z| = 1 as after MDLAED2's scaling."""
    rng = np.random.default_rng(seed)
    d = np.sort(rng.uniform(0.0, 1.0, k))
    # keep poles distinct and z away from deflation, as after MDLAED2
    d = d + np.arange(k) * 1e-12
    z = rng.standard_normal(k) / np.sqrt(k)
    if normalize:
        z /= np.linalg.norm(z)
    return d, z, 1.0


def interlace_grid(n, lo=0.1, hi=9.0):
    """F_i = lo + (2i-1) g, D_i = F_i + g, g = (hi - lo)/(2n)
    (TEST/testCauchyHss_serial.f90:46-52, TEST/testfmm.f90:20-32)."""
    g = (hi - lo) / (2 * n)
    i = np.arange(1, n + 1)
    F = lo + (2 * i - 1) * g
    return F, F + g
