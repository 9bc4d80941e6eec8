"""Generate the golden fixtures in this directory (run from the repo root:
``python tests/golden/make_golden.py``).

* secular_mp.npz -- secular problems with roots computed to 50 digits by
  bisection in mpmath (independent of LAPACK); the parity tests pin both the
  oracle (LAPACK DLAED4) and the GPU solver against them.
* dc_small.npz -- eigenvalues (and for n = 64 the eigenvectors) of seeded
  tridiagonals from the oracle's restated MDSTEDC, cross-checked here against
  LAPACK DSTEDC before they are written.
* hss_grid.npz -- the interlacing Cauchy grid of TEST/testCauchyHss_serial.f90
  (F_i = 0.1 + (2i-1)g, D_i = F_i + g) with random generators and a dense
  product C @ B computed in numpy, for the standalone Cauchy/HSS APIs.
* secular_edge_mp.npz -- nearly deflatable secular problems (a pole with a tiny
  weight placed on a root of the other poles' equation, as glued matrices
  produce) with roots to 50 digits.
* merge8192_mp.npz -- eight roots (the last included) of the n = 8192
  Cauchy-merge problem to 50 digits.

``python tests/golden/make_golden.py [secular dc hss edge merge8192]`` writes the named
fixtures only (default: all).

The reference ships no golden vectors of its own (its test drivers only print
errors against LAPACK), so these are the pins.
"""
import os
import sys

import mpmath as mp
import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

import oracle  # noqa: E402
from helpers import (eig_metrics, interlace_grid, rand_tridiag, secular_problem,  # noqa: E402
                     toeplitz_tridiag)


def mp_roots(d, z, rho, dps=50):
    mp.mp.dps = dps
    dm = [mp.mpf(float(x)) for x in d]
    z2 = [mp.mpf(float(x)) ** 2 for x in z]
    r = mp.mpf(float(rho))
    K = len(d)

    def f(x):
        return 1 / r + mp.fsum(zz / (di - x) for di, zz in zip(dm, z2))

    lam, difl, difr = [], [], []
    for j in range(K):
        lo = dm[j]
        hi = dm[j + 1] if j + 1 < K else dm[j] + r * mp.fsum(z2)
        for _ in range(190):
            mid = (lo + hi) / 2
            if f(mid) < 0:
                lo = mid
            else:
                hi = mid
        x = (lo + hi) / 2
        lam.append(float(x))
        difl.append(float(x - dm[j]))
        difr.append(float(x - dm[j + 1]) if j + 1 < K else 0.0)
    return np.array(lam), np.array(difl), np.array(difr)


def edge():
    """Pole of weight wz inserted at root `which` of a 40-pole problem
    (seed 11), z renormalised; roots of the new problem to 50 digits."""
    out = {}
    d0, z0, rho = secular_problem(40, 11)
    lam0, _, _ = oracle.secular(d0, z0, rho)
    for name, which in (("last", 39), ("middle", 20), ("first", 0)):
        for wname, wz in (("w7", 1e-7), ("w14", 3e-14)):
            p = lam0[which]
            d = np.sort(np.append(d0, p))
            z = np.insert(z0, int(np.searchsorted(d, p)), wz)
            z = z / np.linalg.norm(z)
            lam, difl, difr = mp_roots(d, z, rho)
            key = "%s_%s" % (name, wname)
            out[key + "_d"], out[key + "_z"], out[key + "_rho"] = d, z, np.array(rho)
            out[key + "_lam"], out[key + "_difl"], out[key + "_difr"] = lam, difl, difr
    np.savez_compressed(os.path.join(HERE, "secular_edge_mp.npz"), **out)


def merge8192():
    """The n = 8192 Cauchy-merge problem (d sorted U[0,1], z ~ N(0,1)/sqrt(n),
    rho = 1, seed 0): roots 0, 1, 4095, 8190, 8191 and three seeded others to
    50 digits (bisection on the full 8192-term equation).  DLAED4's last root is
    1.5e-13 off on this problem, so its parity test pins that root here."""
    n = 8192
    rng = np.random.default_rng(0)
    d = np.sort(rng.uniform(0.0, 1.0, n))
    z = rng.standard_normal(n) / np.sqrt(n)
    idx = np.array(sorted({0, 1, 4095, 8190, 8191} |
                          set(np.random.default_rng(5).choice(n, 3, replace=False).tolist())))
    mp.mp.dps = 50
    dm = [mp.mpf(float(x)) for x in d]
    z2 = [mp.mpf(float(x)) ** 2 for x in z]

    def f(x):
        return 1 + mp.fsum(zz / (di - x) for di, zz in zip(dm, z2))

    lam, difl, difr = [], [], []
    for j in idx:
        lo = dm[j]
        hi = dm[j + 1] if j + 1 < n else dm[j] + mp.fsum(z2)
        for _ in range(120):
            mid = (lo + hi) / 2
            if f(mid) < 0:
                lo = mid
            else:
                hi = mid
        x = (lo + hi) / 2
        lam.append(float(x))
        difl.append(float(x - dm[j]))
        difr.append(float(x - dm[j + 1]) if j + 1 < n else 0.0)
    np.savez_compressed(os.path.join(HERE, "merge8192_mp.npz"), idx=idx, lam=np.array(lam),
                        difl=np.array(difl), difr=np.array(difr))


def secular_fixture():
    out = {}
    for k, seed in [(3, 11), (40, 12), (200, 13)]:
        d, z, rho = secular_problem(k, seed)
        lam, difl, difr = mp_roots(d, z, rho)
        out["k%d_d" % k], out["k%d_z" % k], out["k%d_rho" % k] = d, z, np.array(rho)
        out["k%d_lam" % k], out["k%d_difl" % k], out["k%d_difr" % k] = lam, difl, difr
    np.savez_compressed(os.path.join(HERE, "secular_mp.npz"), **out)


def dc_fixture():
    dc = {}
    cases = [("rand64", rand_tridiag(64, seed=64)), ("rand200", rand_tridiag(200, seed=200)),
             ("rand512", rand_tridiag(512, seed=512)), ("toep100", toeplitz_tridiag(100))]
    for name, (d, e) in cases:
        w, Q = oracle.eigh_tridiagonal(d, e, hss_leaf=64, bsmlz=40, tol=1e-14)
        wl, _ = oracle.dstedc_lapack(d, e)
        ev, res, orth = eig_metrics(d, e, w, Q, wl)
        assert ev <= 1e-13 and res <= 1e-12 and orth <= 1e-12, (name, ev, res, orth)
        dc[name + "_d"], dc[name + "_e"], dc[name + "_w"] = d, e, w
        if len(d) == 64:
            dc[name + "_Q"] = Q
    np.savez_compressed(os.path.join(HERE, "dc_small.npz"), **dc)


def hss_fixture():
    n = 300
    F, D = interlace_grid(n)
    rng = np.random.default_rng(300)
    u, v = rng.uniform(0, 1, n), rng.uniform(0, 1, n)
    B = rng.uniform(0, 1, (n, 8))
    C = u[:, None] * v[None, :] / (D[:, None] - F[None, :])
    np.savez_compressed(os.path.join(HERE, "hss_grid.npz"), F=F, D=D, u=u, v=v, B=B, CB=C @ B)


def main(which):
    makers = {"secular": secular_fixture, "dc": dc_fixture, "hss": hss_fixture, "edge": edge,
              "merge8192": merge8192}
    for name in which:
        makers[name]()
    print("fixtures written to", HERE, ":", ", ".join(which))


if __name__ == "__main__":
    main(tuple(sys.argv[1:]) or ("secular", "dc", "hss", "edge", "merge8192"))
