"""SVD updating restated in numpy -- TEST INFRASTRUCTURE ONLY (never imported by
the library).

HSSPACK's SvdHssUpdat (SRC/SvdHssUpdat.f90:1-178) computes the singular values
and right singular vectors of [A; a^T] from A = U diag(f) V^T and z = V^T a:

* MDLASD20 (SRC/mdlasd20.f90:122-300): deflation of M = [diag(f); z^T] -- small
  z_j (|z_j| <= tol, tol = 8 eps max(|f_1|, |f_n|)) and close poles
  (|f_j - f_jprev| <= tol: a Givens rotation on rows jprev, j of V^T zeroes
  z_jprev); non-deflated entries first, deflated ones after them in reverse
  order of discovery; V^T's rows permuted the same way.
* MDLASD31 (SRC/mdlasd31.f90:1-201): the K roots sigma_j of
  1 + rho sum z_i^2 / (f_i^2 - sigma^2) (z normalised, rho = |z|^2) by LAPACK's
  DLASD4 (SciPy's wrapper, 0-based root index), DIFL_j = sigma_j - f_j,
  DIFR_j = sigma_j - f_{j+1}, z recomputed by Loewner's formula
  zhat_i^2 = |prod_j (f_i^2 - sigma_j^2) / prod_{j != i} (f_i^2 - f_j^2)|, and
  alpha_j = 1 / |(zhat_i / (f_i^2 - sigma_j^2))_i|.
* The right singular vectors: rows i < K of the new V^T are
  sum_j A(i,j) V2^T(j, :) with A(i,j) = alpha_i zhat_j / (sigma_i^2 - f_j^2)
  (the matrix Cauchy2hssvd compresses, SRC/CauchyHssvd_VPS.f90:2781-2785,
  applied by fastHssmm); here the product is dense, i.e. the HSS
  approximation's exact target.

The two readings of undefined behaviour that the library also makes: MDLASD20's
never-set locals ALPHA and BETA count as 0 in the tolerance, and SvdHssUpdat's
uninitialised HFLAG is .FALSE. (all rows of V^T permuted).  MDLASD31's K = 1
shortcut (sigma = |z|, written for a zero pole) is replaced by the root of the
one-term equation, sigma^2 = f^2 + z^2.
"""
import numpy as np
import scipy.linalg.lapack as lapack

EPS = 2.0 ** -53


def deflate(f, z):
    """MDLASD20 on copies: returns (K, f, z, idxp, rots), rots = [(p, q, c, s)]."""
    f = np.array(f, dtype=np.float64)
    z = np.array(z, dtype=np.float64)
    n = len(f)
    tol = 8.0 * EPS * max(abs(f[-1]), abs(f[0]))
    idxp = np.zeros(n, dtype=np.int64)
    ww = np.zeros(n)
    rots = []
    K, K2, jprev = 0, n, -1
    for j in range(n):
        if abs(z[j]) <= tol:
            K2 -= 1
            idxp[K2] = j
        else:
            jprev = j
            break
    if jprev >= 0:
        for j in range(jprev + 1, n):
            if abs(z[j]) <= tol:
                K2 -= 1
                idxp[K2] = j
            elif abs(f[j] - f[jprev]) <= tol:
                tau = np.hypot(z[j], z[jprev])
                c, s = z[j] / tau, -z[jprev] / tau
                z[j], z[jprev] = tau, 0.0
                rots.append((jprev, j, c, s))
                K2 -= 1
                idxp[K2] = jprev
                jprev = j
            else:
                ww[K] = z[jprev]
                idxp[K] = jprev
                K += 1
                jprev = j
        ww[K] = z[jprev]
        idxp[K] = jprev
        K += 1
    z[:K] = ww[:K]
    f = f[idxp].copy()
    if abs(z[0]) <= tol:
        z[0] = tol
    return K, f, z, idxp, rots


def secular(K, dsig, z):
    """MDLASD31: (sigma, difl, difr, zhat, alpha) for poles dsig[:K], weights z[:K]."""
    d = np.array(dsig[:K], dtype=np.float64)
    zz = np.array(z[:K], dtype=np.float64)
    if K == 1:
        s = np.sqrt(d[0] * d[0] + zz[0] * zz[0])
        dl = np.array([s - d[0]])
        zh = zz.copy()
        al = np.array([abs(d[0] * d[0] - s * s) / abs(zh[0])])
        return np.array([s]), dl, np.zeros(1), zh, al
    rho = np.linalg.norm(zz)
    zn = zz / rho
    rho2 = rho * rho
    sig = np.zeros(K)
    difl = np.zeros(K)
    difr = np.zeros(K)
    w3 = np.ones(K)
    for j in range(K):
        delta, sigma, work, info = lapack.dlasd4(j, d, zn, rho=rho2)
        assert info == 0, info
        sig[j] = sigma
        # delta_i = d_i - sigma_j, work_i = d_i + sigma_j
        w3 *= delta * work
        others = np.arange(K) != j
        w3[others] /= (d[others] - d[j]) * (d[others] + d[j])
        difl[j] = -delta[j]
        if j + 1 < K:
            difr[j] = -delta[j + 1]
    zh = np.copysign(np.sqrt(np.abs(w3)), zn) * 1.0
    S = sigma_minus_pole(d, difl, difr)
    alpha = np.zeros(K)
    for j in range(K):
        col = zh / (S[:, j] * (d + sig[j]))
        alpha[j] = 1.0 / np.linalg.norm(col)
    return sig, difl, difr, zh, alpha


def sigma_minus_pole(d, difl, difr):
    """S[i, j] = sigma_j - d_i from the differences DLASD4 returns
    (sigma_j = d_j + DIFL_j = d_{j+1} + DIFR_j), as MDLASD31 forms them
    (SRC/mdlasd31.f90:181-192): no cancellation when a root hugs a pole."""
    K = len(d)
    S = np.empty((K, K))
    for j in range(K):
        S[:j + 1, j] = (d[j] - d[:j + 1]) + difl[j]
        if j + 1 < K:
            S[j + 1:, j] = (d[j + 1] - d[j + 1:]) + difr[j]
    return S


def svdhssupdat(f, z, VT):
    """The whole update with a dense product.  VT: (n, n), rows = right singular
    vectors.  Returns (K, sigma (K), f_out, z_out, VT_new)."""
    n = len(f)
    K, fo, zo, idxp, rots = deflate(f, z)
    W = np.array(VT, dtype=np.float64)
    for p, q, c, s in rots:  # DROT on rows p, q
        x, y = W[p].copy(), W[q].copy()
        W[p] = c * x + s * y
        W[q] = c * y - s * x
    W2 = W[idxp]
    if K == 0:
        return 0, np.zeros(0), fo, zo, W2
    sig, difl, difr, zh, alpha = secular(K, fo, zo)
    d = fo[:K]
    S = sigma_minus_pole(d, difl, difr)  # S[j, i] = sigma_i - d_j
    A = alpha[:, None] * zh[None, :] / (S.T * (sig[:, None] + d[None, :]))
    out = W2.copy()
    out[:K] = A @ W2[:K]
    zo = zo.copy()
    zo[:K] = zh
    return K, sig, fo, zo, out
