"""Structured banded divide and conquer SVD restated in numpy -- TEST
INFRASTRUCTURE ONLY (never imported by the library).

HSSPACK's MDBDSVD (SRC/mdbdsvd.f90:1-338) computes the SVD of an n x n upper
banded matrix B with sb superdiagonals (upper band storage AB(sb+1+i-j, j) =
B(i, j), 1-based, as DSB2FLC in SRC/SFtransf.f:140-290):

* MDBDSVDT (SRC/mdbdsvdt.f90): msub = max(smlsiz, 3 sb), levels =
  int(log2(n / (msub + 1))); a node of X rows keeps X // 2 rows on the left,
  sb center rows, X - X // 2 - sb on the right.  n <= smlsiz: one dense SVD.
* Leaves: DGESVD of the nl x (nl + sb) left blocks and the nr x (nr + sqre)
  right blocks (mdbdsvd.f90:158-254), sqre = sb except at the matrix's end.
* MDBDSVD1 (SRC/mdbdsvd1.f90) per merge: the sb center rows in the children's
  right singular bases, ordered [left null vectors | left sigma | right sigma |
  right null vectors] (mdbdsvd2.f90:262-274); their QR factorization, Q going
  into U's center rows (DGEQRF/DORGQR, :277-284, :540-544); when the right
  child has extra columns, the RZ factorization of [front | back] columns
  zeroing the back part (DTZRZF/DORMRZ, :546-589).  Then row sb of R, whose
  only null entry is column sb: the bidiagonal-type merge with the pole d = 0
  (MDBDSVD2 + MDBDSVD3); rows sb-1 .. 1 likewise, each an SVD update of the
  growing problem (MDBDSVD22 + MDBDSVD4, mdbdsvd1.f90:295-349).
* Each arrow [[zeta, z^T], [0, diag(d)]]: deflation of small z and of close d by
  Givens rotations (tolerance 8 eps max(d_max, |z|_max), mdbdsvd2.f90:329-331),
  the roots by LAPACK's DLASD4 (SciPy's wrapper), z rebuilt by Loewner's
  formula, V columns z_i / (d_i^2 - sigma^2) and U columns (-1, d_i z_i /
  (d_i^2 - sigma^2)), each normalised (DLASD3's vectors).
* The reference scales each merge by max(|ALPHA|, |BETA|, |D|) once
  (mdbdsvd1.f90:195-209); here each update is scaled by its own maximum.

The reading of an undefined case: when log2(n / (msub + 1)) < 1 with
n > smlsiz the reference builds one node and never merges it; here the
depth is at least 1.
"""
import numpy as np
import scipy.linalg as sla

from oracle import svdupd_ref

EPS = 2.0 ** -53


def band_to_dense(ab, sb):
    """Upper band storage (sb + 1, n) -> dense n x n."""
    n = ab.shape[1]
    B = np.zeros((n, n))
    for j in range(n):
        for i in range(max(0, j - sb), j + 1):
            B[i, j] = ab[sb + i - j, j]
    return B


def tree(n, sb, smlsiz):
    """MDBDSVDT: returns (levels, leaves).  levels[d] lists the nodes of depth d
    (root first) as (s, X, sq): rows [s, s + X), sq extra columns; leaves as
    (s, rows, cols)."""
    msub = max(smlsiz, 3 * sb)
    lvl = max(1, int(np.log2(max(1, n) / (msub + 1))))
    levels = [[(0, n, 0)]]
    for _ in range(lvl - 1):
        nxt = []
        for s, X, sq in levels[-1]:
            nl = X // 2
            nxt.append((s, nl, sb))
            nxt.append((s + nl + sb, X - nl - sb, sq))
        levels.append(nxt)
    leaves = []
    for s, X, sq in levels[-1]:
        nl = X // 2
        nr = X - nl - sb
        assert nl >= 1 and nr >= 1, "empty side"
        leaves.append((s, nl, nl + sb))
        leaves.append((s + nl + sb, nr, nr + sq))
    return levels, leaves


def _arrow(zeta, z, s):
    """SVD of M = [[zeta, z^T], [0, diag(s)]] ((r+1) x (r+1)), s >= 0 unsorted.
    Returns (sigma (r+1), Um, Vm) with M = Um diag(sigma) Vm^T; position 0 of
    rows / columns is the pole."""
    r = len(s)
    order = np.argsort(s, kind="stable")
    d = np.concatenate([[0.0], s[order]])
    zz = np.concatenate([[zeta], z[order]])
    idx = np.concatenate([[0], order + 1])  # position -> row / column of M
    nrm = max(np.max(np.abs(d)), np.max(np.abs(zz)))
    nrm = nrm if nrm > 0 else 1.0
    d = d / nrm
    zz = zz / nrm
    tol = 8.0 * EPS * max(d[-1], np.max(np.abs(zz)))
    # Givens rotations among positions (both sides, as on U and V columns)
    Gu = np.eye(r + 1)
    Gv = np.eye(r + 1)
    keep, defl = [0], []
    jprev = None
    for j in range(1, r + 1):
        if abs(zz[j]) <= tol:
            defl.append(j)
            continue
        if jprev is not None and abs(d[j] - d[jprev]) <= tol:
            tau = np.hypot(zz[j], zz[jprev])
            c, sn = zz[j] / tau, -zz[jprev] / tau
            for G in (Gu, Gv):
                x, y = G[:, jprev].copy(), G[:, j].copy()
                G[:, jprev] = c * x + sn * y
                G[:, j] = c * y - sn * x
            zz[j], zz[jprev] = tau, 0.0
            keep.remove(jprev)
            defl.append(jprev)
        keep.append(j)
        jprev = j
    if abs(zz[0]) <= tol:
        zz[0] = tol
    K = len(keep)
    dk = d[keep].copy()
    if K >= 2 and abs(dk[1]) <= 0.5 * tol:
        dk[1] = 0.5 * tol
    sig, difl, difr, zh, _ = svdupd_ref.secular(K, dk, zz[keep])
    S = svdupd_ref.sigma_minus_pole(dk, difl, difr)  # S[i, j] = sigma_j - d_i
    den = S * (dk[:, None] + sig[None, :])          # sigma_j^2 - d_i^2
    Vk = -zh[:, None] / den
    Uk = -(dk * zh)[:, None] / den
    Uk[0, :] = -1.0
    Vk /= np.linalg.norm(Vk, axis=0)
    Uk /= np.linalg.norm(Uk, axis=0)
    sigma = np.concatenate([sig, d[defl]]) * nrm
    Um = np.zeros((r + 1, r + 1))
    Vm = np.zeros((r + 1, r + 1))
    Um[np.ix_(keep, range(K))] = Uk
    Vm[np.ix_(keep, range(K))] = Vk
    for t, j in enumerate(defl):
        Um[j, K + t] = 1.0
        Vm[j, K + t] = 1.0
    Um = Gu @ Um
    Vm = Gv @ Vm
    P = np.empty(r + 1, dtype=np.int64)
    P[idx] = np.arange(r + 1)
    return sigma, Um[P], Vm[P]


def _merge(B, s0, X, sq, sb, left, right):
    """MDBDSVD1 for the node rows [s0, s0 + X); left / right = (sigma, U, V) of
    the children (V: columns = right singular vectors, nulls last)."""
    nl = X // 2
    nr = X - nl - sb
    N, M = X, X + sq
    s1, U1, V1 = left
    s2, U2, V2 = right
    # right basis, ordered [left nulls | left sigma | right sigma | right nulls]
    Vb = np.zeros((M, M))
    Vb[:nl + sb, :sb] = V1[:, nl:]
    Vb[:nl + sb, sb:sb + nl] = V1[:, :nl]
    Vb[nl + sb:, sb + nl:sb + nl + nr] = V2[:, :nr]
    Vb[nl + sb:, sb + nl + nr:] = V2[:, nr:]
    # left basis: [center rows | left vectors | right vectors]
    Ub = np.zeros((N, N))
    Ub[nl:nl + sb, :sb] = np.eye(sb)
    Ub[:nl, sb:sb + nl] = U1
    Ub[nl + sb:, sb + nl:] = U2
    W = B[s0 + nl:s0 + nl + sb, s0:s0 + M] @ Vb
    Q, R = np.linalg.qr(W)  # W = Q R, R upper trapezoidal (sb x M)
    Ub[:, :sb] = Ub[:, :sb] @ Q
    if sq > 0:  # RZ: zero the back columns row by row from the bottom
        back = np.arange(M - sq, M)
        for i in range(sb - 1, -1, -1):
            cols = np.concatenate([[i], back])
            x = R[i, cols]
            xn = np.linalg.norm(x)
            if xn == 0.0 or np.linalg.norm(x[1:]) == 0.0:
                continue
            v = x.copy()
            v[0] += np.copysign(xn, x[0])
            beta = 2.0 / (v @ v)
            R[:, cols] -= beta * np.outer(R[:, cols] @ v, v)
            Vb[:, cols] -= beta * np.outer(Vb[:, cols] @ v, v)
    # current triplets in the middle coordinates (rows / columns of [R; diag])
    sig = np.concatenate([s1, s2])
    Uc = np.zeros((N, nl + nr))
    Uc[sb:, :] = np.eye(nl + nr)
    Vc = np.zeros((M, nl + nr))
    Vc[sb:sb + nl + nr, :] = np.eye(nl + nr)
    for i in range(sb - 1, -1, -1):
        g = R[i]
        z = Vc.T @ g
        zeta = g[i]
        sigma, Um, Vm = _arrow(zeta, z, sig)
        eu = np.zeros((N, 1))
        eu[i] = 1.0
        ev = np.zeros((M, 1))
        ev[i] = 1.0
        Uc = np.hstack([eu, Uc]) @ Um
        Vc = np.hstack([ev, Vc]) @ Vm
        sig = sigma
    U = Ub @ Uc
    V = Vb @ np.hstack([Vc, np.eye(M)[:, M - sq:]]) if sq > 0 else Vb @ Vc
    return sig, U, V


def mdbdsvd(ab, sb, smlsiz=25):
    """The whole MDBDSVD: returns (s descending, U, VT)."""
    n = ab.shape[1]
    B = band_to_dense(ab, sb)
    if n <= smlsiz:
        U, s, VT = np.linalg.svd(B)
        return s, U, VT
    levels, leaves = tree(n, sb, smlsiz)
    res = {}
    for s0, r, c in leaves:
        Ul, sl, VTl = np.linalg.svd(B[s0:s0 + r, s0:s0 + c], full_matrices=True)
        res[s0] = (sl, Ul, VTl.T)
    for lv in reversed(levels):
        for s0, X, sq in lv:
            nl = X // 2
            left = res.pop(s0)
            right = res.pop(s0 + nl + sb)
            res[s0] = _merge(B, s0, X, sq, sb, left, right)
    sig, U, V = res[0]
    order = np.argsort(-sig, kind="stable")
    return sig[order], U[:, order], V[:, order].T
