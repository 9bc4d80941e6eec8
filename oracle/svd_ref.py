"""Bidiagonal SVD divide and conquer restated in numpy -- TEST INFRASTRUCTURE ONLY.

A dense, small-n restatement of HSSPACK's MDBDSDC / MDLASD0-2 structure
(SRC/mdbdsdc.f90, SRC/mdlasd1.f90, SRC/mdlasd2.f90):

* tree as DLASDT: a node of N rows splits into nl = N // 2 rows, the center
  row c, and nr = N - nl - 1 rows; the left child is nl x (nl + 1) (it carries
  the center's column), the right child inherits the node's extra column;
* leaves: dense SVD of the r x (r + sqre) upper bidiagonal, with the null
  vector of V when sqre = 1;
* merge at c: z = [alpha V1(c, :) for the left triples, beta V2(c + 1, :) for
  the right], z_1 = alpha V1(c, null) combined with beta V2(c + 1, null) by a
  rotation when the node has an extra column (mdlasd2.f90), the broken-arrow
  matrix e_1 z^T + diag(0, d) solved densely, U and V updated.

Pins the tree, the center / null-vector bookkeeping and the z formation; the
deflation and secular solver are checked against LAPACK by the GPU tests.
"""
import numpy as np


def bidiag(d, e, sqre=0):
    r = len(d)
    B = np.zeros((r, r + sqre))
    B[np.arange(r), np.arange(r)] = d
    for i in range(r - 1 + sqre):
        B[i, i + 1] = e[i]
    return B


def _solve(d, e, a, N, sq, smlsiz):
    """SVD of rows a .. a+N-1 (columns a .. a+N-1+sq).  Returns (s asc,
    U (N x N), V ((N+sq) x (N+sq)) with the null vector last when sq)."""
    if N <= smlsiz:
        B = bidiag(d[a:a + N], e[a:a + N - 1 + sq], sq)
        Uf, s, Vt = np.linalg.svd(B)
        o = np.argsort(s, kind="stable")
        V = Vt.T
        Vo = V.copy()
        Vo[:, :N] = V[:, o]
        return s[o], Uf[:, o], Vo
    nl = N // 2
    nr = N - nl - 1
    c = a + nl
    s1, U1, V1 = _solve(d, e, a, nl, 1, smlsiz)
    s2, U2, V2 = _solve(d, e, c + 1, nr, sq, smlsiz)
    alpha, beta = d[c], e[c]
    M = N + sq
    # block matrices in the node's coordinates (rows / columns from a)
    U = np.zeros((N, N))
    U[:nl, :nl] = U1
    U[nl, nl] = 1.0                    # the center row's e_c
    U[nl + 1:, nl + 1:] = U2
    V = np.zeros((M, M))
    V[:nl + 1, :nl] = V1[:, :nl]        # left triples
    V[:nl + 1, nl] = V1[:, nl]          # left null vector -> the center slot
    V[nl + 1:, nl + 1:N] = V2[:, :nr]   # right triples
    if sq:
        V[nl + 1:, N] = V2[:, nr]       # right null vector -> slot N
    z = np.zeros(N)
    z[:nl] = alpha * V1[nl, :nl]
    z[nl + 1:] = beta * V2[0, :nr]
    z1 = alpha * V1[nl, nl]
    if sq:
        zM = beta * V2[0, nr]
        t = np.hypot(z1, zM)
        cg, sg = (z1 / t, zM / t) if t > 0 else (1.0, 0.0)
        vc, vn = V[:, nl].copy(), V[:, N].copy()
        V[:, nl] = cg * vc + sg * vn
        V[:, N] = -sg * vc + cg * vn
        z1 = t
    z[nl] = z1
    dvals = np.concatenate([s1, [0.0], s2])
    # broken arrow in slot order: row "center" carries z, diagonal dvals
    Mx = np.diag(dvals)
    Mx[nl, :] = z
    Mx[nl, nl] = z1
    Us, ss, Vst = np.linalg.svd(Mx)
    o = np.argsort(ss, kind="stable")
    Un = U @ Us[:, o]
    Vn = V.copy()
    Vn[:, :N] = V[:, :N] @ Vst.T[:, o]
    return ss[o], Un, Vn


def bdsdc(d, e, smlsiz=25):
    """Singular values (descending), U, VT of the n x n upper bidiagonal."""
    n = len(d)
    s, U, V = _solve(np.asarray(d, float), np.asarray(e, float), 0, n, 0, smlsiz)
    return s[::-1].copy(), U[:, ::-1].copy(), V[:, ::-1].T.copy()
