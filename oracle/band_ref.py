"""Banded divide and conquer restated in numpy -- TEST INFRASTRUCTURE ONLY.

A dense, small-n restatement of HSSPACK's MDSBEVD (SRC/mdsbevd.f90:183):

* halving tree down to SMLSIZ (mdsbevd.f90:266-277);
* every cut after row c: SVD of the coupling block B = A[c-kd+1 : c+1,
  c+1 : c+kd+1] = U S V^T (mdsbevd.f90:291-297), A_top[-kd:, -kd:] -= U S U^T
  and A_bottom[:kd, :kd] -= V S V^T (DSymSplit, SRC/BasicMM.f90:1195-1311);
* leaves: dense symmetric eigensolve (DSYEVD at mdsbevd.f90:304-313);
* merge: Z = Q^T [w_1 .. w_kd] with w_k = [u_k on the top block's last kd rows;
  v_k on the bottom block's first kd rows] (mdsbed1.f90:174-186), then kd
  rank-one updates D + s_k z_k z_k^T in order, each applied to Q and to the
  remaining columns of Z (mdsbed4.f90:266-273).

Each rank-one update is solved densely (numpy eigh) -- the restatement pins
the splitting, the order of the updates and the transport of Z, which are the
banded-specific parts; deflation and the secular solver are pinned by the
tridiagonal oracle.  Used only by tests.
"""
import numpy as np


def band_to_dense(ab, lower=False):
    """Symmetric dense matrix from LAPACK band storage ab (kd + 1, n)."""
    kd, n = ab.shape[0] - 1, ab.shape[1]
    A = np.zeros((n, n))
    for j in range(n):
        for i in range(max(0, j - kd), j + 1):  # A(i, j), i <= j
            v = ab[j - i, i] if lower else ab[kd + i - j, j]
            A[i, j] = A[j, i] = v
    return A


def leaf_sizes(n, smlsiz):
    sz = [n]
    while max(sz) > smlsiz:
        sz = [x for s in sz for x in (s // 2, (s + 1) // 2)]
    return sz


def band_dc(A, kd, smlsiz=25):
    """Eigenvalues (ascending) and eigenvectors of the dense symmetric band
    matrix A (half-bandwidth kd) by the banded DC above."""
    n = A.shape[0]
    bound = max(smlsiz, 2 * kd)
    sz = leaf_sizes(n, bound)
    ends = np.cumsum(sz)
    A = A.copy()
    cuts = []
    for c in ends[:-1] - 1:  # split every cut (DSymSplit)
        B = A[c - kd + 1:c + 1, c + 1:c + kd + 1].copy()
        U, S, Vt = np.linalg.svd(B)
        V = Vt.T
        A[c - kd + 1:c + 1, c - kd + 1:c + 1] -= (U * S) @ U.T
        A[c + 1:c + kd + 1, c + 1:c + kd + 1] -= (V * S) @ V.T
        A[c - kd + 1:c + 1, c + 1:c + kd + 1] = 0.0
        A[c + 1:c + kd + 1, c - kd + 1:c + 1] = 0.0
        cuts.append((c, U, S, V))
    blocks = []  # (start, eigenvalues, eigenvectors) per current subproblem
    s = 0
    for m in sz:
        w, Q = np.linalg.eigh(A[s:s + m, s:s + m])
        blocks.append((s, w, Q))
        s += m
    ci = 0
    cut_of = {int(c): (U, S, V) for c, U, S, V in cuts}
    while len(blocks) > 1:
        nxt = []
        for i in range(0, len(blocks), 2):
            (s1, w1, Q1), (s2, w2, Q2) = blocks[i], blocks[i + 1]
            n1, n2 = len(w1), len(w2)
            U, S, V = cut_of[s2 - 1]
            Q = np.zeros((n1 + n2, n1 + n2))
            Q[:n1, :n1] = Q1
            Q[n1:, n1:] = Q2
            D = np.concatenate([w1, w2])
            Wm = np.zeros((n1 + n2, kd))
            Wm[n1 - kd:n1] = U
            Wm[n1:n1 + kd] = V
            Z = Q.T @ Wm
            for k in range(kd):
                Dk, Sk = np.linalg.eigh(np.diag(D) + S[k] * np.outer(Z[:, k], Z[:, k]))
                Q = Q @ Sk
                Z = Sk.T @ Z
                D = Dk
            nxt.append((s1, D, Q))
            ci += 1
        blocks = nxt
    _, w, Q = blocks[0]
    return w, Q


def eig_banded_lapack(ab, lower=False):
    """LAPACK (DSBEVD through SciPy) eigenpairs of a band matrix: the accuracy oracle."""
    from scipy.linalg import eig_banded
    return eig_banded(ab, lower=lower)
