"""HSS Cholesky factorisation and solves restated in numpy -- TEST
INFRASTRUCTURE ONLY (never imported by the library).

HSSPACK's HssCholSolver (SRC/HssCholSolver.f90:1-139) factors a dense SPD
matrix with mat2hsscholsvd ('S', SRC/mat2hsssvd.f90:284-550) or
mat2hsscholsvdr ('R', :9-281) and solves with solvecholsvd (:553-671), directly
('N') or as the preconditioner of cg (:674-726, 'Y').  Restated here in the
reference's own order -- nodes of npart's tree (SRC/aux_hss.f90:803-827,
n2tree's post order) one at a time -- on an explicit reduced matrix instead of
the reference's packed stack; the arithmetic per node is the reference's:

* a node whose block has at least 20 rows and at least 20 other current
  variables: D = L L^T (DPOTRF); the scaled block column T L^{-T} (T: the node's
  columns against every other current variable) -- 'S': R of QR(T), right
  singular vectors of R L^{-T}; 'R': of (Omega T) L^{-T} with a uniform [0, 1)
  Omega of prank + pp rows; rk = min(prank, #{sigma > tol});
* when rk < m: Q = [V2 V1] (the non-kept vectors first, circshift2), QL of
  L Q = Qt Lt (DGEQLF), the block column becomes T L^{-T} V1 Lt22^T and the
  diagonal block Lt22 Lt22^T (hssexpsvd, SRC/aux_hss.f90:97-152); else the node
  keeps its variables and its block;
* the root: DPOTRF of what is left.

Solve: forward in post order (Qt^T, Lt11 substitution, Lt21 update, the kept
part to the parent), the root's Cholesky solve, backward in reverse order.
"""
import numpy as np
import scipy.linalg as sla

from oracle import hssmm_ref


def npart_tree(n, ni):
    """Leaf sizes and the post-ordered tree of npart / n2tree (the restatement in
    oracle/hssmm_ref.py): returns (sizes, parent) with nodes 1..ltr (root ltr)."""
    sizes = hssmm_ref.leaf_sizes(n, ni)
    par = hssmm_ref.post_order_tree(len(sizes))[1]
    return sizes, par


def _ql(M):
    """M = Q L with L lower triangular (through QR of the reversed matrix)."""
    J = M[::-1, ::-1]
    q, r = np.linalg.qr(J)
    return q[::-1, ::-1], r[::-1, ::-1]


def factor(A, ni, tol, prank, ps=0, omega=None):
    """Returns the factor: a dict with per-node records and the root's L."""
    n = A.shape[0]
    sizes, par = npart_tree(n, ni)
    ltr = len(par) - 1
    ch = {i: [] for i in range(1, ltr + 1)}
    for i in range(1, ltr):
        ch[par[i]].append(i)
    Ah = np.array(A, dtype=np.float64)
    # active blocks left to right: [node, size]; Ah's rows/cols follow them
    blocks = []
    leaves = [i for i in range(1, ltr + 1) if not ch[i]]
    for i, m in zip(leaves, sizes):
        blocks.append([i, m])
    rec = {}
    max_rank = 0
    for i in range(1, ltr + 1):
        if ch[i]:
            a = [b[0] for b in blocks].index(ch[i][0])
            assert blocks[a + 1][0] == ch[i][1]
            blocks[a] = [i, blocks[a][1] + blocks[a + 1][1]]
            del blocks[a + 1]
        k = [b[0] for b in blocks].index(i)
        o = sum(b[1] for b in blocks[:k])
        m = blocks[k][1]
        Nc = Ah.shape[0]
        if i == ltr:
            return {"rec": rec, "root": np.linalg.cholesky(Ah), "tree": (sizes, par, ch),
                    "max_rank": max_rank}
        idx = np.arange(o, o + m)
        rest = np.concatenate([np.arange(0, o), np.arange(o + m, Nc)])
        nt = len(rest)
        if m < 20 or nt < 20:
            rec[i] = None
            continue
        D = Ah[np.ix_(idx, idx)]
        T = Ah[np.ix_(rest, idx)]
        L = np.linalg.cholesky(D)
        if ps > 0:
            Y = omega[:ps, :nt] @ T
            Y = sla.solve_triangular(L, Y.T, lower=True).T  # Y L^{-T}
            _, s, vt = np.linalg.svd(Y, full_matrices=True)
        else:
            R = np.linalg.qr(T, mode="r")
            S = sla.solve_triangular(L, R.T, lower=True).T  # R L^{-T}
            _, s, vt = np.linalg.svd(S, full_matrices=True)
        V = vt.T
        rk = min(prank, int(np.sum(s[:m] > tol)))
        if rk >= m:
            rec[i] = None
            continue
        max_rank = max(max_rank, rk)
        ir = m - rk
        Q = np.concatenate([V[:, rk:], V[:, :rk]], axis=1)
        Qt, Lt = _ql(L @ Q)
        Lt22 = Lt[ir:, ir:]
        W = sla.solve_triangular(L.T, V[:, :rk], lower=False) @ Lt22.T
        Tn = T @ W
        DD = Lt22 @ Lt22.T
        rec[i] = (Qt, Lt, ir)
        # replace the node's m variables by its rk remaining ones
        new_order = np.concatenate([np.arange(0, o), np.arange(o + m, Nc)])
        B = Ah[np.ix_(new_order, new_order)]
        N2 = Nc - ir
        An = np.zeros((N2, N2))
        keep = np.concatenate([np.arange(0, o), np.arange(o + rk, N2)])
        An[np.ix_(keep, keep)] = B
        mid = np.arange(o, o + rk)
        An[np.ix_(keep, mid)] = Tn
        An[np.ix_(mid, keep)] = Tn.T
        An[np.ix_(mid, mid)] = DD
        Ah = An
        blocks[k][1] = rk
    raise AssertionError("no root")


def solve(F, b):
    """solvecholsvd: the factor's solve of b (n,)."""
    sizes, par, ch = F["tree"]
    rec = F["rec"]
    ltr = len(par) - 1
    leaves = [i for i in range(1, ltr + 1) if not ch[i]]
    seg = {}
    o = 0
    for i, m in zip(leaves, sizes):
        seg[i] = (o, m)
        o += m
    rem, z1 = {}, {}
    for i in range(1, ltr):
        y = b[seg[i][0]:seg[i][0] + seg[i][1]].copy() if not ch[i] else \
            np.concatenate([rem[ch[i][0]], rem[ch[i][1]]])
        r = rec[i]
        if r is None:
            rem[i] = y
            continue
        Qt, Lt, ir = r
        u = Qt.T @ y
        u1 = sla.solve_triangular(Lt[:ir, :ir], u[:ir], lower=True)
        rem[i] = u[ir:] - Lt[ir:, :ir] @ u1
        z1[i] = u1
    root = ltr
    yr = np.concatenate([rem[ch[root][0]], rem[ch[root][1]]]) if ch[root] else b.copy()
    Lr = F["root"]
    xr = sla.solve_triangular(Lr.T, sla.solve_triangular(Lr, yr, lower=True), lower=False)
    sol = {}

    def split(i, x):
        if ch[i]:
            a = len(rem[ch[i][0]])
            sol[ch[i][0]] = x[:a]
            sol[ch[i][1]] = x[a:]

    if not ch[root]:
        return xr
    split(root, xr)
    out = np.zeros_like(b)
    for i in range(ltr - 1, 0, -1):
        x2 = sol[i]
        r = rec[i]
        if r is None:
            x = x2
        else:
            Qt, Lt, ir = r
            u1 = sla.solve_triangular(Lt[:ir, :ir].T, z1[i] - Lt[ir:, :ir].T @ x2, lower=False)
            x = Qt @ np.concatenate([u1, x2])
        if ch[i]:
            split(i, x)
        else:
            o, m = seg[i]
            out[o:o + m] = x
    return out


def cg(A, b, tau, maxit, F=None):
    """cg (SRC/mat2hsssvd.f90:674-726): returns (x, steps, relres)."""
    n = len(b)
    x = np.zeros(n)
    tb = np.linalg.norm(b)
    p = b.copy()
    rs = b.copy()
    if F is not None:
        p = solve(F, p)
    y = p.copy()
    res = np.linalg.norm(rs) / tb
    it = 0
    while res >= tau and it <= maxit:
        it += 1
        z = A @ p
        dt = y @ rs
        nu = dt / (p @ z)
        x += nu * p
        rs -= nu * z
        y = rs.copy()
        if F is not None:
            y = solve(F, y)
        mu = (y @ rs) / dt
        p = y + mu * p
        res = np.linalg.norm(rs) / tb
    return x, it, res


def kernel_matrix(n, length=0.1, nugget=1e-2, seed=0):
    """An SPD test matrix with numerically low-rank off-diagonal blocks: a
    Gaussian kernel on sorted uniform points plus a nugget."""
    rng = np.random.default_rng(seed)
    x = np.sort(rng.uniform(0.0, 1.0, n))
    d = x[:, None] - x[None, :]
    return np.exp(-0.5 * (d / length) ** 2) + nugget * np.eye(n)
