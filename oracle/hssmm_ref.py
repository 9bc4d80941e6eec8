"""Test infrastructure only (the oracle; never imported by the library): a numpy
restatement of HSSPACK's dense -> HSS construction by truncated SVD and of the
two HSS products behind DHSSMM and DHSSMML.

  npart, n2tree  SRC/aux_hss.f90:803-827, :737-778   leaf sizes, post-order tree
  mat2hssvd      SRC/ConstructHssd.f90:371-693        construction
  fastHssmm      SRC/ConstructHssd.f90:926-1155       Y = A X    (DHSSMM.f90:103-116)
  fastHssmmL     SRC/ConstructHssd.f90:699-923        Y = X A    (DHSSMML.f90:104-113)

mat2hssvd visits the nodes in post order with a stack of partially compressed
block rows and columns.  This restatement keeps the visiting order and the
rank rule with an explicit reduced matrix instead of the stack: when node i is
visited, its block column (every current row outside i) is replaced by its
product with the right singular vectors whose singular values exceed tol, then
its block row (every current column outside i) by the product of the left
singular vectors' transpose with it (rank = count(svs > tol), an absolute
threshold, :470, :486, :601, :615).  A parent's rows and columns are its two
children's compressed ones; the sibling blocks B are read off the reduced
matrix when the parent is visited (:574-581, root :680-689).

Generators (dict per node): U[i] (rows_i x k_i), V[i] (cols_i x k'_i), B[i]
(k_i x k'_sibling), D[i] (leaf diagonal block), so that for siblings c1, c2
A(I_c1, I_c2) = Ubig_c1 B[c1] Vbig_c2^T with the nested bases expanded.
"""
import numpy as np


def leaf_sizes(n, ni):
    """npart with LTR = 0 (SRC/aux_hss.f90:807-818)."""
    lm = n // ni
    if lm == 0:
        return [n]
    m = [ni] * lm
    mr = n % ni
    if mr >= ni // 2:
        m.append(mr)
    else:
        m[-1] += mr
    return m


def post_order_tree(nleaf):
    """n2tree / btree (SRC/aux_hss.f90:737-778): parent of nodes 1..ltr (root 0)."""
    ltr = 2 * nleaf - 1
    par = [0] * (ltr + 1)

    def perfect(n, off):
        if n == 1:
            par[off + 1] = 0
            return
        h = (n - 1) // 2
        perfect(h, off)
        perfect(h, off + h)
        par[off + h] = par[off + 2 * h] = off + n
        par[off + n] = 0

    def n2(n, off):
        if n == 1:
            par[off + 1] = 0
            return
        p2 = 1
        while p2 * 2 <= n:
            p2 *= 2
        n1 = p2 - 1
        perfect(n1, off)
        n2(n - n1 - 1, off + n1)
        par[off + n1] = par[off + n - 1] = off + n
        par[off + n] = 0

    n2(ltr, 0)
    ch = {i: [] for i in range(1, ltr + 1)}
    for i in range(1, ltr):
        ch[par[i]].append(i)
    return ltr, par, ch


def _trunc(sv, tol):
    return int(np.count_nonzero(sv > tol))


def mat2hss(A, ni, tol):
    """Generators of the HSS approximation of the square matrix A."""
    A = np.array(A, dtype=np.float64)
    n = A.shape[0]
    m = leaf_sizes(n, ni)
    ltr, par, ch = post_order_tree(len(m))
    gen = {"n": n, "ltr": ltr, "par": par, "ch": ch, "m": m,
           "U": {}, "V": {}, "B": {}, "D": {}, "rank": 0}
    if ltr == 1:
        gen["D"][1] = A.copy()
        return gen
    lr, it, pos = {}, 0, 0  # leaf ranges in the original matrix
    for i in range(1, ltr + 1):
        if not ch[i]:
            lr[i] = (pos, pos + m[it])
            pos += m[it]
            it += 1
    # current reduced matrix R; each frontier node's (contiguous) row / column indices
    R = A.copy()
    rows = {i: list(range(*lr[i])) for i in lr}
    cols = {i: list(range(*lr[i])) for i in lr}
    for i in range(1, ltr):
        if not ch[i]:
            a, b = lr[i]
            gen["D"][i] = A[a:b, a:b].copy()
        else:
            c1, c2 = ch[i]
            gen["B"][c1] = R[np.ix_(rows[c1], cols[c2])].copy()
            gen["B"][c2] = R[np.ix_(rows[c2], cols[c1])].copy()
            rows[i] = rows.pop(c1) + rows.pop(c2)
            cols[i] = cols.pop(c1) + cols.pop(c2)
        ri, ci = rows[i], cols[i]
        # block column: every current row outside i
        other_r = sorted(r for nd, rr in rows.items() if nd != i for r in rr)
        Hc = R[np.ix_(other_r, ci)]
        if Hc.size:
            _, sv, wt = np.linalg.svd(Hc, full_matrices=False)
            kc = _trunc(sv, tol)
            Vi = wt[:kc].T
        else:
            kc, Vi = 0, np.zeros((len(ci), 0))
        gen["V"][i] = Vi
        newc = R[:, ci] @ Vi
        # block row: every current column outside i
        other_c = sorted(c for nd, cc in cols.items() if nd != i for c in cc)
        Gr = R[np.ix_(ri, other_c)]
        if Gr.size:
            u, sv, _ = np.linalg.svd(Gr, full_matrices=False)
            kr = _trunc(sv, tol)
            Ui = u[:, :kr]
        else:
            kr, Ui = 0, np.zeros((len(ri), 0))
        gen["U"][i] = Ui
        gen["rank"] = max(gen["rank"], kr, kc)
        # node i's columns, then rows, replaced by their compressed ones
        c0, c1_ = (ci[0], ci[-1]) if ci else (0, -1)
        left, right = list(range(c0)), list(range(c1_ + 1, R.shape[1]))
        R = np.concatenate([R[:, left], newc, R[:, right]], axis=1)
        for nd in cols:
            if nd == i:
                cols[nd] = list(range(len(left), len(left) + kc))
            elif cols[nd] and cols[nd][0] > c0:
                cols[nd] = [c - len(ci) + kc for c in cols[nd]]
        newr = Ui.T @ R[ri, :]
        r0, r1_ = (ri[0], ri[-1]) if ri else (0, -1)
        up, dn = list(range(r0)), list(range(r1_ + 1, R.shape[0]))
        R = np.concatenate([R[up, :], newr, R[dn, :]], axis=0)
        for nd in rows:
            if nd == i:
                rows[nd] = list(range(len(up), len(up) + kr))
            elif rows[nd] and rows[nd][0] > r0:
                rows[nd] = [r - len(ri) + kr for r in rows[nd]]
    c1, c2 = ch[ltr]
    gen["B"][c1] = R[np.ix_(rows[c1], cols[c2])].copy()
    gen["B"][c2] = R[np.ix_(rows[c2], cols[c1])].copy()
    return gen


def hss_times(gen, X):
    """fastHssmm: Y = A_hss X (X: n x ncol)."""
    ch, ltr = gen["ch"], gen["ltr"]
    if ltr == 1:
        return gen["D"][1] @ X
    U, V, B, D = gen["U"], gen["V"], gen["B"], gen["D"]
    off, pos = {}, 0
    for i in range(1, ltr + 1):
        if not ch[i]:
            off[i] = pos
            pos += D[i].shape[0]
    g = {}
    for i in range(1, ltr):  # upsweep g_i = V_i^T x_i
        if not ch[i]:
            xi = X[off[i]:off[i] + D[i].shape[0]]
        else:
            xi = np.vstack([g[c] for c in ch[i]])
        g[i] = V[i].T @ xi
    Y = np.zeros_like(X)

    def down(p, fp):
        c1, c2 = ch[p]
        f1 = B[c1] @ g[c2]
        f2 = B[c2] @ g[c1]
        if fp is not None:
            k1 = U[c1].shape[1]
            t = U[p] @ fp
            f1 = f1 + t[:k1]
            f2 = f2 + t[k1:]
        for c, fc in ((c1, f1), (c2, f2)):
            if ch[c]:
                down(c, fc)
            else:
                a = off[c]
                b = a + D[c].shape[0]
                Y[a:b] = D[c] @ X[a:b] + U[c] @ fc

    down(ltr, None)
    return Y


def transpose_gens(gen):
    """Generators of A^T: U <-> V, B[c1] <-> B[c2]^T, D^T."""
    ch = gen["ch"]
    t = dict(gen)
    t["U"], t["V"] = gen["V"], gen["U"]
    t["D"] = {i: d.T for i, d in gen["D"].items()}
    Bt = {}
    for p in range(1, gen["ltr"] + 1):
        if ch[p]:
            c1, c2 = ch[p]
            Bt[c1] = gen["B"][c2].T
            Bt[c2] = gen["B"][c1].T
    t["B"] = Bt
    return t


def dhssmm(A, B, ni, tol):
    """DHSSMM (SRC/DHSSMM.f90:1-125): returns (A_hss B, max rank)."""
    gen = mat2hss(A, ni, tol)
    return hss_times(gen, np.asarray(B, dtype=np.float64)), gen["rank"]


def dhssmml(A, B, ni, tol):
    """DHSSMML (SRC/DHSSMML.f90:2-122): returns (B A_hss, max rank)."""
    gen = mat2hss(A, ni, tol)
    Bt = np.asarray(B, dtype=np.float64).T
    return hss_times(transpose_gens(gen), Bt).T, gen["rank"]


def fmm_test_matrix(n, seed=0):
    """The matrix of TEST/testfmm.f90:19-36: Cauchy-like A_ij = z_i v_j / (x_i - y_j)
    on interlaced points x_i = 0.1 + g(2i-1), y_i = x_i + g, g = 8.9 / (2n), with
    z, v uniform(0, 1) (seeded numpy draws stand in for Fortran random_number)."""
    sa, sb = 0.1, 9.0
    gap = (sb - sa) / (2 * n)
    x = sa + gap * (2 * np.arange(1, n + 1) - 1)
    y = x + gap
    rng = np.random.default_rng(seed)
    z, v = rng.uniform(size=n), rng.uniform(size=n)
    return z[:, None] * v[None, :] / (x[:, None] - y[None, :])
