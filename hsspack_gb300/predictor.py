"""Training and installation of the learned secular initial iterate.

Training data: secular problems exactly as a DC merge produces them (two seeded
random tridiagonal halves, their eigenvalues as poles, z from the last / first
eigenvector rows, rho = 2|e_cut|, small-z and close-pole deflation as in
MDLAED2), solved by the library's plain secular solver on the GPU; every
non-last root gives one sample (features from the library's feature kernel,
target = logit of the root's position minus the analytic two-pole guess).
The network is trained on the GPU by the library's own forward / backward /
Adam kernels; torch only holds the device buffers.
"""
import ctypes
import os

import numpy as np

WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "predictor_weights.npz")


def _tridiag(d, e):
    return np.diag(d) + np.diag(e, 1) + np.diag(e, -1)


def merge_problems(count, sizes=(32, 64, 128, 256, 512), seed=0, kinds=("uniform",)):
    """Secular problems of DC merges of seeded tridiagonals (CPU, numpy)."""
    rng = np.random.default_rng(seed)
    eps = 2.0 ** -53
    out = []
    while len(out) < count:
        n = int(rng.choice(sizes))
        n1 = n // 2
        kind = kinds[len(out) % len(kinds)]
        if kind == "toeplitz":
            d, e = np.full(n, 2.0), np.ones(n - 1)
        elif kind == "graded":
            d = rng.uniform(-1, 1, n) * np.logspace(0, -6, n)
            e = rng.uniform(-1, 1, n - 1) * np.logspace(0, -6, n - 1)
        else:
            d, e = rng.uniform(-1, 1, n), rng.uniform(-1, 1, n - 1)
        cut = e[n1 - 1]
        d1, d2 = d[:n1].copy(), d[n1:].copy()
        d1[-1] -= abs(cut)
        d2[0] -= abs(cut)
        w1, Q1 = np.linalg.eigh(_tridiag(d1, e[: n1 - 1]))
        w2, Q2 = np.linalg.eigh(_tridiag(d2, e[n1:]))
        z2 = Q2[0, :] * (-1.0 if cut < 0 else 1.0)
        z = np.concatenate([Q1[-1, :], z2]) / np.sqrt(2.0)
        poles = np.concatenate([w1, w2])
        rho = abs(2.0 * cut)
        order = np.argsort(poles, kind="stable")
        poles, z = poles[order], z[order]
        tol = 8.0 * eps * max(np.abs(poles).max(), np.abs(z).max())
        keep = rho * np.abs(z) > tol
        poles, z = poles[keep], z[keep]
        if len(poles) < 3:
            continue
        gap_ok = np.concatenate([[True], np.diff(poles) > 64 * tol])
        poles, z = poles[gap_ok], z[gap_ok]
        if len(poles) < 3:
            continue
        out.append((poles, z, rho))
    return out


def collect(problems):
    """Solve with the plain GPU solver; return (X, T) device tensors."""
    import torch
    import hsspack_gb300 as hp
    L = hp.load()
    nf = L.hss_predictor_nfeat()
    old = hp.set_config(predictor=0)
    Xs, Ts = [], []
    try:
        for d, z, rho in problems:
            k = len(d)
            dd = torch.tensor(d, dtype=torch.float64, device="cuda")
            zz = torch.tensor(z, dtype=torch.float64, device="cuda")
            lam, difl, difr = (torch.zeros(k, dtype=torch.float64, device="cuda") for _ in range(3))
            hp.secular_dev(dd, zz, rho, lam, difl, difr)
            X = torch.zeros((k - 1) * nf, dtype=torch.float32, device="cuda")
            T = torch.zeros(k - 1, dtype=torch.float32, device="cuda")
            rc = L.hss_predictor_features_dev(k, hp._ptr(dd), hp._ptr(zz), float(rho), hp._ptr(difl),
                                              hp._ptr(difr), hp._ptr(X), hp._ptr(T),
                                              hp._stream(None))
            if rc != 0:
                raise hp.HssError("features rc=%d" % rc)
            Xs.append(X.view(k - 1, nf))
            Ts.append(T)
    finally:
        hp.restore_config(old)
    return torch.cat(Xs), torch.cat(Ts)


def init_weights(seed=0):
    import hsspack_gb300 as hp
    L = hp.load()
    nf, nh = L.hss_predictor_nfeat(), 64
    rng = np.random.default_rng(seed)
    parts = [rng.standard_normal((nf, nh)) * np.sqrt(2.0 / nf), np.zeros(nh),
             rng.standard_normal((nh, nh)) * np.sqrt(2.0 / nh), np.zeros(nh),
             rng.standard_normal((nh, nh)) * np.sqrt(2.0 / nh), np.zeros(nh),
             rng.standard_normal(nh) * 1e-3, np.zeros(1)]
    W = np.concatenate([p.ravel() for p in parts]).astype(np.float32)
    assert W.size == L.hss_predictor_nparam()
    return W


def grad(X, T, norm, W):
    """(loss, G) on device tensors through the library's gradient kernel."""
    import torch
    import hsspack_gb300 as hp
    L = hp.load()
    G = torch.zeros(L.hss_predictor_nparam(), dtype=torch.float32, device="cuda")
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    rc = L.hss_predictor_grad_dev(T.numel(), hp._ptr(X), hp._ptr(T), hp._ptr(norm), hp._ptr(W),
                                  hp._ptr(G), hp._ptr(loss), hp._stream(None))
    if rc != 0:
        raise hp.HssError("grad rc=%d" % rc)
    return loss, G


def train(X, T, epochs=30, batch=4096, lr=2e-3, seed=0, log=None):
    """Adam on the GPU; returns (W fp32 numpy, norm numpy, final loss)."""
    import torch
    import hsspack_gb300 as hp
    L = hp.load()
    nf = L.hss_predictor_nfeat()
    mu = X.mean(0)
    sd = X.std(0) + 1e-6
    norm = torch.cat([mu, sd]).contiguous()
    W = torch.tensor(init_weights(seed), device="cuda")
    M = torch.zeros_like(W)
    V = torch.zeros_like(W)
    gen = torch.Generator(device="cuda").manual_seed(seed)
    n = T.numel()
    step = 0
    last = None
    for ep in range(epochs):
        perm = torch.randperm(n, device="cuda", generator=gen)
        tot = 0.0
        for b0 in range(0, n, batch):
            idx = perm[b0:b0 + batch]
            xb, tb = X[idx].contiguous(), T[idx].contiguous()
            loss, G = grad(xb, tb, norm, W)
            step += 1
            rc = L.hss_predictor_adam_dev(hp._ptr(G), hp._ptr(W), hp._ptr(M), hp._ptr(V),
                                          ctypes.c_float(lr * (0.5 ** (ep // 10))), step,
                                          hp._stream(None))
            if rc != 0:
                raise hp.HssError("adam rc=%d" % rc)
            tot += float(loss) * idx.numel()
        last = tot / n
        if log:
            log("epoch %d loss %.4e" % (ep, last))
    return W.cpu().numpy(), norm.cpu().numpy(), last


def install(path=WEIGHTS):
    """Load saved weights into the library (returns False if none saved)."""
    import hsspack_gb300 as hp
    if not os.path.exists(path):
        return False
    z = np.load(path)
    W = np.ascontiguousarray(z["W"], dtype=np.float32)
    norm = np.ascontiguousarray(z["norm"], dtype=np.float32)
    rc = hp.load().hss_predictor_set(W.ctypes.data_as(ctypes.c_void_p),
                                     norm.ctypes.data_as(ctypes.c_void_p))
    if rc != 0:
        raise hp.HssError("predictor_set rc=%d" % rc)
    return True


def iterations(problems, use_predictor):
    """Mean secular evaluations per root and roots, with / without the predictor."""
    import torch
    import hsspack_gb300 as hp
    old = hp.set_config(predictor=int(use_predictor))
    its, roots, fb = 0, 0, 0
    lams = []
    try:
        for d, z, rho in problems:
            k = len(d)
            dd = torch.tensor(d, dtype=torch.float64, device="cuda")
            zz = torch.tensor(z, dtype=torch.float64, device="cuda")
            lam, difl, difr = (torch.zeros(k, dtype=torch.float64, device="cuda") for _ in range(3))
            it = torch.zeros(k, dtype=torch.int32, device="cuda")
            hp.secular_dev(dd, zz, rho, lam, difl, difr, it)
            its += int(it.sum())
            roots += k
            fb += hp.get_stats()["predictor_fallbacks"]
            lams.append(lam.cpu().numpy())
    finally:
        hp.restore_config(old)
    return its / roots, fb, lams


def main(argv=None):
    import argparse
    import json
    import hsspack_gb300 as hp
    ap = argparse.ArgumentParser(description="train the secular predictor on the GPU")
    ap.add_argument("--out", default=WEIGHTS)
    ap.add_argument("--epochs", type=int, default=30)
    a = ap.parse_args(argv)
    hp.load()
    train_p = merge_problems(600, seed=1, kinds=("uniform", "uniform", "toeplitz", "graded"))
    test_p = merge_problems(100, seed=2, kinds=("uniform", "uniform", "toeplitz", "graded"))
    X, T = collect(train_p)
    W, norm, loss = train(X, T, epochs=a.epochs, log=print)
    np.savez(a.out, W=W, norm=norm, train_loss=loss, samples=T.numel())
    install(a.out)
    base, _, lam0 = iterations(test_p, False)
    pred, fb, lam1 = iterations(test_p, True)
    dmax = max(float(np.max(np.abs(a - b))) for a, b in zip(lam0, lam1))
    # ablation: the analytic slope-refined start alone (network output 0)
    zero = np.zeros_like(W)
    hp.load().hss_predictor_set(zero.ctypes.data, norm.ctypes.data)
    analytic, fb0, _ = iterations(test_p, True)
    install(a.out)
    print(json.dumps({"samples": int(T.numel()), "train_loss": loss,
                      "evaluations_per_root_standard": base,
                      "evaluations_per_root_analytic_start": analytic,
                      "evaluations_per_root_learned": pred, "fallbacks": fb,
                      "fallbacks_analytic": fb0, "max_root_difference": dmax}))


if __name__ == "__main__":
    main()
