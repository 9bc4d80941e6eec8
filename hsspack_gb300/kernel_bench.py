"""Microbenchmarks of single library stages on one GPU, for profiling.

    python -m hsspack_gb300.kernel_bench gemm --m 32768 --n 128 --k 128 --precision 1
    python -m hsspack_gb300.kernel_bench secular --k 8192
    python -m hsspack_gb300.kernel_bench dhssevc --k 8192 --nrows 8192 --leaf 128 --tol 1e-14
    python -m hsspack_gb300.kernel_bench dc --n 32768

Each run does --warmup untimed and --reps timed calls (CUDA events on the
calling stream) and prints one JSON line.  Inputs are seeded: GEMM operands
N(0,1); secular / Cauchy problems with poles sorted U[0,1], weights
N(0,1)/sqrt(k), rho = 1; DC: diagonal and off-diagonal U[-1,1].
"""
import argparse
import json
import sys

import numpy as np


def _events(torch):
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def bench_gemm(a, torch, hp):
    rng = np.random.default_rng(0)
    A = torch.tensor(rng.standard_normal(a.m * a.k), dtype=torch.float64, device="cuda")
    B = torch.tensor(rng.standard_normal(a.k * a.n), dtype=torch.float64, device="cuda")
    C = torch.zeros(a.m * a.n, dtype=torch.float64, device="cuda")
    for _ in range(a.warmup):
        hp.gemm_dev(A, B, C, a.m, a.n, a.k, a.m, a.k, a.m, precision=a.precision)
    t0, t1 = _events(torch)
    t0.record()
    for _ in range(a.reps):
        hp.gemm_dev(A, B, C, a.m, a.n, a.k, a.m, a.k, a.m, precision=a.precision)
    t1.record()
    torch.cuda.synchronize()
    ms = t0.elapsed_time(t1) / a.reps
    fl = 2.0 * a.m * a.n * a.k
    return {"stage": "gemm", "m": a.m, "n": a.n, "k": a.k, "precision": a.precision, "ms": ms,
            "fp64_equiv_tflops": fl / ms / 1e9}


def _secular_problem(k, seed=0):
    rng = np.random.default_rng(seed)
    d = np.sort(rng.uniform(0.0, 1.0, k)) + np.arange(k) * 1e-12
    z = rng.standard_normal(k) / np.sqrt(k)
    return d, z, 1.0


def bench_secular(a, torch, hp):
    d, z, rho = _secular_problem(a.k)
    dd = torch.tensor(d, dtype=torch.float64, device="cuda")
    zz = torch.tensor(z, dtype=torch.float64, device="cuda")
    lam, difl, difr = (torch.zeros(a.k, dtype=torch.float64, device="cuda") for _ in range(3))
    it = torch.zeros(a.k, dtype=torch.int32, device="cuda")
    for _ in range(a.warmup):
        hp.secular_dev(dd, zz, rho, lam, difl, difr, it)
    t0, t1 = _events(torch)
    t0.record()
    for _ in range(a.reps):
        hp.secular_dev(dd, zz, rho, lam, difl, difr, it)
    t1.record()
    torch.cuda.synchronize()
    ms = t0.elapsed_time(t1) / a.reps
    evals = float(it.sum())
    return {"stage": "secular", "k": a.k, "ms": ms, "mean_evaluations": evals / a.k,
            "pole_terms_per_s": evals * a.k / (ms * 1e-3)}


def bench_dhssevc(a, torch, hp):
    d, z, rho = _secular_problem(a.k)
    dd = torch.tensor(d, dtype=torch.float64, device="cuda")
    zz = torch.tensor(z, dtype=torch.float64, device="cuda")
    lam, difl, difr = (torch.zeros(a.k, dtype=torch.float64, device="cuda") for _ in range(3))
    hp.secular_dev(dd, zz, rho, lam, difl, difr)
    zh, alpha = zz.clone(), torch.zeros(a.k, dtype=torch.float64, device="cuda")
    hp.lowner_dev(dd, difl, difr, zh, alpha)
    gen = torch.Generator(device="cuda").manual_seed(1)
    Q0 = torch.randn(a.k * a.nrows, dtype=torch.float64, device="cuda", generator=gen)
    Q = Q0.clone()
    old = hp.set_config(precision=a.precision)
    try:
        for _ in range(a.warmup):
            Q.copy_(Q0)
            hp.dhssevc_dev(dd, zh, alpha, difl, difr, Q, a.nrows, a.nrows, ni=a.leaf, tol=a.tol)
        t0, t1 = _events(torch)
        t0.record()
        for _ in range(a.reps):
            hp.dhssevc_dev(dd, zh, alpha, difl, difr, Q, a.nrows, a.nrows, ni=a.leaf, tol=a.tol)
        t1.record()
        torch.cuda.synchronize()
    finally:
        hp.restore_config(old)
    ms = t0.elapsed_time(t1) / a.reps
    return {"stage": "dhssevc", "k": a.k, "nrows": a.nrows, "leaf": a.leaf, "tol": a.tol,
            "precision": a.precision, "ms": ms, "max_rank": hp.get_stats()["max_rank"]}


def bench_dc(a, torch, hp):
    rng = np.random.default_rng(0)
    d, e = rng.uniform(-1, 1, a.n), rng.uniform(-1, 1, a.n - 1)
    d0 = torch.tensor(d, dtype=torch.float64, device="cuda")
    e0 = torch.tensor(e, dtype=torch.float64, device="cuda")
    dw, ew = d0.clone(), e0.clone()
    Z = torch.empty(a.n * a.n, dtype=torch.float64, device="cuda")
    old = hp.set_config(precision=a.precision, smlsiz=a.smlsiz)
    try:
        ms = []
        for i in range(a.warmup + a.reps):
            dw.copy_(d0)
            ew.copy_(e0)
            hp.mdstedc_dev(dw, ew, Z)
            if i >= a.warmup:
                ms.append(hp.get_stats()["ms_total"])
    finally:
        hp.restore_config(old)
    return {"stage": "dc", "n": a.n, "precision": a.precision, "smlsiz": a.smlsiz,
            "ms": float(np.mean(ms)), "stats": {k: v for k, v in hp.get_stats().items()
                                                if not k.startswith("stage_")}}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("stage", choices=["gemm", "secular", "dhssevc", "dc"])
    ap.add_argument("--m", type=int, default=32768)
    ap.add_argument("--n", type=int, default=128)
    ap.add_argument("--k", type=int, default=128)
    ap.add_argument("--nrows", type=int, default=8192)
    ap.add_argument("--leaf", type=int, default=128)
    ap.add_argument("--tol", type=float, default=1e-14)
    ap.add_argument("--precision", type=int, default=1)
    ap.add_argument("--smlsiz", type=int, default=25)
    ap.add_argument("--warmup", type=int, default=2)
    ap.add_argument("--reps", type=int, default=3)
    a = ap.parse_args(argv)
    import torch
    import hsspack_gb300 as hp
    fn = {"gemm": bench_gemm, "secular": bench_secular, "dhssevc": bench_dhssevc, "dc": bench_dc}
    print(json.dumps(fn[a.stage](a, torch, hp)), flush=True)


if __name__ == "__main__":
    sys.exit(main())
