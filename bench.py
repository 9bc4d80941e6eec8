"""Benchmark: FP64 tridiagonal divide-and-conquer eigensolve, n = 32768.

Workload (one step): MDSTEDC('I') of the symmetric tridiagonal with diagonal
and off-diagonal iid uniform[-1, 1] (numpy PCG64, seed 0), n = 32768: all
eigenvalues and the full 32768 x 32768 FP64 eigenvector matrix.  The
eigenvector matrix (8.6 GB) is far larger than L2, so no flush is needed
between steps.

value: device-resident seconds per solve (inputs already in HBM, CUDA events
on the launching stream over exactly K steps, no per-stage events).  batch: the
second half of the metric, 512 uneven tridiagonals (n log-uniform in
[256, 4096]) solved in one batched call, as solves/s, beside one call per
problem and the plain GPU merge.  e2e: the same solve through the Fortran
drop-in ``mdstedc_`` with pageable host arrays (D/E host->device, the
eigenvectors and eigenvalues device->host and the host-side zero fill of Z
inside the timed region).  roofline: the final gather, the longest single
launch, its algorithmic bytes over its event-timed duration.  cpu_baseline /
--impl reference: the CPU oracle (C++ restatement of HSSPACK's MDSTEDC +
LAPACK from OpenBLAS) on the host cores.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_DEFAULT = 32768
METRIC = ("DC eigensolve s n=32768 + batch solves/s: learned/batched vs plain GPU, "
          "resid≤1e-12")


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        j = json.load(open(p))
        return {"hbm_gbs": j.get("hbm_gbs", 6800.0), "bf16_tflops": j.get("bf16_tflops", 1900.0),
                "source": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "source": "fallback"}


def inputs(n, seed=0):
    rng = np.random.default_rng(seed)
    return rng.uniform(-1.0, 1.0, n), rng.uniform(-1.0, 1.0, n - 1)


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.rows, self.proc, self.th = [], None, None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "25"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.th = threading.Thread(target=self._read, daemon=True)
        self.th.start()
        # nvidia-smi takes a moment to start: let it, so the samples cover the
        # warm-up and timed solves that follow
        t0 = time.time()
        while not self.rows and time.time() - t0 < 2.0:
            time.sleep(0.01)

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = [r for r in self.rows if len(r) >= 8 and r[1].replace(".", "").isdigit()]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = sorted(float(r[1]) for r in rows)
        reasons = set()
        for r in rows:
            for name, v in zip(["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                                "sw_power_cap"], r[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": float(rows[0][2]),
                "samples": len(rows), "reasons": sorted(reasons)}


def check_accuracy(torch, d, e, w, Z, n):
    """||TQ - QW||_F/(n||T||) exactly and ||Q^T Q - I||_F/n by 8 Gaussian probes
    (E||(Q^T Q - I) g||^2 = ||Q^T Q - I||_F^2), in FP64 on the GPU."""
    Q = Z.view(n, n)  # row c of the tensor = column c of Q (column-major storage)
    dd = torch.tensor(d, dtype=torch.float64, device="cuda")
    ee = torch.tensor(e, dtype=torch.float64, device="cuda")
    tn = float(torch.max(torch.abs(dd) + torch.nn.functional.pad(torch.abs(ee), (0, 1))
                         + torch.nn.functional.pad(torch.abs(ee), (1, 0))))
    res2 = 0.0
    for c0 in range(0, n, 4096):
        blk = Q[c0:c0 + 4096]  # (b, n): columns c0.. of Q as rows
        tq = blk * dd[None, :]
        tq[:, :-1] += blk[:, 1:] * ee[None, :]
        tq[:, 1:] += blk[:, :-1] * ee[None, :]
        r = tq - blk * w[c0:c0 + 4096, None]
        res2 += float(torch.sum(r * r))
    gen = torch.Generator(device="cuda").manual_seed(1)
    g = torch.randn(n, 8, dtype=torch.float64, device="cuda", generator=gen)
    y = Q.T.matmul(Q.matmul(g)) - g  # (Q^T Q - I) g with Q = tensor.T
    orth = float(torch.sqrt(torch.sum(y * y) / 8)) / n
    return {"resid": (res2 ** 0.5) / (n * tn), "orth_est": orth}


def cpu_reference_solve(n, threads):
    """One solve of the n x n benchmark matrix by the CPU oracle (the restated
    HSSPACK MDSTEDC('I') + OpenBLAS LAPACK) on `threads` host threads; seconds."""
    import oracle
    oracle.set_threads(threads)
    d, e = inputs(n, seed=0)
    t = time.perf_counter()
    oracle.eigh_tridiagonal(d, e)
    return time.perf_counter() - t


def cpu_lapack_solve(n, threads):
    """LAPACK DSTEDC('I') (OpenBLAS, the oracle's accuracy reference) on the
    same matrix; seconds."""
    import oracle
    oracle.set_threads(threads)
    d, e = inputs(n, seed=0)
    t = time.perf_counter()
    oracle.dstedc_lapack(d, e)
    return time.perf_counter() - t


BATCH_COUNT, BATCH_LO, BATCH_HI = 512, 256, 4096


def batch_inputs(seed=2):
    """512 tridiagonals, n = round(exp(U[ln 256, ln 4096])) (seed 2), D, E iid
    U[-1, 1] (problem p from seed 1000 + p)."""
    rng = np.random.default_rng(seed)
    sizes = np.round(np.exp(rng.uniform(np.log(BATCH_LO), np.log(BATCH_HI), BATCH_COUNT)))
    sizes = sizes.astype(np.int32)
    probs = [inputs(int(n), seed=1000 + p) for p, n in enumerate(sizes)]
    return sizes, probs


def batch_cpu_solve(probs, threads):
    """The CPU oracle on every problem of the batch, one after the other (the
    reference solves independent problems serially); seconds."""
    import oracle
    oracle.set_threads(threads)
    t = time.perf_counter()
    for d, e in probs:
        oracle.eigh_tridiagonal(d, e)
    return time.perf_counter() - t


def profile_batch(args, torch, hp, full_cfg):
    """Only the batched solves of the uneven batch (warm-up + steps): the
    command an ncu launch list of the batch wraps."""
    sizes, probs = batch_inputs()
    _, D, E = hp.pack_batch(probs)
    o, oz = hp.batch_offsets(sizes)
    d0 = torch.tensor(D, device="cuda")
    e0 = torch.tensor(E, device="cuda")
    d, e = d0.clone(), e0.clone()
    z = torch.empty(int(oz[-1]), dtype=torch.float64, device="cuda")
    old = hp.set_config(**full_cfg)
    try:
        for it in range(args.warmup + args.steps):
            if it == args.warmup:
                torch.cuda.synchronize()
                t0 = time.perf_counter()
            d.copy_(d0)
            e.copy_(e0)
            hp.mdstedc_batch_dev(sizes, d, e, z)
        torch.cuda.synchronize()
        ms = (time.perf_counter() - t0) * 1e3 / max(1, args.steps)
        return {"profile_batch": True, "ms_per_batch": ms, "launches_per_batch":
                hp.get_stats()["kernel_launches"], "config": full_cfg}
    finally:
        hp.restore_config(old)


def run_batch(args, torch, hp, full_cfg, plain_cfg, world, rank, dist):
    """The uneven batch: solves/s batched (one call), one call per problem, and
    with the plain GPU merge; residual of every problem on the device.  With
    several ranks every rank solves its share of the 512 problems (greedy n^3
    partition, no collective on the data path) and the time is the slowest
    rank's."""
    sizes_all, probs_all = batch_inputs()
    sizes, probs = sizes_all, probs_all
    if world > 1:
        from hsspack_gb300 import shard
        mine = shard.partition(sizes_all, world)[rank]
        sizes = sizes_all[mine]
        probs = [probs_all[int(i)] for i in mine]
    _, D, E = hp.pack_batch(probs)
    o, oz = hp.batch_offsets(sizes)
    d0 = torch.tensor(D, device="cuda")
    e0 = torch.tensor(E, device="cuda")
    d, e = d0.clone(), e0.clone()
    z = torch.empty(int(oz[-1]), dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()

    def batched():
        d.copy_(d0)
        e.copy_(e0)
        hp.mdstedc_batch_dev(sizes, d, e, z, stream=stream)

    def loop():
        for p in range(len(sizes)):
            a, b = int(o[p]), int(o[p + 1])
            d[a:b].copy_(d0[a:b])
            e[a:b].copy_(e0[a:b])
            hp.mdstedc_dev(d[a:b], e[a:b], z[int(oz[p]):int(oz[p + 1])], stream=stream)

    def timed(fn, steps, warmup, cfg):
        old = hp.set_config(**cfg)
        launches = 0
        try:
            for _ in range(warmup):
                fn()
            if world > 1:
                dist.barrier()
            torch.cuda.synchronize()
            t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            t0.record(stream)
            for _ in range(steps):
                fn()
            t1.record(stream)
            torch.cuda.synchronize()
            # the last call's launch count (each step does the same work),
            # read after the timed region
            launches = hp.get_stats()["kernel_launches"] * steps
            ms = t0.elapsed_time(t1) / steps
            if world > 1:  # the slowest rank's time
                x = torch.tensor([ms], device="cuda")
                dist.all_reduce(x, op=dist.ReduceOp.MAX)
                ms = float(x)
            return ms, launches
        finally:
            hp.restore_config(old)

    # the batch's own leaf size (its problems are far smaller than n = 32768):
    # one warm and one timed call per candidate, outside the measured region
    bcfg, tune_ms = dict(full_cfg), {}
    if args.smlsiz <= 0:
        for sml in (8, 12, 16):
            tune_ms[str(sml)] = timed(batched, 1, 1, dict(full_cfg, smlsiz=sml))[0]
        bcfg["smlsiz"] = int(min(tune_ms, key=tune_ms.get))
        # products of 64 to 127 rows on the tensor cores (128-row tiles, the rest
        # zero) instead of the FP64 element kernel
        key = "%d+m64" % bcfg["smlsiz"]
        tune_ms[key] = timed(batched, 1, 1, dict(bcfg, split_min_m=64))[0]
        best = tune_ms[str(bcfg["smlsiz"])]
        if tune_ms[key] < best:
            bcfg["split_min_m"] = 64
            best = tune_ms[key]
        # the FP32 pre-solve refined by one float-float step (predictor 3)
        if int(bcfg.get("predictor", 0)) == 2:
            key = "%d+ff" % bcfg["smlsiz"]
            tune_ms[key] = timed(batched, 1, 1, dict(bcfg, predictor=3))[0]
            if tune_ms[key] < best:
                bcfg["predictor"] = 3
    steps = max(1, min(args.steps, 5))
    ms, launches = timed(batched, steps, max(3, args.warmup), bcfg)
    # every problem's residual ||TQ - QW||_F / (n ||T||) from the last solve
    res = 0.0
    for p, n in enumerate(sizes):
        n = int(n)
        a, b = int(o[p]), int(o[p + 1])
        Q = z[int(oz[p]):int(oz[p + 1])].view(n, n).T
        dd, ee = d0[a:b], e0[a:b - 1]
        R = dd[:, None] * Q - Q * d[a:b][None, :]
        R[:-1] += ee[:, None] * Q[1:]
        R[1:] += ee[:, None] * Q[:-1]
        tn = float(dd.abs().max() + 2 * ee.abs().max())
        res = max(res, float(torch.linalg.norm(R)) / (n * tn))
    # the other arms, each warmed once: one call per problem, batched levels
    # with FP64 products (no tensor cores), and the plain GPU merge (per-merge
    # launches, FP64 products, standard start)
    ms_loop, _ = timed(loop, 2, 1, bcfg)
    ms_fp64, _ = timed(batched, 2, 1, dict(bcfg, precision=0))
    ms_std, _ = timed(batched, 2, 1, dict(bcfg, predictor=0))
    ms_plain, _ = timed(batched, 1, 1, dict(plain_cfg, smlsiz=bcfg.get("smlsiz", 0)))
    out = {"workload": "512 tridiagonals, n log-uniform in [256, 4096] (seed 2), D,E iid U[-1,1]",
           "sum_n": int(o[-1]), "sum_n2": int(oz[-1]),
           "solves_per_s": len(sizes_all) * 1000.0 / ms, "ms_per_batch": ms,
           "problems_this_rank": int(len(sizes)), "ranks": world,
           "gpu_launches_per_batch": launches / steps,
           "loop_solves_per_s": len(sizes_all) * 1000.0 / ms_loop,
           "batched_fp64_solves_per_s": len(sizes_all) * 1000.0 / ms_fp64,
           "standard_start_solves_per_s": len(sizes_all) * 1000.0 / ms_std,
           "plain_solves_per_s": len(sizes_all) * 1000.0 / ms_plain,
           "full_vs_plain": ms_plain / ms, "full_vs_batched_fp64": ms_fp64 / ms,
           "full_vs_standard_start": ms_std / ms, "batched_vs_loop": ms_loop / ms,
           "resid_max": res, "smlsiz": bcfg.get("smlsiz"),
           "split_min_m": bcfg.get("split_min_m", 128), "predictor": bcfg.get("predictor"),
           "autotune_ms": tune_ms or None}
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        t_s = batch_cpu_solve(probs_all, threads)
        out["cpu_baseline"] = {"value": len(sizes_all) / t_s, "unit": "solves/s", "cores": threads,
                               "kind": "port",
                               "sample": "all 512 problems once (%.2f s)" % t_s}
    return out


FP64_NOMINAL_TFLOPS = 1.25  # GB300 FP64 (CUDA cores) rate, nominal: context only
# per stage: the unit that bounds it on GB300
STAGE_BOUND = {"secular": "fp64", "lowner": "fp64", "build_S": "fp64", "leaf": "fp64",
               "gemm": "fp64-equivalent", "final_gather": "hbm", "prepare": "hbm",
               "gather": "hbm", "scatter": "hbm", "givens": "hbm", "finish": "hbm"}


def stage_rooflines(acc, pk):
    """Achieved rate of every timed stage from its algorithmic bytes / flops:
    HBM stages against the measured copy bandwidth, FP64 stages against the
    FP64 FMA rate measured in this run (hss_fp64_fma_rate), the products as
    FP64-equivalent TFLOP/s (the split-BF16 path is meant to exceed the FP64
    rate)."""
    out = {}
    for st, ms in acc["ms"].items():
        if ms <= 0 or st not in STAGE_BOUND:
            continue
        b = STAGE_BOUND[st]
        if b == "hbm":
            a = acc["bytes"][st] / (ms * 1e-3) / 1e9
            out[st] = {"bound": "hbm", "achieved": a, "peak": pk["hbm_gbs"], "unit": "GB/s",
                       "frac": a / pk["hbm_gbs"], "peak_source": pk["source"]}
        else:
            a = acc["flops"][st] / (ms * 1e-3) / 1e12
            out[st] = {"bound": b, "achieved": a, "peak": pk["fp64_tflops"], "unit": "TFLOP/s",
                       "frac": a / pk["fp64_tflops"], "peak_source": pk["fp64_source"]}
    return out


def _timed_ms(torch, fn, reps=3):
    fn()
    torch.cuda.synchronize()
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0.record()
    for _ in range(reps):
        fn()
    t1.record()
    torch.cuda.synchronize()
    return t0.elapsed_time(t1) / reps


def run_extra_child(full_cfg):
    """run_extra in a child process with its own CUDA context: a failure there
    (a device error included) cannot take this run's line with it."""
    cmd = [sys.executable, os.path.abspath(__file__), "--extra-only", "--extra-cfg",
           json.dumps(full_cfg)]
    try:
        r = subprocess.run(cmd, capture_output=True, text=True, timeout=900)
    except subprocess.TimeoutExpired:
        return {"error": "secondary figures: no result within 900 s"}
    lines = [x for x in r.stdout.splitlines() if x.startswith("{")]
    if r.returncode != 0 or not lines:
        tail = (r.stderr or r.stdout).strip().splitlines()
        return {"error": "secondary figures: exit %d: %s" % (r.returncode, tail[-1] if tail else "")}
    return json.loads(lines[-1])


def run_extra(torch, hp, full_cfg):
    """Secondary figures (not the metric): the other configurations' device
    times through the library's device entry points."""
    out = {}
    old = hp.set_config(**{k: v for k, v in full_cfg.items() if k != "predictor"})
    try:
        # bidiagonal SVD n = 16384, d, e iid U(0, 1] (seed 0)
        n = 16384
        rng = np.random.default_rng(0)
        d = torch.tensor(1.0 - rng.uniform(0.0, 1.0, n), device="cuda")
        e = torch.tensor(1.0 - rng.uniform(0.0, 1.0, n - 1), device="cuda")
        dw, ew = d.clone(), e.clone()
        u = torch.empty(n * n, dtype=torch.float64, device="cuda")
        vt = torch.empty_like(u)

        def svd():
            dw.copy_(d)
            ew.copy_(e)
            hp.mdbdsdc_dev(dw, ew, u, vt)

        hp.set_config(predictor=2)  # FP32 pre-solved secular starts (squared mode)
        out["bidiagonal_svd_n16384_ms"] = _timed_ms(torch, svd)
        hp.set_config(predictor=0)
        del u, vt
        # banded SVD (MDBDSVD) n = 5000, SB = 5, AB iid U[0, 1), SMLSIZ = 75: the
        # reference's test case (TEST/test_bdc1.f90); products split-BF16 and FP64
        n, sb = 5000, 5
        abh = np.random.default_rng(2013).uniform(0.0, 1.0, (sb + 1, n))
        abt = torch.tensor(np.asfortranarray(abh).ravel(order="F"), device="cuda")
        sv = torch.empty(n, dtype=torch.float64, device="cuda")
        uv = torch.empty(n * n, dtype=torch.float64, device="cuda")
        vv = torch.empty(n * n, dtype=torch.float64, device="cuda")
        for prec, key in ((1, "split"), (0, "fp64")):
            hp.set_config(precision=prec, predictor=2)
            out["banded_svd_n5000_sb5_%s_ms" % key] = _timed_ms(
                torch, lambda: hp.mdbdsvd_dev(sb, abt, sv, uv, vv, smlsiz=75))
        hp.set_config(precision=full_cfg.get("precision", 1), predictor=0)
        st = hp.get_stats()
        out["banded_svd_n5000_sb5_stats"] = {"levels": st["n_levels"], "appends": st["n_merges"],
                                             "max_k": st["max_k"], "total_k": st["total_k"]}
        del uv, vv
        # banded n = 16384, kd = 4, entries iid U[-1, 1] (seed 0)
        n, kd = 16384, 4
        ab = rng.uniform(-1.0, 1.0, (kd + 1, n))
        abd = torch.tensor(np.ascontiguousarray(ab.T), device="cuda")
        w = torch.empty(n, dtype=torch.float64, device="cuda")
        z = torch.empty(n * n, dtype=torch.float64, device="cuda")
        out["banded_n16384_kd4_ms"] = _timed_ms(torch, lambda: hp.mdsbevd_dev(kd, abd, w, z))
        del z
        # Cauchy merge n = 8192: secular, Loewner, HSS compression (leaf 128,
        # tol 1e-14) and the product with a dense 8192 x 8192 matrix
        n = 8192
        rng = np.random.default_rng(0)
        dd = torch.tensor(np.sort(rng.uniform(0.0, 1.0, n)), device="cuda")
        zz = torch.tensor(rng.standard_normal(n) / np.sqrt(n), device="cuda")
        lam, difl, difr = (torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(3))
        out["cauchy_secular_n8192_ms"] = _timed_ms(
            torch, lambda: hp.secular_dev(dd, zz, 1.0, lam, difl, difr))
        zh, al = zz.clone(), torch.zeros(n, dtype=torch.float64, device="cuda")
        hp.lowner_dev(dd, difl, difr, zh, al)
        Q = torch.randn(n * n, dtype=torch.float64, device="cuda")
        for prec in (0, 1):
            hp.set_config(precision=prec)
            key = "fp64" if prec == 0 else "split_bf16"
            out["cauchy_hss_multiply_n8192_%s_ms" % key] = \
                _timed_ms(torch, lambda: hp.dhssevc_dev(dd, zh, al, difl, difr, Q, n, n, ni=128,
                                                        tol=1e-14))
            # the last call's construction and product (CUDA events in the library)
            stt = hp.get_stats()["stage_ms"]
            out["cauchy_hss_n8192_%s_build_ms" % key] = stt["hss_build"]
            out["cauchy_hss_n8192_%s_product_ms" % key] = stt["hss_multiply"]
        out["cauchy_hss_max_rank"] = hp.get_stats()["max_rank"]
        del Q
        # DHSSMM: the Cauchy-like matrix of TEST/testfmm.f90 (interlaced points,
        # z, v iid U(0, 1)), tol 1e-11, leaf 64, times B (n x k, iid U(0, 1))
        hp.set_config(precision=full_cfg.get("precision", 1))
        for n, k in ((2000, 2000), (8192, 1024)):
            gap = 8.9 / (2 * n)
            x = 0.1 + gap * (2 * np.arange(1, n + 1) - 1)
            rng = np.random.default_rng(0)
            zv, vv = rng.uniform(size=n), rng.uniform(size=n)
            A = torch.tensor(np.ascontiguousarray((zv[:, None] * vv[None, :] / (x[:, None] - x[None, :] - gap)).T),
                             device="cuda")
            B0 = torch.rand(k, n, dtype=torch.float64, device="cuda")
            ref = (A.T @ B0.T).T
            Bd = B0.clone()
            hp.dhssmm_dev(A, Bd, 64, 1e-11, side=0)
            ts = []
            for _ in range(3):
                Bd.copy_(B0)
                ts.append(hp.dhssmm_dev(A, Bd, 64, 1e-11, side=0))
            tb = min(t[0] for t in ts)
            tm = min(t[1] for t in ts)
            out["dhssmm_n%d_k%d" % (n, k)] = {
                "build_ms": round(tb, 3), "multiply_ms": round(tm, 3),
                "max_rank": hp.get_stats()["max_rank"],
                "max_abs_err_vs_dense": float((Bd - ref).abs().max())}
            del A, B0, Bd, ref
        # HSS Cholesky (HssCholSolver) n = 8192: Gaussian kernel (length 0.01) on
        # sorted uniform points plus 1e-2 I; leaves of 32, tol 1e-8, at most 20
        # per node; factor, solve, CG preconditioned by it and plain CG (tau 1e-13)
        hp.set_config(precision=0)
        n = 8192
        xs = torch.sort(torch.rand(n, dtype=torch.float64, device="cuda",
                                   generator=torch.Generator("cuda").manual_seed(0)))[0]
        Ak = torch.exp(-0.5 * ((xs[:, None] - xs[None, :]) / 0.01) ** 2)
        Ak += 1e-2 * torch.eye(n, dtype=torch.float64, device="cuda")
        Ak = Ak.reshape(-1)
        bk = Ak.view(n, n).sum(1)
        xk = torch.zeros_like(bk)
        fac = [None]

        def factor():
            if fac[0] is not None:
                fac[0].free()
            fac[0] = hp.HssChol(Ak, 32, 1e-8, 20)

        out["hss_cholesky_n8192_factor_ms"] = _timed_ms(torch, factor)
        out["hss_cholesky_n8192_max_rank"] = fac[0].info()["max_rank"]
        yk = bk.clone()
        out["hss_cholesky_n8192_solve_ms"] = _timed_ms(torch, lambda: (yk.copy_(bk), fac[0].solve(yk)))
        t0 = time.perf_counter()
        it, rr = fac[0].pcg(Ak, bk, xk, 1e-13, 30)
        out["hss_cholesky_n8192_pcg"] = {"steps": it, "relres": rr,
                                         "ms": (time.perf_counter() - t0) * 1e3}
        it0, rr0 = fac[0].pcg(Ak, bk, xk, 1e-13, 30, precondition=False)
        out["hss_cholesky_n8192_plain_cg"] = {"steps": it0, "relres": rr0}
        fac[0].free()
        del Ak
    finally:
        hp.restore_config(old)
    return out


def run_reference(args):
    """The reference arm: the CPU restatement of HSSPACK's MDSTEDC('I') (with
    OpenBLAS LAPACK for the routines the reference calls but does not ship) on
    all host cores; each step is one full solve of the same n = 32768 matrix
    as our arm (no scaling, no sampling)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import oracle
    threads = os.cpu_count() or 1
    oracle.set_threads(threads)
    times = []
    t_run = time.perf_counter()
    for i in range(args.warmup + args.steps):
        t = cpu_reference_solve(args.n, threads)
        if i >= args.warmup:
            times.append(t)
    v = float(np.mean(times))
    line = {
        "metric": METRIC, "value": v, "unit": "s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": v * 1000.0, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "impl": "reference",
        "config": {"workload": "tridiagonal DC eigensolve n=%d, D,E iid U[-1,1] seed 0, COMPZ='I'"
                   % args.n, "n": args.n, "l2": "eigenvector matrix 8.6 GB >> L2"},
        "cpu_baseline": {"value": v, "unit": "s", "cores": threads, "kind": "port",
                         "sample": "one full n=%d solve per step (min %.2f s, max %.2f s)"
                                   % (args.n, min(times), max(times))},
        "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "run_s": time.perf_counter() - t_run,
    }
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch
    import torch.distributed as dist
    import hsspack_gb300 as hp

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    n = args.n
    d, e = inputs(n, seed=rank)  # replicas: each rank solves its own problem
    d0 = torch.tensor(d, dtype=torch.float64, device="cuda")
    e0 = torch.tensor(e, dtype=torch.float64, device="cuda")
    dw, ew = d0.clone(), e0.clone()
    Z = torch.empty(n * n, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()

    def solve():
        dw.copy_(d0)
        ew.copy_(e0)
        hp.mdstedc_dev(dw, ew, Z, stream=stream)

    def timed(steps, warmup, profile, cfg):
        old = hp.set_config(profile=int(profile), **cfg)
        try:
            for _ in range(warmup):
                solve()
            torch.cuda.synchronize()
            acc = {"ms": {}, "bytes": {}, "flops": {}, "calls": {}}
            launches = 0
            if world > 1:
                dist.barrier()
            torch.cuda.synchronize()
            t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            t0.record(stream)
            for _ in range(steps):
                solve()
                if profile:  # per-step stage times (stats are reset by every call)
                    st = hp.get_stats()
                    launches += st["kernel_launches"]
                    for k in acc:
                        for s, v in st["stage_" + k].items():
                            acc[k][s] = acc[k].get(s, 0) + v
            t1.record(stream)
            torch.cuda.synchronize()
            ms = t0.elapsed_time(t1) / steps
            if not profile:
                # every step does the same work: the last call's counts, times
                # the steps (read after the timed region, so that no host work
                # between steps is timed)
                st = hp.get_stats()
                launches = st["kernel_launches"] * steps
                for k in acc:
                    for s, v in st["stage_" + k].items():
                        acc[k][s] = v * steps
            if world > 1:
                x = torch.tensor([ms], device="cuda")
                dist.all_reduce(x, op=dist.ReduceOp.MAX)
                ms = float(x)
            return ms, acc, launches, st
        finally:
            hp.restore_config(old)

    # "full": level-batched launches + split-BF16 tensor-core products;
    # "plain": per-merge launches, FP64 products, standard secular guess
    full_cfg = {"batched": 1, "precision": 1}
    from hsspack_gb300 import predictor as _pred
    have_pred = _pred.install()  # committed weights trained by hsspack_gb300/predictor.py
    # DC leaf size and learned start from the project's autotuner (timed
    # outside the measured region)
    from hsspack_gb300 import autotune
    if args.smlsiz > 0:
        tuned, tune_ms = {"smlsiz": args.smlsiz, "predictor": args.predictor}, None
    else:
        tuned, tune_ms = autotune.tune(n, reps=1, base=full_cfg,
                                       predictor=(0, 1, 2, 3) if have_pred else (0, 2, 3))
    full_cfg.update(tuned)
    if args.profile_batch:  # the batch's solves only (ncu launch lists)
        if rank == 0:
            print(json.dumps(profile_batch(args, torch, hp, full_cfg)))
        return
    plain_cfg = {"batched": 0, "precision": 0, "predictor": 0}
    clocks = ClockSampler()
    clocks.start()
    # the headline: no per-stage events, statistics read after the timed region
    ms, _, launches, st = timed(args.steps, args.warmup, False, full_cfg)
    clk = clocks.stop()
    if args.profile_only:  # solves only: the command the ncu launch list wraps
        if rank == 0:
            print(json.dumps({"profile_only": True, "ms_per_step": ms, "launches": launches}))
        return
    # stage times (CUDA events per stage) from a separate, shorter run
    prof_steps = max(1, min(3, args.steps))
    _, acc, _, _ = timed(prof_steps, 1, True, full_cfg)
    # plain GPU merge (per-merge launches), fewer steps
    ms_plain, _, _, _ = timed(max(1, min(3, args.steps)), 1, False, plain_cfg)
    ms_fp64, _, _, _ = timed(max(1, min(3, args.steps)), 1, False,
                             dict(full_cfg, precision=0))
    # the secular start A/B at the tuned leaf size: standard (midpoint), learned
    # MLP, FP32 pre-solve, the pre-solve refined in float-float; time per solve
    # and FP64 evaluations per root
    start_ab = {}
    for pred, name in ((0, "standard"), (1, "learned"), (2, "fp32_presolve"),
                       (3, "fp32_presolve_ff")):
        if pred == 1 and not have_pred:
            continue
        m_ab, _, _, st_ab = timed(max(1, min(3, args.steps)), 1, False,
                                  dict(full_cfg, predictor=pred))
        start_ab[name] = {"ms": m_ab,
                          "evals_per_root": st_ab["secular_iters"] / max(1, st_ab["secular_roots"]),
                          "fallbacks": st_ab["predictor_fallbacks"]}
    acc_chk = check_accuracy(torch, d, e, dw, Z, n)

    # end to end through the Fortran drop-in with ordinary (pageable) host
    # arrays, as a Fortran caller passes them
    work = np.zeros(1)
    iwork = np.zeros(1, dtype=np.int32)
    dn, en = np.empty(n), np.empty(n)
    zn = np.empty((n, n), order="F")
    lw, liw = 1 + 4 * n + n * n, 3 + 5 * n

    def e2e_step():
        dn[:] = d
        en[: n - 1] = e
        info = hp.mdstedc("I", n, dn, en, zn, n, work, lw, iwork, liw)
        assert info == 0, info

    # the same configuration as the device-timed solves
    old_cfg = hp.set_config(**full_cfg)
    try:
        e2e_step()
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        t = time.perf_counter()
        e2e_steps = max(1, min(args.steps, 5))
        for _ in range(e2e_steps):
            e2e_step()
        e2e_s = (time.perf_counter() - t) / e2e_steps
        e2e_st = hp.get_stats()  # the last step's device solve and its copies
        e2e_solve_ms = e2e_st["ms_total"]
    finally:
        hp.restore_config(old_cfg)
    if world > 1:
        x = torch.tensor([e2e_s], device="cuda")
        dist.all_reduce(x, op=dist.ReduceOp.MAX)
        e2e_s = float(x)

    batch = None
    if not args.no_batch:
        batch = run_batch(args, torch, hp, full_cfg, plain_cfg, world, rank, dist)

    extra = None
    if not args.no_extra and rank == 0:
        extra = run_extra_child(full_cfg)

    # dominant stage -> roofline (contract object), plus every stage against
    # the bound that applies to it
    pk = peaks()
    # the FP64 rate is not in the measured-peaks file: measure it here (best of
    # three launches of the FMA-chain kernel)
    pk["fp64_tflops"] = max(hp.fp64_fma_rate()[0] for _ in range(3))
    pk["fp64_source"] = "measured in this run (FP64 FMA chains, hss_fp64_fma_rate)"
    # the dominant kernel: the longest single launch of the solve, the final
    # gather (8.6 GB written once; the secular kernel's 12 launches together
    # take a similar share and appear, FP64-bound, in stage_rooflines); else
    # the longest stage that is one kernel
    single = [s for s in ("final_gather", "secular", "build_S", "lowner", "leaf", "gather",
                          "scatter") if acc["ms"].get(s, 0) > 0]
    top = "final_gather" if "final_gather" in single else max(single, key=lambda s: acc["ms"][s])
    calls = max(1, acc["calls"][top])
    per_launch_ms = acc["ms"][top] / calls
    per_launch_bytes = acc["bytes"][top] / calls
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic_%s.json" % top)
    if os.path.exists(tpath):
        traffic = json.load(open(tpath)).get("bytes_per_launch")
    stage_roof = stage_rooflines(acc, pk)
    if STAGE_BOUND[top] == "hbm":
        achieved = per_launch_bytes / (per_launch_ms * 1e-3) / 1e9
        roof = {"bound": "hbm", "kernel_stage": top, "achieved": achieved,
                "peak": pk["hbm_gbs"], "unit": "GB/s", "frac": achieved / pk["hbm_gbs"],
                "traffic": traffic, "peak_source": pk["source"],
                "algorithmic_bytes_per_launch": per_launch_bytes}
    else:  # an FP64-pipe kernel: its algorithmic flops against the FP64 rate
        per_launch_flops = acc["flops"][top] / calls
        achieved = per_launch_flops / (per_launch_ms * 1e-3) / 1e12
        roof = {"bound": STAGE_BOUND[top], "kernel_stage": top, "achieved": achieved,
                "peak": pk["fp64_tflops"], "unit": "TFLOP/s",
                "frac": achieved / pk["fp64_tflops"], "traffic": traffic,
                "peak_source": pk["fp64_source"], "algorithmic_flops_per_launch": per_launch_flops}
    roof.update({"per_launch_ms": per_launch_ms, "launches_per_step": calls})
    if rank != 0:
        return
    cpu = None
    if not args.no_cpu:
        threads = os.cpu_count() or 1
        t_s = cpu_reference_solve(n, threads)
        cpu = {"value": t_s, "unit": "s", "cores": threads, "kind": "port",
               "sample": "one full n=%d solve of the same matrix" % n}
        # LAPACK's own DSTEDC (the accuracy oracle) on the same matrix and cores
        t2 = cpu_lapack_solve(n, threads)
        cpu["lapack_dstedc"] = {"value": t2, "unit": "s", "cores": threads,
                                "sample": "one full n=%d DSTEDC('I') of the same matrix" % n}
    total_ms = sum(acc["ms"].values())
    line = {
        "metric": METRIC, "value": ms / 1000.0, "unit": "s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "tridiagonal DC eigensolve n=%d, D,E iid U[-1,1] seed 0, COMPZ='I'"
                   % n, "n": n, "mode": "batched levels, split-BF16 tensor-core products" +
                           ("", ", learned secular start", ", FP32 pre-solved secular start")
                           [int(full_cfg.get("predictor", 0))],
                   "smlsiz": full_cfg.get("smlsiz"), "autotune_ms": tune_ms,
                   "l2": "no flush: the 8.6 GB eigenvector matrix exceeds L2",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        # bytes the call copied: D, E in; eigenvalues and either Z or only the
        # rows each column holds data on (the call zero-fills Z on the host)
        "e2e": {"value": e2e_s, "unit": "s", "h2d_bytes_per_step": e2e_st["host_h2d_bytes"],
                "d2h_bytes_per_step": e2e_st["host_d2h_bytes"],
                # the library's event time of the solve inside a step; the
                # rest is the host<->device copies and the call's host work
                "device_solve_s": e2e_solve_ms / 1000.0},
        "gpu_launches": int(launches),
        "roofline": roof,
        "cpu_baseline": cpu,
        "clocks": clk,
        "plain_gpu_s": ms_plain / 1000.0,
        "batched_fp64_s": ms_fp64 / 1000.0,
        "full_vs_plain": ms_plain / ms,
        "full_vs_batched_fp64": ms_fp64 / ms,
        "secular_start_ab": start_ab,
        "accuracy": acc_chk,
        "batch": batch,
        "stage_rooflines": stage_roof,
        "fp64_peak_tflops": pk["fp64_tflops"],
        "other_workloads": extra,
        "stages_ms_per_step": {k: v / prof_steps for k, v in acc["ms"].items() if v > 0},
        "profiled_stage_share": {k: v / total_ms for k, v in acc["ms"].items() if v > 0},
        "stats": {k: st[k] for k in ("n_levels", "n_merges", "n_hss_merges", "n_dense_merges",
                                     "max_k", "max_rank", "total_k", "secular_iters",
                                     "secular_roots", "predictor_fallbacks")},
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=N_DEFAULT)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the 512-problem batch figures")
    ap.add_argument("--no-extra", action="store_true", help="skip the other configurations")
    ap.add_argument("--extra-only", action="store_true",
                    help="only the other configurations' figures (one JSON dict; the child "
                         "process of a full run)")
    ap.add_argument("--extra-cfg", default="{}", help="the library configuration for --extra-only")
    ap.add_argument("--smlsiz", type=int, default=0,
                    help="fixed DC leaf size instead of the autotuner (profiling runs)")
    ap.add_argument("--predictor", type=int, default=2, choices=[0, 1, 2],
                    help="secular start when --smlsiz bypasses the autotuner (0 standard, "
                         "1 learned, 2 FP32 pre-solve)")
    ap.add_argument("--profile-batch", action="store_true",
                    help="run only the batch's warmup + timed batched solves (ncu launch lists)")
    ap.add_argument("--profile-only", action="store_true",
                    help="run only the warmup + timed solves (for ncu launch lists)")
    args = ap.parse_args()
    if args.extra_only:
        import torch
        import hsspack_gb300 as hp
        torch.cuda.set_device(0)
        print(json.dumps(run_extra(torch, hp, json.loads(args.extra_cfg))), flush=True)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
