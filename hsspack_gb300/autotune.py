"""Autotuner for the divide-and-conquer configuration.

Chooses, per problem-size bucket (powers of two), the DC leaf size SMLSIZ, the
secular start (standard, learned, FP32 pre-solve or the pre-solve refined in
float-float) and, with split-BF16
products, whether products of 64-127 rows go to the tensor cores, by timing the
candidate settings on a seeded random tridiagonal of that size (device time
from the library's CUDA events).  Results are cached in ``_lib/autotune.json``
next to the library and applied with :func:`apply`.
"""
import json
import os

import numpy as np

from . import build as _build

CACHE = os.path.join(os.path.dirname(_build.LIB), "autotune.json")
SMLSIZ_CANDIDATES = (6, 12, 16, 25)


def _bucket(n):
    return str(1 << max(0, int(np.ceil(np.log2(max(n, 1))))))


def load_cache():
    if os.path.exists(CACHE):
        try:
            return json.load(open(CACHE))
        except (OSError, ValueError):
            return {}
    return {}


def tune(n, candidates=SMLSIZ_CANDIDATES, reps=2, seed=0, base=None, predictor=(0,)):
    """Time MDSTEDC('I') at size n for each DC leaf size and secular start
    (predictor 0 standard, 1 learned, 2 FP32 pre-solve, 3 FP32 pre-solve
    refined in float-float); return the best config dict (and all timings,
    keyed "smlsiz", "smlsiz+learned", "smlsiz+fp32" or "smlsiz+ff") and cache
    it under the size bucket."""
    import torch
    import hsspack_gb300 as hp
    rng = np.random.default_rng(seed)
    d, e = rng.uniform(-1, 1, n), rng.uniform(-1, 1, n - 1)
    d0 = torch.tensor(d, dtype=torch.float64, device="cuda")
    e0 = torch.tensor(e, dtype=torch.float64, device="cuda")
    dw, ew = d0.clone(), e0.clone()
    z = torch.empty(n * n, dtype=torch.float64, device="cuda")
    results, cfgs = {}, {}
    for pred in predictor:
        for sml in candidates:
            key = "%d%s" % (sml, ("", "+learned", "+fp32", "+ff")[int(pred)])
            cfg = dict(base or {}, smlsiz=int(sml), predictor=int(pred))
            old = hp.set_config(**cfg)
            try:
                best = float("inf")
                for _ in range(reps + 1):
                    dw.copy_(d0)
                    ew.copy_(e0)
                    hp.mdstedc_dev(dw, ew, z)
                    best = min(best, hp.get_stats()["ms_total"])
                results[key] = best
                cfgs[key] = {"smlsiz": int(sml), "predictor": int(pred)}
            finally:
                hp.restore_config(old)
    key = min(results, key=results.get)
    if int((base or {}).get("precision", 0)) == 1:
        # the winner once more with the products of 64-127 rows on the tensor
        # cores (128-row tiles) instead of the FP64 element kernel
        k64 = key + "+m64"
        cfg = dict(base, **cfgs[key], split_min_m=64)
        old = hp.set_config(**cfg)
        try:
            best = float("inf")
            for _ in range(reps + 1):
                dw.copy_(d0)
                ew.copy_(e0)
                hp.mdstedc_dev(dw, ew, z)
                best = min(best, hp.get_stats()["ms_total"])
            results[k64] = best
            cfgs[k64] = dict(cfgs[key], split_min_m=64)
        finally:
            hp.restore_config(old)
        if results[k64] < results[key]:
            key = k64
    cache = load_cache()
    cache[_bucket(n)] = dict(cfgs[key], ms=results)
    try:
        os.makedirs(os.path.dirname(CACHE), exist_ok=True)
        json.dump(cache, open(CACHE, "w"), indent=1)
    except OSError:
        pass
    return dict(cfgs[key]), results


def lookup(n):
    ent = load_cache().get(_bucket(n))
    if not ent:
        return None
    return {k: ent[k] for k in ("smlsiz", "predictor", "split_min_m") if k in ent}


def apply(n):
    """Set the cached tuned configuration for size n (if any); returns the
    previous configuration for restore_config()."""
    import hsspack_gb300 as hp
    cfg = lookup(n)
    return hp.set_config(**cfg) if cfg else hp.get_config()
