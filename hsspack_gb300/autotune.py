"""Autotuner for the divide-and-conquer configuration.

Chooses, per problem-size bucket (powers of two), the DC leaf size SMLSIZ and
the K threshold between dense and HSS merges by timing candidate settings on a
seeded random tridiagonal of that size (device time from the library's CUDA
events).  Results are cached in ``_lib/autotune.json`` next to the library and
applied with :func:`apply`.
"""
import json
import os

import numpy as np

from . import build as _build

CACHE = os.path.join(os.path.dirname(_build.LIB), "autotune.json")
SMLSIZ_CANDIDATES = (6, 12, 25)


def _bucket(n):
    return str(1 << max(0, int(np.ceil(np.log2(max(n, 1))))))


def load_cache():
    if os.path.exists(CACHE):
        try:
            return json.load(open(CACHE))
        except (OSError, ValueError):
            return {}
    return {}


def tune(n, candidates=SMLSIZ_CANDIDATES, reps=2, seed=0, base=None):
    """Time MDSTEDC('I') at size n for each DC leaf size; return the best
    config dict and cache it under the size bucket."""
    import torch
    import hsspack_gb300 as hp
    rng = np.random.default_rng(seed)
    d, e = rng.uniform(-1, 1, n), rng.uniform(-1, 1, n - 1)
    d0 = torch.tensor(d, dtype=torch.float64, device="cuda")
    e0 = torch.tensor(e, dtype=torch.float64, device="cuda")
    dw, ew = d0.clone(), e0.clone()
    z = torch.empty(n * n, dtype=torch.float64, device="cuda")
    results = {}
    for sml in candidates:
        old = hp.set_config(smlsiz=int(sml), **(base or {}))
        try:
            best = float("inf")
            for _ in range(reps + 1):
                dw.copy_(d0)
                ew.copy_(e0)
                hp.mdstedc_dev(dw, ew, z)
                best = min(best, hp.get_stats()["ms_total"])
            results[int(sml)] = best
        finally:
            hp.restore_config(old)
    sml = min(results, key=results.get)
    cache = load_cache()
    cache[_bucket(n)] = {"smlsiz": sml, "ms": results}
    try:
        os.makedirs(os.path.dirname(CACHE), exist_ok=True)
        json.dump(cache, open(CACHE, "w"), indent=1)
    except OSError:
        pass
    return {"smlsiz": sml}, results


def lookup(n):
    ent = load_cache().get(_bucket(n))
    return {"smlsiz": ent["smlsiz"]} if ent else None


def apply(n):
    """Set the cached tuned configuration for size n (if any); returns the
    previous configuration for restore_config()."""
    import hsspack_gb300 as hp
    cfg = lookup(n)
    return hp.set_config(**cfg) if cfg else hp.get_config()
