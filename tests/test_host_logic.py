"""Host-side logic that needs no GPU: the packed layout of many problems per
call, the autotuner's cache, and the benchmark's seeded batch workload."""
import json
import os
import sys

import numpy as np

import hsspack_gb300 as hp
from hsspack_gb300 import autotune

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_batch_offsets_and_packing():
    # problem p occupies positions o[p]..o[p+1]-1 of d and e (its last
    # off-diagonal slot stays 0, so no coupling crosses problems) and the
    # n_p^2 entries oz[p]..oz[p+1]-1 of z
    probs = [(np.array([1.0, 2.0, 3.0]), np.array([0.5, 0.25])),
             (np.array([4.0]), np.array([])),
             (np.array([5.0, 6.0, 7.0, 8.0]), np.array([0.1, 0.2, 0.3]))]
    sizes, D, E = hp.pack_batch(probs)
    o, oz = hp.batch_offsets(sizes)
    assert list(sizes) == [3, 1, 4]
    assert list(o) == [0, 3, 4, 8] and list(oz) == [0, 9, 10, 26]
    assert np.array_equal(D, [1, 2, 3, 4, 5, 6, 7, 8])
    assert np.array_equal(E, [0.5, 0.25, 0, 0, 0.1, 0.2, 0.3, 0])
    for p in range(3):
        assert E[o[p + 1] - 1] == 0.0


def test_autotune_cache_roundtrip(tmp_path, monkeypatch):
    # results are cached per power-of-two size bucket and looked up by size
    cache = tmp_path / "autotune.json"
    monkeypatch.setattr(autotune, "CACHE", str(cache))
    assert autotune.lookup(30000) is None
    cache.write_text(json.dumps({"32768": {"smlsiz": 12, "predictor": 2,
                                           "ms": {"12+fp32": 7.7, "12": 8.2}}}))
    assert autotune.lookup(30000) == {"smlsiz": 12, "predictor": 2}
    assert autotune.lookup(32768) == {"smlsiz": 12, "predictor": 2}
    assert autotune.lookup(40000) is None
    assert autotune._bucket(1) == "1" and autotune._bucket(4097) == "8192"
    cache.write_text("not json")
    assert autotune.load_cache() == {}


def test_benchmark_batch_is_seeded():
    # the batch workload: 512 tridiagonals, n log-uniform in [256, 4096],
    # the same problems on every call
    sys.path.insert(0, ROOT)
    import bench
    s1, p1 = bench.batch_inputs()
    s2, p2 = bench.batch_inputs()
    assert len(s1) == 512 and min(s1) >= 256 and max(s1) <= 4096
    assert np.array_equal(s1, s2)
    assert all(np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]) for a, b in zip(p1, p2))
    assert all(len(d) == n and len(e) == n - 1 for (d, e), n in zip(p1, s1))
