"""Sharding independent tridiagonal problems over ranks (host logic, CPU).

The partition is checked for coverage and balance; the gather runs as two
`gloo` ranks on the CPU, each solving its share with a CPU stand-in for the
batched GPU solve (SciPy's LAPACK tridiagonal eigensolver), and rank 0's
gathered results must equal a direct solve of every problem in input order."""
import os
import socket
import tempfile

import numpy as np
import pytest

from hsspack_gb300 import shard


def _problems(count=24, seed=2):
    rng = np.random.default_rng(seed)
    sizes = np.round(np.exp(rng.uniform(np.log(16), np.log(200), count))).astype(int)
    return [(rng.uniform(-1, 1, n), rng.uniform(-1, 1, n - 1)) for n in sizes]


def _cpu_solve(problems):
    from scipy.linalg import eigh_tridiagonal
    return [eigh_tridiagonal(d, e) for d, e in problems]


@pytest.mark.parametrize("world", [1, 2, 3, 8])
def test_partition_covers_and_balances(world):
    rng = np.random.default_rng(2)
    sizes = np.round(np.exp(rng.uniform(np.log(256), np.log(4096), 512))).astype(int)
    parts = shard.partition(sizes, world)
    allidx = np.sort(np.concatenate(parts))
    assert np.array_equal(allidx, np.arange(len(sizes)))
    costs = shard.shard_costs(sizes, parts)
    # greedy LPT: no rank exceeds the mean by more than the largest single cost
    assert costs.max() <= costs.sum() / world + (sizes.astype(float) ** 3).max() + 1e-6
    assert all(np.all(np.diff(p) > 0) for p in parts)


def test_partition_deterministic_and_tie_order():
    parts = shard.partition([10, 10, 10, 10], 2)
    assert [p.tolist() for p in parts] == [[0, 2], [1, 3]]
    assert [p.tolist() for p in shard.partition([5, 7], 4)] == [[1], [0], [], []]


def _worker(rank, world, port, outdir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        probs = _problems()
        solved = []

        def local(ps):
            solved.extend(len(d) for d, _ in ps)
            return _cpu_solve(ps)

        out = shard.solve_sharded(probs, solve_local=local)
        np.save(os.path.join(outdir, "solved%d.npy" % rank), np.array(solved))
        if rank == 0:
            np.savez(os.path.join(outdir, "out.npz"),
                     **{"w%d" % i: w for i, (w, _) in enumerate(out)},
                     **{"q%d" % i: q for i, (_, q) in enumerate(out)})
        else:
            assert out is None
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_gather_in_input_order():
    import torch.multiprocessing as mp
    probs = _problems()
    ref = _cpu_solve(probs)
    with tempfile.TemporaryDirectory() as td:
        mp.start_processes(_worker, args=(2, _free_port(), td), nprocs=2, join=True,
                           start_method="spawn")
        got = np.load(os.path.join(td, "out.npz"))
        s0 = np.load(os.path.join(td, "solved0.npy"))
        s1 = np.load(os.path.join(td, "solved1.npy"))
    for i, (w, q) in enumerate(ref):
        assert np.array_equal(got["w%d" % i], w)
        assert np.array_equal(got["q%d" % i], q)
    # each rank solved exactly its share, and the shares are disjoint and complete
    parts = shard.partition([len(d) for d, _ in probs], 2)
    sizes = np.array([len(d) for d, _ in probs])
    assert sorted(s0.tolist()) == sorted(sizes[parts[0]].tolist())
    assert sorted(s1.tolist()) == sorted(sizes[parts[1]].tolist())
    assert len(s0) + len(s1) == len(probs) and len(s0) > 0 and len(s1) > 0
