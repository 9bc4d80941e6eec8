"""Independent tridiagonal problems sharded across ranks (one GPU per rank).

The reference solves the independent subproblems of a DC level, and the
independent blocks a split matrix falls into, one after another
(SRC/mdlaed0.f90:298-337, SRC/mdstedc.f90:305-389).  Many independent problems
need no exchange at all: each rank takes a share, solves it with the batched
device entry (``hss_mdstedc_batch_dev``) on its own GPU, and only the results
travel, to rank 0, once.

* :func:`partition` -- greedy longest-processing-time split by the DC cost
  model n^3 (the eigenvector updates of a size-n problem cost O(n^3) at worst;
  with the heavy deflation of random tridiagonals the solve is closer to n^2 log
  n, and the greedy order is the same for any increasing cost): problems in
  decreasing cost, each to the rank with the least total so far.  Deterministic:
  ties go to the lower rank, equal costs keep the input order.
* :func:`solve_sharded` -- every rank solves its share with a caller-given
  local solver (the batched GPU solve by default) and rank 0 gathers
  eigenvalues (and, if asked, eigenvectors) back into input order.
"""
import numpy as np


def partition(sizes, world, cost=None):
    """Split problem indices over `world` ranks; returns a list of index
    arrays (each ascending) whose costs are balanced greedily."""
    sizes = np.asarray(sizes, dtype=np.int64)
    if world < 1:
        raise ValueError("world must be >= 1")
    c = sizes.astype(np.float64) ** 3 if cost is None else np.asarray(cost, dtype=np.float64)
    order = np.argsort(-c, kind="stable")
    load = np.zeros(world)
    owner = np.empty(len(sizes), dtype=np.int64)
    for p in order:
        r = int(np.argmin(load))  # first minimum: the lowest rank wins ties
        owner[p] = r
        load[r] += c[p]
    return [np.flatnonzero(owner == r) for r in range(world)]


def shard_costs(sizes, parts, cost=None):
    """Total cost per rank of a partition (for checking the balance)."""
    sizes = np.asarray(sizes, dtype=np.int64)
    c = sizes.astype(np.float64) ** 3 if cost is None else np.asarray(cost, dtype=np.float64)
    return np.array([c[idx].sum() for idx in parts])


def _gpu_local(problems, stream=None):
    from . import eigh_tridiagonal_batch
    if not problems:
        return []
    return eigh_tridiagonal_batch(problems, stream)


def solve_sharded(problems, solve_local=None, group=None, want_vectors=True):
    """Solve a list of (d, e) tridiagonal problems over the ranks of the
    initialised default process group (or `group`).

    Every rank must pass the same `problems` list (it is cheap: only the
    diagonals); each solves its share ``partition(sizes, world)[rank]`` with
    ``solve_local(list_of_(d, e)) -> list_of_(w, Q)`` (default: the batched GPU
    solve on the rank's current device).  Rank 0 returns the results of all
    problems in input order -- ``(w, Q)`` pairs, or ``w`` arrays alone when
    ``want_vectors`` is false -- and the other ranks return None.  A single
    process (no process group) solves everything itself."""
    import torch.distributed as dist

    solve_local = solve_local or _gpu_local
    if not (dist.is_available() and dist.is_initialized()):
        out = solve_local(list(problems))
        return out if want_vectors else [w for w, _ in out]
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    sizes = [len(d) for d, _ in problems]
    mine = partition(sizes, world)[rank]
    local = solve_local([problems[int(p)] for p in mine])
    payload = [(int(p), w, Q if want_vectors else None) for p, (w, Q) in zip(mine, local)]
    gathered = [None] * world if rank == 0 else None
    dist.gather_object(payload, gathered, dst=0, group=group)
    if rank != 0:
        return None
    out = [None] * len(problems)
    for part in gathered:
        for p, w, Q in part:
            out[p] = (w, Q) if want_vectors else w
    missing = [p for p, v in enumerate(out) if v is None]
    if missing:
        raise RuntimeError("problems %s were solved by no rank" % missing[:8])
    return out
