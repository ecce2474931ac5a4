"""Multi-GPU form of the permutation loop: replicas over disjoint ranges of the
seeded permutation stream, one process per GPU.

The reference parallelises the same loop by launching independent randomise
jobs over permutation ranges (-r START STOP, GNU parallel / HTCondor:
tfce_mediation/tmanalysis/vertex_tfce_multiple_regression_randomise.py:49-60,
tm_multisurface/tm_mmr_rand_low_ram_parallel.py) and concatenating their CSVs.
Here every rank runs its contiguous range of the RandomState(seed + i) stream
on its own GPU; the only exchange is the per-permutation maxima (a few KB),
gathered on rank 0 in rank order, so the merged null distribution is the one a
single process produces over the whole range.  There is no data-path
collective.  With torch.distributed not initialised everything runs as one
rank."""
from __future__ import annotations

import numpy as np


def _dist():
    try:
        import torch.distributed as dist
    except ImportError:  # pragma: no cover - torch is a dependency
        return None
    return dist if dist.is_available() and dist.is_initialized() else None


def world():
    """(world_size, rank) of the initialised process group, else (1, 0)."""
    d = _dist()
    return (d.get_world_size(), d.get_rank()) if d else (1, 0)


def shard_range(n_perm, world_size, rank, start=0):
    """Contiguous [lo, hi) of permutations start .. start+n_perm for one rank:
    ceil(n_perm / world_size) each, the last ranks possibly shorter or empty."""
    if world_size < 1 or not 0 <= rank < world_size:
        raise ValueError("need 0 <= rank < world_size")
    per = -(-int(n_perm) // world_size)
    lo = start + min(rank * per, n_perm)
    hi = start + min((rank + 1) * per, n_perm)
    return lo, hi


def gather_null(local, dst=0):
    """Per-rank maxima (rows = permutations) -> their concatenation in rank
    order on rank dst (None elsewhere); the local array when not distributed."""
    d = _dist()
    local = np.asarray(local)
    if d is None:
        return local
    parts = [None] * d.get_world_size()
    d.all_gather_object(parts, local)
    return np.concatenate(parts) if d.get_rank() == dst else None


def max_over_ranks(value):
    """The maximum of a host scalar over all ranks (the whole-job time of a
    step is the slowest rank's)."""
    d = _dist()
    if d is None:
        return float(value)
    import torch
    backend = d.get_backend()
    dev = "cuda" if backend == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    d.all_reduce(t, op=d.ReduceOp.MAX)
    return float(t.item())


def run_sharded(run_range, n_perm, start=0, dst=0):
    """Run permutations [start, start + n_perm) across the ranks:
    run_range(lo, hi) -> maxima of permutations lo .. hi-1 on this rank (e.g.
    lambda lo, hi: engine.run(seed=seed, start=lo, stop=hi)); returns the
    merged maxima on rank dst, None on the other ranks."""
    ws, rank = world()
    lo, hi = shard_range(n_perm, ws, rank, start)
    local = run_range(lo, hi)
    return gather_null(local, dst)
