"""Multi-GPU sharding of the permutation loop, on the CPU: disjoint contiguous
ranges of the seeded stream per rank, the maxima gathered on rank 0 in rank
order, the slowest rank's time -- with world_size-2 gloo process groups (the
per-rank work is the oracle pipeline, standing in for a GPU engine)."""
import os
import socket
import tempfile

import numpy as np
import pytest

from tfce_mediation_gb300 import shard


def test_shard_range_partitions_the_stream():
    for n, ws in [(10, 2), (7, 3), (2, 4), (0, 2), (1000, 8)]:
        ranges = [shard.shard_range(n, ws, r, start=5) for r in range(ws)]
        covered = [i for lo, hi in ranges for i in range(lo, hi)]
        assert covered == list(range(5, 5 + n))
    with pytest.raises(ValueError):
        shard.shard_range(5, 2, 2)


def test_single_process_fallbacks():
    assert shard.world() == (1, 0)
    a = np.arange(6).reshape(3, 2)
    np.testing.assert_array_equal(shard.gather_null(a), a)
    assert shard.max_over_ranks(2.5) == 2.5
    got = shard.run_sharded(lambda lo, hi: np.arange(lo, hi), 4, start=3)
    np.testing.assert_array_equal(got, [3, 4, 5, 6])


def _study():
    from tfce_mediation_gb300 import adjacency as A
    from tfce_mediation_gb300 import synth
    v, f = synth.icosphere(2)
    off, idx = A.mesh_csr(f, v.shape[0])
    rng = np.random.default_rng(3)
    n = 20
    x = rng.standard_normal(n)
    Y = (rng.standard_normal((n, v.shape[0])) + 0.8 * x[:, None]).astype(np.float32)
    return off, idx, Y, np.column_stack([np.ones(n), x])


def _oracle_null(lo, hi):
    from oracle import oracle
    from tfce_mediation_gb300.engine import permutations
    off, idx, Y, X = _study()
    out = np.zeros((hi - lo, 2), np.float32)
    for r, p in enumerate(permutations(X.shape[0], 11, lo, hi)):
        t = oracle.tval_fp64(X[p], Y)[1].astype(np.float32)
        for si, s in enumerate((1.0, -1.0)):
            out[r, si] = oracle.tfce_max_batch(off, idx, t, 2.0, 1.0, sign=s)[0]
    return out


def _worker(rank, world_size, port, out_dir, n_perm):
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world_size)
    try:
        null = shard.run_sharded(_oracle_null, n_perm)
        slowest = shard.max_over_ranks(1.5 + rank)
        lo, hi = shard.shard_range(n_perm, world_size, rank)
        np.savez(os.path.join(out_dir, f"rank{rank}.npz"), null=np.zeros(0) if null is None else null,
                 is_none=null is None, slowest=slowest, lo=lo, hi=hi)
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.parametrize("n_perm", [7, 1])
def test_gloo_two_ranks_merge_equals_one_process(n_perm):
    import torch.multiprocessing as mp
    with tempfile.TemporaryDirectory() as d:
        mp.start_processes(_worker, args=(2, _free_port(), d, n_perm), nprocs=2, start_method="spawn", join=True)
        r0, r1 = np.load(os.path.join(d, "rank0.npz")), np.load(os.path.join(d, "rank1.npz"))
        assert not bool(r0["is_none"]) and bool(r1["is_none"])
        np.testing.assert_array_equal(r0["null"], _oracle_null(0, n_perm))
        assert float(r0["slowest"]) == float(r1["slowest"]) == 2.5
        assert (int(r0["lo"]), int(r0["hi"]), int(r1["lo"]), int(r1["hi"])) == \
            (0, -(-n_perm // 2), -(-n_perm // 2), n_perm)
