"""The allocation-free sweep entry point, called through the C-ABI.

``tfce_sweep_batch_noalloc`` serves callers that cannot allocate device
memory while they sweep (device memory reserved up front by another
allocator, fixed-footprint real-time loops, hosts that cannot take the
synchronisation cudaFree implies): its scratch is a static device array in
the library.  These tests check that two calls in a row give exactly what the
allocating entry point (``tfce_sweep_batch`` through an adjacency handle)
gives, on the same inputs, and that sizes beyond the static scratch are
refused.  The file sorts last so a run that stops at the first failure has
already run every other test; it builds all its own inputs, so it also passes
alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

from tfce_mediation_gb300 import _lib
from tfce_mediation_gb300 import adjacency as A
from tfce_mediation_gb300 import synth

pytestmark = pytest.mark.gpu


def _maps(offsets, indices, V, n_maps, seed):
    S = synth.smoothing_matrix(offsets, indices)
    rng = np.random.default_rng(seed)
    m = rng.standard_normal((V, n_maps)).astype(np.float32)
    for _ in range(4):
        m = (S @ m).astype(np.float32)
    return np.ascontiguousarray((3.0 * m.T).astype(np.float32))


def _noalloc(torch, off_d, idx_d, V, D, seg_d, n_seg, vmax, H_d, E_d, stats_d, n_maps, signs):
    lib = _lib.load()
    out = torch.full((n_maps, signs, n_seg), float("nan"), device="cuda")
    rc = lib.tfce_sweep_batch_noalloc(off_d.data_ptr(), idx_d.data_ptr(), V, D, seg_d.data_ptr(), n_seg,
                                      vmax, H_d.data_ptr(), E_d.data_ptr(), stats_d.data_ptr(), V,
                                      n_maps, signs, None, 1, out.data_ptr(),
                                      torch.cuda.current_stream().cuda_stream)
    _lib.check(rc)
    return out.cpu().numpy()


def _reference_path(torch, off, idx, seg, H, E, stats, signs):
    adj = A.AdjacencySet((off, idx), H, E, seg)
    n_maps = stats.shape[0]
    out = torch.empty((n_maps, signs, adj.n_seg), device="cuda")
    d = torch.from_numpy(stats).cuda()
    adj.sweep_batch(d.data_ptr(), stats.shape[1], n_maps, signs, None, 1, out.data_ptr())
    adj.status()
    return out.cpu().numpy()


def test_noalloc_matches_allocating_sweep_twice():
    import torch
    v, f = synth.icosphere(4)
    o1, i1 = A.mesh_csr(f, v.shape[0])
    off, idx, seg = A.concat_csr([(o1, i1), (o1, i1)])
    V, D = off.shape[0] - 1, int(off[-1])
    H = np.array([2.0, 2.0], np.float32)
    E = np.array([1.0, 0.5], np.float32)
    dev = {k: torch.from_numpy(np.ascontiguousarray(a)).cuda()
           for k, a in (("off", off), ("idx", idx), ("seg", seg), ("H", H), ("E", E))}
    vmax = int(np.diff(seg).max())
    for call, seed in enumerate((11, 12)):  # two calls in a row, different maps
        stats = _maps(off, idx, V, 10, seed)
        stats[:, :40] = 0.0  # masked vertices scattered as zeros
        got = _noalloc(torch, dev["off"], dev["idx"], V, D, dev["seg"], 2, vmax, dev["H"], dev["E"],
                       torch.from_numpy(stats).cuda(), stats.shape[0], 2)
        ref = _reference_path(torch, off, idx, seg, H, E, stats, 2)
        np.testing.assert_array_equal(got, ref, err_msg=f"call {call}")


def test_noalloc_asymmetric_lists_match():
    """Lists with one-way entries and self entries (the multimodal voxel
    builder): the allocation-free path applies the insertion-order rule to all
    entries, the handle path to the flagged ones -- same result."""
    import torch
    mask = np.zeros((10, 9, 8), bool)
    mask[1:9, 1:8, 1:7] = True
    mask[0, 0, 0] = True
    off, idx = A.voxel_csr(mask, 26, "mmr")
    V, D = off.shape[0] - 1, int(off[-1])
    seg = np.array([0, V], np.int64)
    H = np.array([2.0], np.float32)
    E = np.array([0.5], np.float32)
    rng = np.random.default_rng(5)
    stats = (rng.standard_normal((6, V)) + 0.3).astype(np.float32)
    tor = {k: torch.from_numpy(np.ascontiguousarray(a)).cuda()
           for k, a in (("off", off), ("idx", idx), ("seg", seg), ("H", H), ("E", E))}
    for _ in range(2):
        got = _noalloc(torch, tor["off"], tor["idx"], V, D, tor["seg"], 1, V, tor["H"], tor["E"],
                       torch.from_numpy(stats).cuda(), stats.shape[0], 2)
        ref = _reference_path(torch, off, idx, seg, H, E, stats, 2)
        np.testing.assert_array_equal(got, ref)


def test_noalloc_refuses_segments_beyond_scratch():
    lib = _lib.load()
    rc = lib.tfce_sweep_batch_noalloc(1, 1, 10, 0, 1, 1, 3_000_000, 1, 1, 1, 10, 1, 2, None, 0, 1, None)
    assert rc == _lib.TFCE_ERANGE
    assert b"static scratch" in lib.tfce_last_error()


def _two_segment_case():
    v, f = synth.icosphere(3)
    o1, i1 = A.mesh_csr(f, v.shape[0])
    off, idx, seg = A.concat_csr([(o1, i1), (o1, i1)])
    V, D = off.shape[0] - 1, int(off[-1])
    H = np.array([2.0, 2.0], np.float32)
    E = np.array([1.0, 1.0], np.float32)
    stats = _maps(off, idx, V, 4, 21)
    return off, idx, seg, V, D, H, E, stats


def test_noalloc_rejects_a_segment_longer_than_declared():
    """max_segment_vertices below a segment's real length: the call returns
    TFCE_EINVAL and the items of that segment report 0; the kernel skips
    them without touching the workspace beyond the declared size."""
    import torch
    off, idx, seg, V, D, H, E, stats = _two_segment_case()
    seg = np.array([0, 100, V], np.int64)  # segment 1 is longer than declared
    lib = _lib.load()
    out = torch.full((4, 2, 2), float("nan"), device="cuda")
    # segment 0 = vertices [0, 100) of the first mesh: drop the entries that
    # cross between [0, 100) and the rest, then rebuild the CSR
    rows = np.repeat(np.arange(V), np.diff(off))
    ok = (rows < 100) == (idx < 100)
    o2 = np.zeros(V + 1, np.int64)
    np.add.at(o2, rows[ok] + 1, 1)
    o2 = np.cumsum(o2)
    i2 = idx[ok].astype(np.int32)
    dev = {k: torch.from_numpy(np.ascontiguousarray(a)).cuda()
           for k, a in (("off", o2), ("idx", i2), ("seg", seg), ("H", H), ("E", E))}
    rc = lib.tfce_sweep_batch_noalloc(dev["off"].data_ptr(), dev["idx"].data_ptr(), V, int(o2[-1]),
                                      dev["seg"].data_ptr(), 2, 200, dev["H"].data_ptr(), dev["E"].data_ptr(),
                                      torch.from_numpy(stats).cuda().data_ptr(), V, 4, 2, None, 1,
                                      out.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert rc == _lib.TFCE_EINVAL
    got = out.cpu().numpy()
    assert (got[:, :, 1] == 0).all()
    ref = _reference_path(torch, o2, i2, seg, H, E, stats, 2)
    np.testing.assert_array_equal(got[:, :, 0], ref[:, :, 0])


def test_noalloc_rejects_entries_outside_their_segment():
    """A negative list entry and an entry pointing into the other segment:
    TFCE_EINVAL, the entries are skipped (never read through), and the items
    of the segment without bad entries still equal the allocating sweep."""
    import torch
    off, idx, seg, V, D, H, E, stats = _two_segment_case()
    bad = idx.copy()
    Vh = V // 2
    e_neg = int(off[Vh + 3])          # first entry of vertex Vh+3 (segment 1)
    e_cross = int(off[Vh + 10]) + 1   # second entry of vertex Vh+10 (segment 1)
    bad[e_neg] = np.int32(-2147483643)  # bit 31 set; masked it would read as vertex 5
    bad[e_cross] = 7                    # a vertex of segment 0
    dev = {k: torch.from_numpy(np.ascontiguousarray(a)).cuda()
           for k, a in (("off", off), ("idx", bad), ("seg", seg), ("H", H), ("E", E))}
    lib = _lib.load()
    for _ in range(2):
        out = torch.full((4, 2, 2), float("nan"), device="cuda")
        rc = lib.tfce_sweep_batch_noalloc(dev["off"].data_ptr(), dev["idx"].data_ptr(), V, D,
                                          dev["seg"].data_ptr(), 2, int(np.diff(seg).max()), dev["H"].data_ptr(),
                                          dev["E"].data_ptr(), torch.from_numpy(stats).cuda().data_ptr(), V, 4, 2,
                                          None, 1, out.data_ptr(), torch.cuda.current_stream().cuda_stream)
        assert rc == _lib.TFCE_EINVAL
        assert b"outside" in lib.tfce_last_error()
        ref = _reference_path(torch, off, idx, seg, H, E, stats, 2)
        np.testing.assert_array_equal(out.cpu().numpy()[:, :, 0], ref[:, :, 0])
