"""Exact geodesic neighbour lists on the GPU (csrc/geodesic.cu through the
C-ABI) against the reference's own outputs (golden vectors made by
tests/golden/make_geodesic_golden.py from the reference's adjacency.pyx over
lib/geodesic) and against the oracle (oracle/geodesic_oracle.c, pinned to
those vectors in tests/test_geodesic.py).  Bar: the same (i, j) pairs, and
distances within 1e-12 relative (double precision throughout)."""
import os

import numpy as np
import pytest

from oracle import oracle
from tfce_mediation_gb300 import geodesic, synth

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "geodesic_vectors.npz")
RTOL = 1e-12


@pytest.fixture(scope="module")
def geo():
    return np.load(GOLDEN)


def _same(got, ref):
    np.testing.assert_array_equal(got[0], ref[0])
    np.testing.assert_array_equal(got[1], ref[1])
    np.testing.assert_allclose(got[2], ref[2], rtol=RTOL, atol=0)


@pytest.mark.parametrize("name", ["sphere", "cap", "bumpy"])
def test_lists_match_reference_golden(geo, name):
    v, f = geo[f"{name}_v"], geo[f"{name}_f"]
    m = geodesic.GeodesicMesh(v, f)
    got = m.lists(float(geo[f"{name}_threshold"]), True, 0, int(geo[f"{name}_n_src"]))
    _same(got, (geo[f"{name}_i"], geo[f"{name}_j"], geo[f"{name}_d"]))


def test_compute_dropin_equals_reference_compute(geo):
    """adjacency.compute: the reference's own per-threshold lists, exactly."""
    from tfce_mediation_gb300 import adjacency
    v, f = geo["sphere_v"], geo["sphere_f"]
    thr = geo["compute_thresholds"]
    lists = adjacency.compute(v, f, thr)
    for k in range(thr.shape[0]):
        off, idx = geo[f"compute_{k}_off"], geo[f"compute_{k}_idx"]
        assert [len(x) for x in lists[k]] == np.diff(off).tolist()
        assert [y for x in lists[k] for y in x] == idx.tolist()


def test_compute_distance_parallel_dropin(geo):
    """adjacency.compute_distance_parallel(v, f, threshold, i): the reference's
    [[i, j, distance], ...] rows for single sources."""
    v, f, thr = geo["cap_v"], geo["cap_f"], float(geo["cap_threshold"])
    gi, gj, gd = geo["cap_i"], geo["cap_j"], geo["cap_d"]
    for i in (0, 17, 100, v.shape[0] - 2):
        rows = geodesic.compute_distance_parallel(v, f, thr, i)
        sel = gi == i
        assert [r[1] for r in rows] == gj[sel].tolist()
        np.testing.assert_allclose([r[2] for r in rows], gd[sel], rtol=RTOL, atol=0)
        assert all(r[0] == i for r in rows)


def _noisy(level, radius, noise, seed):
    v, f = synth.icosphere(level)
    rng = np.random.default_rng(seed)
    return (v * radius * (1.0 + noise * rng.standard_normal((v.shape[0], 1)))).astype(np.float32), f


def test_both_directions_vs_oracle_level5():
    """10,242 vertices, saddles everywhere, every source, j < i included."""
    v, f = _noisy(5, 20.0, 0.04, 3)
    m = geodesic.GeodesicMesh(v, f)
    assert m.n_saddle > 0
    got = m.lists(2.5, False)
    _same(got, oracle.geodesic_lists(v, f, 2.5, False))


def test_capacity_retry_vs_oracle():
    """A radius that reaches ~1,600 vertices per source: more than the first
    launch's distance table holds, so those sources run again with four
    times the room; the lists still equal the oracle's."""
    v, f = _noisy(5, 10.0, 0.02, 4)
    m = geodesic.GeodesicMesh(v, f)
    got = m.lists(8.0, True, 0, 96)
    ref = oracle.geodesic_lists(v, f, 8.0, True, 0, 96)
    assert np.bincount(ref[0]).max() > 700
    _same(got, ref)


def test_distance_lists_form():
    """distance_lists: the pairs and distances
    fwhm_compute_distances_parallel.py:104-110 assembles, j > i."""
    v, f = _noisy(4, 12.0, 0.05, 6)
    pairs, d = geodesic.distance_lists(v, f, 3.0)
    i, j, dd = oracle.geodesic_lists(v, f, 3.0, True)
    np.testing.assert_array_equal(pairs, np.stack([i, j], axis=1))
    np.testing.assert_allclose(d, dd, rtol=RTOL, atol=0)
    assert np.all(pairs[:, 1] > pairs[:, 0])
