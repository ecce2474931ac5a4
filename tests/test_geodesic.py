"""Exact geodesic neighbour lists (tfce_mediation/adjacency.pyx:44-106), CPU
side: the oracle against the reference's own outputs (golden vectors made by
tests/golden/make_geodesic_golden.py from the reference's compiled
adjacency.pyx over lib/geodesic, and the reference library itself where
oracle/_ref holds it), the drop-in's list construction, and the host-side
mesh checks of the C-ABI (no device needed)."""
import os

import numpy as np
import pytest

from oracle import oracle
from tfce_mediation_gb300 import _lib, synth
from tfce_mediation_gb300.geodesic import lists_from_pairs

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "geodesic_vectors.npz")
MESHES = ("sphere", "cap", "bumpy")


@pytest.fixture(scope="module")
def geo():
    return np.load(GOLDEN)


def _assert_same_lists(got, ref, rtol=1e-12):
    gi, gj, gd = got
    ri, rj, rd = ref
    np.testing.assert_array_equal(gi, ri)
    np.testing.assert_array_equal(gj, rj)
    np.testing.assert_allclose(gd, rd, rtol=rtol, atol=0)


@pytest.mark.parametrize("name", MESHES)
def test_oracle_matches_reference_golden(geo, name):
    """Saddle vertices (radial noise), a boundary (the open cap), two mesh
    levels: the same pairs as the reference, distances within 1e-12."""
    v, f = geo[f"{name}_v"], geo[f"{name}_f"]
    thr, n_src = float(geo[f"{name}_threshold"]), int(geo[f"{name}_n_src"])
    got = oracle.geodesic_lists(v, f, thr, True, 0, n_src)
    _assert_same_lists(got, (geo[f"{name}_i"], geo[f"{name}_j"], geo[f"{name}_d"]))


def test_oracle_matches_reference_library_directly():
    """Another seed, a larger radius and both directions (j < i too), against
    the reference library built into oracle/_ref from the checkout."""
    if oracle.ref_geodesic_lib() is None:
        pytest.skip("oracle/_ref/libref_geodesic.so not built (no reference checkout here)")
    v, f = synth.icosphere(3)
    rng = np.random.default_rng(11)
    v = (v * 10.0 * (1.0 + 0.07 * rng.standard_normal((v.shape[0], 1)))).astype(np.float32)
    got = oracle.geodesic_lists(v, f, 6.0, False)
    ref = oracle.ref_geodesic_lists(v, f, 6.0, False)
    _assert_same_lists(got, ref)


def test_lists_from_pairs_match_reference_compute(geo):
    """The drop-in's compute() lists from the reference's own pairs equal the
    reference's compute() output at every threshold (ascending lists)."""
    thr = geo["compute_thresholds"]
    V = geo["sphere_v"].shape[0]
    lists = lists_from_pairs(geo["sphere_i"], geo["sphere_j"], geo["sphere_d"], thr, V)
    assert len(lists) == thr.shape[0]
    for k in range(thr.shape[0]):
        off, idx = geo[f"compute_{k}_off"], geo[f"compute_{k}_idx"]
        for x in range(V):
            assert lists[k][x] == idx[off[x]:off[x + 1]].tolist(), (k, x)


def test_symmetry_of_oracle_distances():
    """Both directions of a pair agree to rounding (geodesics are symmetric)."""
    v, f = synth.icosphere(3)
    rng = np.random.default_rng(5)
    v = (v * 10.0 * (1.0 + 0.05 * rng.standard_normal((v.shape[0], 1)))).astype(np.float32)
    i, j, d = oracle.geodesic_lists(v, f, 4.0, False)
    fwd = {(a, b): c for a, b, c in zip(i.tolist(), j.tolist(), d.tolist())}
    for (a, b), c in fwd.items():
        if (b, a) in fwd:
            assert abs(fwd[(b, a)] - c) <= 1e-12 * c


@pytest.mark.parametrize("case", ["index", "repeated", "flat", "nonmanifold"])
def test_mesh_create_rejects_bad_meshes_on_host(case):
    """geodesic_mesh_create checks the mesh before any device work."""
    import ctypes
    lib = _lib.load()
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0], [0, 0, 1], [2, 0, 0]], np.float32)
    faces = {"index": [[0, 1, 7]], "repeated": [[0, 1, 1]], "flat": [[0, 1, 5]],
             "nonmanifold": [[0, 1, 2], [1, 0, 3], [0, 1, 4]]}[case]
    f = np.array(faces, np.int32)
    h = ctypes.c_void_p()
    rc = lib.geodesic_mesh_create(_lib.ptr(v, _lib.c_f32p), v.shape[0], _lib.ptr(f, _lib.c_i32p), f.shape[0],
                                  ctypes.byref(h))
    assert rc == _lib.TFCE_EINVAL
    assert not h.value
