"""TMI container I/O against the reference's own tm_io (imported from a
reference checkout when one is present; skipped otherwise) and round trips.

Cross check: files written here are read by the reference's own reader,
element for element."""
import os
import sys

import numpy as np
import pytest

from tfce_mediation_gb300 import tmi

from oracle.build_ref import ref_root

REF = ref_root()


def _sample(rng):
    data = rng.standard_normal((500, 7)).astype(np.float32)
    mask = np.zeros((6, 5, 4), bool)
    mask[1:5, 1:4, 1:3] = True
    aff = rng.standard_normal((4, 4)).astype(np.float32)
    v = rng.standard_normal((12, 3)).astype(np.float32)
    f = rng.integers(0, 12, (20, 3)).astype(np.uint32)
    adj = np.empty(12, dtype=object)
    for i in range(12):
        adj[i] = np.array(sorted(set(rng.integers(0, 12, 4)) - {i}), dtype=np.int64)
    cols = np.array(["s%02d" % i for i in range(7)])
    return data, mask, aff, v, f, adj, cols


def _check(out, data, mask, aff, v, f, adj, cols):
    element, img, masks, mnames, affs, verts, faces, snames, adjs, hist, colids = out
    assert element[:6] == ["data_array", "masking_array", "affine", "vertex", "face", "adjacency_object"]
    np.testing.assert_array_equal(img[0], data)
    np.testing.assert_array_equal(masks[0], mask)
    np.testing.assert_array_equal(affs[0], aff)
    np.testing.assert_array_equal(verts[0], v)
    np.testing.assert_array_equal(faces[0], f)
    assert mnames == ["m1"] and snames == ["lh"]
    for a, b in zip(adjs[0], adj):
        np.testing.assert_array_equal(a, b)
    assert hist[-1].startswith("history mode_add")


def test_binary_round_trip(tmp_path):
    data, mask, aff, v, f, adj, cols = _sample(np.random.default_rng(1))
    name = tmi.write_tm_filetype(str(tmp_path / "a"), image_array=data, masking_array=[mask], maskname=["m1"],
                                 affine_array=[aff], vertex_array=[v], face_array=[f], surfname=["lh"],
                                 adjacency_array=[adj], columnids=cols)
    assert name.endswith("a.tmi")
    out = tmi.read_tm_filetype(name, verbose=False)
    _check(out, data, mask, aff, v, f, adj, cols)
    np.testing.assert_array_equal(out[10][0], cols)
    # history counts of what the file holds: 1 data, 1 mask, 1 affine, 1 surface, 1 adjacency set
    assert out[9][-1].split()[3:] == ["1", "1", "1", "1", "1"]
    # an existing name is not overwritten
    assert os.path.basename(tmi.check_outname(name)) == "new_a.tmi"


def test_ascii_round_trip(tmp_path):
    data, mask, aff, v, f, _, _ = _sample(np.random.default_rng(2))
    name = tmi.write_tm_filetype(str(tmp_path / "b"), output_binary=False, image_array=data,
                                 masking_array=[mask], maskname=["m1"], affine_array=[aff])
    assert name.endswith(".ascii.tmi")
    el, img, masks, _, affs, *_ = tmi.read_tm_filetype(name, verbose=False)
    np.testing.assert_allclose(img[0], data, rtol=1e-6)
    np.testing.assert_array_equal(masks[0], mask)
    np.testing.assert_allclose(affs[0], aff, rtol=1e-6)


def _reference_tm_io():
    path = os.path.join(REF, "tfce_mediation", "tm_io.py")
    if not os.path.exists(path):
        pytest.skip("no reference checkout")
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
    import make_golden
    R = make_golden.load_reference()
    if "tm_io" not in R:
        pytest.skip("reference tm_io not importable")
    io = R["tm_io"]
    compat = make_golden._OldNumpyArray()
    compat.int = int  # the reader's np.int (numpy < 1.24)
    io.np = compat
    return io


def test_reference_reader_reads_ours(tmp_path):
    """Files written here, read by the reference's own reader (data, mask,
    affine, surface, adjacency).  The reference's binary writer does not run
    on numpy >= 2 (it tests ``image_array == []`` and then takes
    ``image_array.T`` unconditionally), so it is not exercised."""
    ref = _reference_tm_io()
    data, mask, aff, v, f, adj, cols = _sample(np.random.default_rng(3))
    mine = tmi.write_tm_filetype(str(tmp_path / "mine"), image_array=data, masking_array=[mask], maskname=["m1"],
                                 affine_array=[aff], vertex_array=[v], face_array=[f], surfname=["lh"],
                                 adjacency_array=[adj])
    _check(ref.read_tm_filetype(mine, verbose=False), data, mask, aff, v, f, adj, cols)
    # two surfaces and two masks, element counts in the history line
    mine2 = tmi.write_tm_filetype(str(tmp_path / "two"), image_array=data, masking_array=[mask, ~mask],
                                  maskname=["m1", "m2"], vertex_array=[v, v * 2], face_array=[f, f],
                                  surfname=["lh", "rh"])
    out = ref.read_tm_filetype(mine2, verbose=False)
    assert len(out[2]) == 2 and len(out[5]) == 2
    np.testing.assert_array_equal(out[2][1], ~mask)
    np.testing.assert_array_equal(out[5][1], v * 2)
    assert out[9][-1].split()[3:] == ["1", "2", "0", "2", "0"]
