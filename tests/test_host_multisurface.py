"""Host-side logic of the multisurface drivers and the image readers, on CPU:
the per-surface cuts of a merged adjacency, the density weights of the
in-memory driver, TMI files holding masks of different shapes, the NIfTI /
MGH readers, and the bench's study hand-off to its CPU-baseline workers."""
import os

import numpy as np

from oracle import oracle
from tests.mmr_case import mmr_case
from tfce_mediation_gb300 import adjacency as A
from tfce_mediation_gb300 import io, tmi
from tfce_mediation_gb300.randomise import _mmr_layout
from tfce_mediation_gb300.tm_func import _surface_parts, create_full_mask


class _Merged:
    def __init__(self, csr):
        self.csr = csr


def test_surface_parts_cut_the_merged_adjacency(golden):
    """The drop-ins cut a CreateAdjSet's merged adjacency back into one CSR
    per surface over its masked vertices: the same lists as inducing each
    surface's own adjacency on its mask."""
    case = mmr_case(golden)
    merged = oracle.merge_adjacency(case["adjs"])
    parts = _surface_parts(_Merged(merged), case["masks"], create_full_mask(case["masks"]))
    for s, (off, idx) in enumerate(parts):
        m = np.asarray(case["masks"][s])
        keep = m[:, 0, 0] if m.shape[2] == 1 else np.ones(int(m.sum()), bool)
        ro, ri = A.induced_csr(list(case["adjs"][s]), keep)
        np.testing.assert_array_equal(off, ro)
        np.testing.assert_array_equal(idx, ri)


def test_mmr_layout_segments_and_density(golden):
    """Segments in position order and the density weights of
    tm_multimodality_multisurface_regression.py:449-462 (surfaces masked,
    volumes over their voxels)."""
    case = mmr_case(golden)
    off, idx, seg, vd = _mmr_layout(case["masks"], case["adjs"], [0, 1, 2], noweight=False)
    np.testing.assert_array_equal(seg, case["pos"])
    np.testing.assert_allclose(vd, golden["mmr_vd"], rtol=0, atol=0)
    assert off.shape[0] - 1 == case["pos"][-1]
    _, _, _, vd0 = _mmr_layout(case["masks"], case["adjs"], [0, 1, 2], noweight=True)
    assert vd0 is None


def test_tmi_masks_of_different_shapes_round_trip(golden, tmp_path):
    case = mmr_case(golden)
    name = tmi.write_tm_filetype(str(tmp_path / "study"), image_array=case["y"].T, masking_array=list(case["masks"]),
                                 adjacency_array=list(case["adjs"]), checkname=False)
    out = tmi.read_tm_filetype(name, verbose=False)
    assert [m.shape for m in out[2]] == [np.asarray(m).shape for m in case["masks"]]
    for a, b in zip(out[2], case["masks"]):
        np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(out[1][0], case["y"].T)
    for a, b in zip(out[8], case["adjs"]):
        assert [list(x) for x in a] == [list(x) for x in b]


def test_image_readers_round_trip(tmp_path):
    aff = np.array([[-2.0, 0, 0, 90], [0, 0, 2.0, -126], [0, -2.0, 0, 72], [0, 0, 0, 1]])
    vol = np.random.default_rng(1).standard_normal((7, 6, 5)).astype(np.float32)
    for ext in (".nii", ".nii.gz"):
        io.save_nifti(vol, aff, str(tmp_path / ("v" + ext)))
        d, a = io.load_nifti(str(tmp_path / ("v" + ext)))
        np.testing.assert_array_equal(d, vol)
        np.testing.assert_allclose(a, aff)
    d64 = vol.astype(np.float64)
    io.save_nifti(d64, aff, str(tmp_path / "d.nii.gz"))
    d, _ = io.load_nifti(str(tmp_path / "d.nii.gz"))
    assert d.dtype == np.float64
    np.testing.assert_array_equal(d, d64)
    surf = np.random.default_rng(2).standard_normal((40, 1, 1)).astype(np.float32)
    io.save_mgh(surf, aff, str(tmp_path / "s.mgh"))
    d, a = io.load_mgh(str(tmp_path / "s.mgh"), with_affine=True)
    np.testing.assert_array_equal(d, surf)
    np.testing.assert_allclose(a, aff, atol=1e-5)


def test_bench_study_hand_off(tmp_path):
    import bench
    from tfce_mediation_gb300 import synth
    st = synth.vertex_study(seed=3, level=2, n=12, passes=1, hemispheres=2, k=3, patches=((10, 0.5, 1),))
    bench._stash_study(st, str(tmp_path / "s"))
    back = bench._unstash_study(str(tmp_path / "s"))
    np.testing.assert_array_equal(np.asarray(back.Y), st.Y)
    for f in ("pred_x", "offsets", "indices", "segments", "H", "E"):
        np.testing.assert_array_equal(getattr(back, f), getattr(st, f))
    assert back.name == st.name and back.info == st.info
