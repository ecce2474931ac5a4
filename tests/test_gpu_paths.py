"""Mediation, voxel and multisurface paths on the GPU against the oracle and
the reference's own outputs (golden vectors).

Tolerances: the engines compute the permutation t maps with the split-BF16
tensor-core GLM (~3e-5 relative to FP64; z inherits it), the oracle in
float64, so sweeps see maps that differ slightly.  Per-permutation maxima:
relative error <= 1e-3 (median <= 1e-4); TFCE images: |delta| <= 1e-3 * max.
"""
import os

import numpy as np
import pytest

from oracle import oracle
from tfce_mediation_gb300 import adjacency as A
from tfce_mediation_gb300 import engine as E
from tfce_mediation_gb300 import synth

pytestmark = pytest.mark.gpu


def _assert_maxima(got, ref):
    rel = np.abs(got - ref) / np.maximum(np.abs(ref), 1e-12)
    print("maxima: median", np.median(rel), "max", rel.max())
    assert np.median(rel) <= 1e-4, np.median(rel)
    assert rel.max() <= 1e-3, rel.max()


def _seg_csr(st, h):
    v0, v1 = st.segments[h], st.segments[h + 1]
    off = st.offsets[v0:v1 + 1] - st.offsets[v0]
    idx = st.indices[st.offsets[v0]:st.offsets[v1]] - v0
    return off, idx, v0, v1


@pytest.fixture(scope="module")
def med_study():
    st = synth.vertex_study(seed=31, level=4, n=80, passes=4, hemispheres=2, k=3,
                            patches=((150, 0.6, 1),), name="med")
    rng = np.random.default_rng(5)
    x = st.pred_x[:, 0]
    dy = 0.3 * st.Y[:, :150].mean(axis=1) + 0.4 * x + rng.standard_normal(st.n)
    return st, x, dy


@pytest.mark.parametrize("medtype", ["M", "I", "Y"])
def test_mediation_engine_vs_oracle(med_study, medtype):
    st, x, dy = med_study
    eng = E.MediationEngine(st.Y, x, dy, medtype, (st.offsets, st.indices), st.segments, 2.0, 1.0,
                            floor_zero=True, batch=8)
    perms = E.permutations(st.n, 40, 0, 12)
    got = eng.run(perms=perms)[:, 0, 0, :]  # (P, S)
    ref = np.zeros_like(got)
    for p in range(perms.shape[0]):
        xp = x[perms[p]]
        dyp = dy if medtype in ("M", "I") else dy[perms[p]]
        with np.errstate(all="ignore"):
            z = oracle.calc_sobelz(medtype, xp, dyp, st.Y.astype(np.float64), st.n).astype(np.float32)
        for h in range(2):
            off, idx, v0, v1 = _seg_csr(st, h)
            ref[p, h] = oracle.tfce_max_batch(off, idx, z[v0:v1], 2.0, 1.0, floor_zero=True)[0]
    _assert_maxima(got, ref)


def test_mediation_run_stream_uploads_match_serial_runs(med_study):
    """MediationEngine.run_stream with new data every step (uploads on a side
    stream after the previous batch's GLM) returns exactly what upload + run
    per step returns."""
    import torch
    st, x, dy = med_study
    eng = E.MediationEngine(st.Y, x, dy, "M", (st.offsets, st.indices), st.segments, 2.0, 1.0,
                            floor_zero=True, batch=8)
    perms = E.permutations(st.n, 41, 0, 21)
    rng = np.random.default_rng(12)
    datas = [torch.from_numpy((st.Y + 0.3 * rng.standard_normal(st.Y.shape)).astype(np.float32)).pin_memory()
             for _ in range(3)]
    steps = [(datas[0], perms[:8]), (datas[1], perms[8:16]), (datas[2], perms[16:])]
    got = eng.run_stream(steps)
    for (d, pr), g in zip(steps, got):
        eng.inner.upload(d)
        np.testing.assert_array_equal(g, eng.run(perms=pr))


def test_voxel_engine_E_half_vs_oracle():
    st = synth.config3(seed=3, n=48, shape=(26, 30, 24), semi=(11.0, 13.0, 10.0), fwhm=2.0)
    eng = E.PermutationEngine(st.Y, st.pred_x, (st.offsets, st.indices), None, 2.0, 0.5, batch=8)
    perms = E.permutations(st.n, 9, 0, 10)
    got = eng.run(perms=perms)[..., 0]  # (P, C, 2)
    X = st.design()
    ref = np.zeros_like(got)
    for p in range(perms.shape[0]):
        t = oracle.tval_fp64(X[perms[p]], st.Y)
        for ci, c in enumerate((1, 2, 3)):
            for si, s in enumerate((1.0, -1.0)):
                ref[p, ci, si] = oracle.tfce_max_batch(st.offsets, st.indices, t[c].astype(np.float32), 2.0,
                                                       0.5, sign=s)[0]
    _assert_maxima(got, ref)


def test_multisurface_segments_per_segment_HE():
    """Uneven surfaces plus a voxel skeleton in one launch, own H/E each
    (mmr-lr semantics, one permutation stream for all surfaces).  The t maps
    come from the FP32 GLM (~1e-6 of FP64) so that the per-value bar tests the
    segment handling: on segments of a few hundred vertices one vertex moving
    across a threshold under the split-BF16 GLM's ~2e-5 can move a maximum by
    more than 1e-3."""
    st = synth.config4_mmr(seed=5, n=40, levels=[2, 3, 2, 4], skeleton_voxels=600, passes=3)
    eng = E.PermutationEngine(st.Y, st.pred_x, (st.offsets, st.indices), st.segments, st.H, st.E,
                              floor_zero=False, batch=6, precision="fp32")
    perms = E.permutations(st.n, 77, 0, 6)
    got = eng.run(perms=perms)  # (P, C, 2, S)
    X = st.design()
    for p in range(perms.shape[0]):
        t = oracle.tval_fp64(X[perms[p]], st.Y)
        for ci, c in enumerate((1, 2)):
            for si, s in enumerate((1.0, -1.0)):
                for h in range(len(st.segments) - 1):
                    off, idx, v0, v1 = _seg_csr(st, h)
                    ref = oracle.tfce_max_batch(off, idx, t[c, v0:v1].astype(np.float32), float(st.H[h]),
                                                float(st.E[h]), sign=s)[0]
                    g = got[p, ci, si, h]
                    assert abs(g - ref) <= 1e-3 * abs(ref) + 1e-9, (p, c, s, h, g, ref)


def test_low_ram_calculate_tfce_vs_reference(golden):
    from tfce_mediation_gb300 import tm_func
    from tfce_mediation_gb300.tfce import CreateAdjSet
    op = CreateAdjSet(2.0, 1.0, A.from_csr(golden["sweep_off"], golden["sweep_idx"]))
    yl, xl = golden["lr_y"], golden["lr_x"]
    mask = np.ones(yl.shape[1], np.float32)
    tv, tp, tn = tm_func.low_ram_calculate_tfce(yl, mask, xl, op, 1)
    ref_t = golden["lr_t"]
    err = np.abs(tv - ref_t) / np.maximum(1.0, np.abs(ref_t))
    assert err.max() <= 1e-4
    for got, ref in ((tp, golden["lr_pos"]), (tn, golden["lr_neg"])):
        assert np.abs(got - ref).max() <= 1e-3 * np.abs(ref).max()


def test_apply_mfwer_vs_reference(golden, tmp_path):
    from tfce_mediation_gb300 import tm_func
    images = golden["mfwer_images"]
    perm = golden["mfwer_perm"]
    cwd = os.getcwd()
    os.chdir(tmp_path)
    try:
        os.mkdir("output_study")
        k = 0
        for s in range(3):
            for c in range(2):
                np.savetxt(f"output_study/perm_maxTFCE_surf{s}_tcon{c + 1}.csv", perm[k], fmt="%f")
                k += 1
        for w in (None, "logmasksize"):
            p, q = tm_func.apply_mfwer([images], 2, range(3), perm.shape[1], 3, "study",
                                       list(golden["mfwer_pos_array"]), [0, 1], [2, 3], weight=w)
            np.testing.assert_array_equal(p, golden[f"mfwer_pos_{w}"])
            np.testing.assert_array_equal(q, golden[f"mfwer_neg_{w}"])
    finally:
        os.chdir(cwd)


def test_fwer_kernels(golden):
    import torch
    from tfce_mediation_gb300 import fwer
    rng = np.random.default_rng(0)
    for n in (1, 2, 3, 100, 1000, 4097, 20000):
        a = rng.standard_normal(n)
        d = fwer.sorted_null(a)
        np.testing.assert_array_equal(d.cpu().numpy(), np.sort(a))
    null, img = golden["fwe_null"], golden["fwe_img"]
    np.testing.assert_array_equal(fwer.fwep(img, null), golden["fwe_vertex"])
    np.testing.assert_array_equal(fwer.nearest(img, null), golden["fwe_nearest"])
