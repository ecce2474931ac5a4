"""Observed-statistic and 1-p(FWER) outputs on the GPU against the oracle:
write_vertStat_img / write_voxelStat_img (pyfunc.py:80-103), the batched
STEP_1 output drivers (step1.py) and the calculate_fweP_vertex / _voxel
drop-ins (calculate_fwep.py), reading back the images they write.

Tolerances: a drop-in writer sweeps the caller's statistic with the
reference's arithmetic (the threshold weight correctly rounded: <= 1e-6
relative); the STEP_1 drivers compute t with the FP32 GLM (~1e-6 of FP64),
so their images are compared through the max (1e-3) and the bulk of the
vertices (99% within 1e-4 of the image's max); 1-p values are exact.
"""
import os

import numpy as np
import pytest

from oracle import oracle
from tfce_mediation_gb300 import adjacency as A
from tfce_mediation_gb300 import calculate_fwep, io, pyfunc, step1, synth
from tfce_mediation_gb300 import tfce as T

pytestmark = pytest.mark.gpu


def _close_images(got, ref):
    got, ref = np.asarray(got, np.float64).ravel(), np.asarray(ref, np.float64).ravel()
    scale = max(np.abs(ref).max(), 1e-12)
    assert abs(got.max() - ref.max()) <= 1e-3 * scale, (got.max(), ref.max())
    assert (np.abs(got - ref) <= 1e-4 * scale).mean() >= 0.99


def _csv_rows(path):
    rows = {}
    for line in open(path).read().split():
        k, v = line.rsplit(",", 1)
        rows[k] = float(v)
    return rows


@pytest.fixture(scope="module")
def hemi():
    v, f = synth.icosphere(4)
    off, idx = A.mesh_csr(f, v.shape[0])
    S = synth.smoothing_matrix(off, idx)
    rng = np.random.default_rng(41)
    m = rng.standard_normal(v.shape[0])
    for _ in range(4):
        m = S @ m
    mask = np.ones(v.shape[0], bool)
    mask[rng.choice(v.shape[0], 200, replace=False)] = False
    return off, idx, (3.0 * m / m.std()), mask


@pytest.mark.parametrize("density", ["one", "weights"])
def test_write_vertStat_img_vs_oracle(hemi, tmp_path, monkeypatch, density):
    off, idx, m, mask = hemi
    monkeypatch.chdir(tmp_path)
    stat = m[mask]
    dens = 1 if density == "one" else A.vertex_density(A.from_csr(off, idx))
    op = T.CreateAdjSet(2.0, 1.0, A.from_csr(off, idx))
    out = np.zeros((mask.shape[0], 1, 1), np.float32)
    aff = np.diag([1.0, 1.0, 1.0, 1.0])
    pyfunc.write_vertStat_img("tstat_con1", stat, out, aff, "area", "lh", mask, op, mask.shape[0], dens)
    ref = oracle.vert_stat_tfce_image(stat, mask, off, idx, 2.0, 1.0, dens)
    got = io.load_mgh("tstat_con1_area_lh_TFCE.mgh")[:, 0, 0]
    np.testing.assert_allclose(got, ref.astype(np.float32), rtol=2e-6, atol=1e-12 * np.abs(ref).max())
    raw = io.load_mgh("tstat_con1_area_lh.mgh")[:, 0, 0]
    np.testing.assert_array_equal(raw[mask], stat.astype(np.float32))
    assert not raw[~mask].any()
    row = _csv_rows("max_TFCE_contrast_values.csv")["tstat_con1_area_lh"]
    assert abs(row - ref.max()) <= 1e-6 * abs(ref.max()) + 1e-6


def test_write_voxelStat_img_vs_oracle(tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)
    mask = synth.ellipsoid_mask((24, 26, 22), (9.0, 10.0, 8.0))
    off, idx = A.voxel_csr(mask, 26, "pyfunc")
    rng = np.random.default_rng(3)
    Y = synth.volume_data(rng, 2, mask, 2.0)[0]
    stat = (Y * 3.0).astype(np.float64)
    op = T.CreateAdjSet(2.0, 0.5, A.from_csr(off, idx))
    out_path = mask.astype(np.float32)
    aff = np.diag([2.0, 2.0, 2.0, 1.0])
    pyfunc.write_voxelStat_img("tstat_con1", stat, out_path, mask, aff, op)
    ref = oracle.voxel_stat_tfce_image(stat, off, idx, 2.0, 0.5)
    img, a = io.load_nifti("tstat_con1_TFCE.nii.gz")
    np.testing.assert_allclose(img[mask], ref, rtol=2e-6, atol=1e-12 * np.abs(ref).max())
    np.testing.assert_allclose(a, aff)
    raw, _ = io.load_nifti("tstat_con1.nii.gz")
    np.testing.assert_allclose(raw[mask], stat.astype(np.float32))


def _vertex_handoff(surface, rng):
    st = synth.vertex_study(seed=44, level=4, n=60, passes=4, hemispheres=2, k=3, patches=((120, 0.8, 1),))
    Vh = st.V // 2
    masks = []
    for _ in range(2):
        m = np.ones(Vh, bool)
        m[rng.choice(Vh, 150, replace=False)] = False
        masks.append(m)
    v0 = st.segments
    adj = A.from_csr(st.offsets[:Vh + 1], st.indices[:st.offsets[Vh]])
    merge_y = np.concatenate([st.Y[:, :Vh][:, masks[0]], st.Y[:, Vh:][:, masks[1]]], axis=1).astype(np.float32)
    d = "python_temp_%s" % surface
    os.makedirs(d)
    obj = np.empty(Vh, dtype=object)
    for i, a in enumerate(adj):
        obj[i] = list(a)
    vd = A.vertex_density(adj)
    for name, val in (("merge_y", merge_y), ("num_subjects", st.n), ("pred_x", st.pred_x),
                      ("bin_mask_lh", masks[0]), ("bin_mask_rh", masks[1]), ("affine_mask_lh", np.eye(4)),
                      ("affine_mask_rh", np.eye(4)), ("adjac_lh", obj), ("adjac_rh", obj),
                      ("optstfce", np.array([2.0, 1.0])), ("vdensity_lh", vd), ("vdensity_rh", vd),
                      ("num_vertex_lh", int(masks[0].sum())), ("all_vertex", Vh)):
        np.save(f"{d}/{name}", val)
    return st, masks, merge_y, vd, v0


def test_vertex_observed_run_vs_oracle(tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)
    rng = np.random.default_rng(8)
    st, masks, merge_y, vd, _ = _vertex_handoff("area", rng)
    Vh = st.V // 2
    off, idx = st.offsets[:Vh + 1], st.indices[:st.offsets[Vh]]
    step1.vertex_observed_run("area")
    X = st.design()
    t = oracle.tval_int_ref(X, np.linalg.inv(X.T @ X), merge_y.astype(np.float64), st.n, X.shape[1])
    nl = int(masks[0].sum())
    rows = _csv_rows("output_area/max_TFCE_contrast_values.csv")
    assert len(rows) == 2 * 2 * 2
    for j in (1, 2):
        for name, sgn in (("tstat_con%d" % j, 1.0), ("negtstat_con%d" % j, -1.0)):
            for h, hemi in enumerate(("lh", "rh")):
                stat = (t[j, :nl] if h == 0 else t[j, nl:]) * sgn
                ref = oracle.vert_stat_tfce_image(stat, masks[h], off, idx, 2.0, 1.0, vd)
                got = io.load_mgh(f"output_area/{name}_area_{hemi}_TFCE.mgh")[:, 0, 0]
                _close_images(got, ref)
                assert abs(rows[f"{name}_area_{hemi}"] - ref.max()) <= 1e-3 * abs(ref.max())
                raw = io.load_mgh(f"output_area/{name}_area_{hemi}.mgh")[:, 0, 0]
                np.testing.assert_allclose(raw[masks[h]], stat, rtol=2e-5, atol=2e-5)


def test_voxel_observed_run_vs_oracle(tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)
    st = synth.config3(seed=13, n=40, shape=(22, 24, 20), semi=(8.0, 9.0, 7.0), fwhm=2.0)
    mask = synth.ellipsoid_mask((22, 24, 20), (8.0, 9.0, 7.0))
    os.makedirs("python_temp")
    adj = A.from_csr(st.offsets, st.indices)
    obj = np.empty(len(adj), dtype=object)
    for i, a in enumerate(adj):
        obj[i] = list(a)
    for name, val in (("raw_nonzero_corr", st.Y.T.astype(np.float32)), ("pred_x", st.pred_x), ("adjac", obj),
                      ("optstfce", np.array([2.0, 0.5, 26])), ("ancova", 0), ("data_mask", mask.astype(np.float32)),
                      ("affine_mask", np.diag([2.0, 2.0, 2.0, 1.0]))):
        np.save(f"python_temp/{name}", val)
    step1.voxel_observed_run()
    X = st.design()
    t = oracle.tval_int_ref(X, np.linalg.inv(X.T @ X), st.Y.astype(np.float64), st.n, X.shape[1])
    for j in (1, 2, 3):
        for name, sgn in (("tstat_con%d" % j, 1.0), ("negtstat_con%d" % j, -1.0)):
            ref = oracle.voxel_stat_tfce_image(t[j] * sgn, st.offsets, st.indices, 2.0, 0.5)
            img, _ = io.load_nifti(f"output/{name}_TFCE.nii.gz")
            _close_images(img[mask], ref)


def test_calculate_fwep_vertex_and_voxel(hemi, tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)
    off, idx, m, mask = hemi
    rng = np.random.default_rng(12)
    tf = np.where(mask, np.abs(m) * 40.0, 0.0).astype(np.float32)
    tf[:30] = 0.0
    null = np.round(rng.gamma(3.0, 30.0, 400), 4)
    np.savetxt("perm.csv", null, fmt="%.4f")
    io.save_mgh(tf[:, None, None], np.eye(4), "img_TFCE.mgh")
    opts = calculate_fwep.parser().parse_args(["-i", "img_TFCE.mgh", "perm.csv", "-l"])
    calculate_fwep.vertex_run(opts)
    got = io.load_mgh("img_TFCE_FWEcorrP.mgh")[:, 0, 0]
    ref = oracle.fwep_vertex(tf, np.genfromtxt("perm.csv", delimiter=","))
    np.testing.assert_array_equal(got, ref.astype(np.float32))
    with np.errstate(divide="ignore"):
        nl = np.where(tf > 0, -np.log10(1 - ref), 0.0)
    np.testing.assert_allclose(io.load_mgh("img_TFCE_FWEneglog10p.mgh")[:, 0, 0], nl.astype(np.float32))
    vol = np.zeros((9, 8, 7), np.float32)
    vol[1:8, 1:7, 1:6] = rng.gamma(3.0, 35.0, (7, 6, 5))
    io.save_nifti(vol, np.diag([2.0, 2.0, 2.0, 1.0]), "vox_TFCE.nii.gz")
    opts = calculate_fwep.parser().parse_args(["-i", "vox_TFCE.nii.gz", "perm.csv"])
    calculate_fwep.voxel_run(opts)
    got, _ = io.load_nifti("vox_TFCE_FWEcorrP.nii.gz")
    np.testing.assert_array_equal(got, oracle.fwep_vertex(vol, np.genfromtxt("perm.csv", delimiter=",")))
