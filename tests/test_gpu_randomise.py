"""The randomise driver drop-ins read the reference's hand-off files and
append the same CSV lines as the reference's scripts.

Checked against the oracle on host-seeded permutation streams (--seed);
values are parsed back from the CSV text and compared with relative
tolerance 1e-3 (float32 t on the GPU, float64 in the oracle; 4 decimals in
the file).
"""
import os
from types import SimpleNamespace

import numpy as np
import pytest

from oracle import oracle
from tfce_mediation_gb300 import adjacency as A
from tfce_mediation_gb300 import randomise, synth

pytestmark = pytest.mark.gpu


def _obj(lists):
    a = np.empty(len(lists), dtype=object)
    for i, l in enumerate(lists):
        a[i] = l
    return a


@pytest.fixture()
def vertex_temp(tmp_path):
    v, f = synth.icosphere(3)
    off, idx = A.mesh_csr(f, v.shape[0])
    Vh = v.shape[0]
    rng = np.random.default_rng(3)
    mask_lh = np.ones(Vh, bool)
    mask_rh = np.ones(Vh, bool)
    mask_rh[rng.choice(Vh, 60, replace=False)] = False
    n = 50
    Y = synth.surface_data(rng, n, off, idx, 3)
    Y2 = synth.surface_data(rng, n, off, idx, 3)
    merge_y = np.ascontiguousarray(np.concatenate([Y[:, mask_lh], Y2[:, mask_rh]], axis=1))
    pred_x = np.column_stack([synth.binary_half(rng, n), rng.standard_normal(n)])
    merge_y[:, :80] += (0.8 * pred_x[:, 0])[:, None].astype(np.float32)
    adj = _obj(A.from_csr(off, idx))
    vd = A.vertex_density((off, idx))
    d = tmp_path / "python_temp_area"
    d.mkdir()
    for name, val in (("merge_y", merge_y), ("num_vertex", merge_y.shape[1]), ("num_vertex_lh", int(mask_lh.sum())),
                      ("all_vertex", Vh), ("bin_mask_lh", mask_lh), ("bin_mask_rh", mask_rh), ("num_subjects", n),
                      ("pred_x", pred_x), ("adjac_lh", adj), ("adjac_rh", adj), ("optstfce", np.array([2.0, 1.0])),
                      ("vdensity_lh", vd), ("vdensity_rh", vd)):
        np.save(d / f"{name}.npy", val, allow_pickle=True)
    return tmp_path, dict(off=off, idx=idx, mask_lh=mask_lh, mask_rh=mask_rh, merge_y=merge_y, pred_x=pred_x,
                          n=n, vd=vd, Vh=Vh)


def _oracle_vertex_max(info, stat):
    best = -np.inf
    nl = int(info["mask_lh"].sum())
    for mask, part in ((info["mask_lh"], stat[:nl]), (info["mask_rh"], stat[nl:])):
        full = np.zeros(info["Vh"], np.float32)
        full[mask] = part
        e = oracle.tfce(info["off"], info["idx"], full, 2.0, 1.0)
        best = max(best, float(((e * (full.max() / np.float32(100))) * info["vd"]).max()))
    return best


def test_vertex_regress_run(vertex_temp):
    root, info = vertex_temp
    cwd = os.getcwd()
    os.chdir(root)
    try:
        opts = SimpleNamespace(range=[0, 5], surface=["area"], seed=[100], specifyvars=None, exchangeblock=None,
                               batch=4)
        randomise.vertex_regress_run(opts)
        X = np.column_stack([np.ones(info["n"]), info["pred_x"]])
        for c in (1, 2):
            lines = open(f"output_area/perm_Tstat_area/perm_tstat_con{c}_TFCE_maxVertex.csv").read().split()
            assert len(lines) == 12
            for p in range(6):
                perm = np.random.RandomState(100 + p).permutation(info["n"])
                t = oracle.tval_fp64(X[perm], info["merge_y"])[c].astype(np.float32)
                for si, s in enumerate((1.0, -1.0)):
                    ref = _oracle_vertex_max(info, s * t)
                    got = float(lines[2 * p + si])
                    assert abs(got - ref) <= 1e-3 * abs(ref) + 1e-4, (c, p, s, got, ref)
    finally:
        os.chdir(cwd)


def test_vertex_mediation_run(vertex_temp):
    root, info = vertex_temp
    d = root / "python_temp_med_area"
    d.mkdir()
    src = root / "python_temp_area"
    for f in os.listdir(src):
        os.link(src / f, d / f)
    rng = np.random.default_rng(8)
    x = info["pred_x"][:, 0]
    dy = 0.5 * x + rng.standard_normal(info["n"])
    np.save(d / "pred_x.npy", x)
    np.save(d / "depend_y.npy", dy)
    cwd = os.getcwd()
    os.chdir(root)
    try:
        opts = SimpleNamespace(range=[0, 3], surface=["area"], seed=[7], medtype=["M"], batch=4)
        randomise.vertex_mediation_run(opts)
        lines = open("output_med_area/perm_SobelZ_M/perm_Zstat_M_TFCE_maxVertex.csv").read().split()
        assert len(lines) == 4
        for p in range(4):
            perm = np.random.RandomState(7 + p).permutation(info["n"])
            with np.errstate(all="ignore"):
                z = oracle.calc_sobelz("M", x[perm], dy, info["merge_y"].astype(np.float64), info["n"])
            ref = _oracle_vertex_max(info, z.astype(np.float32))
            assert abs(float(lines[p]) - ref) <= 1e-3 * abs(ref) + 1e-4
    finally:
        os.chdir(cwd)


def test_voxel_regress_run_t_and_f(tmp_path):
    st = synth.config3(seed=4, n=40, shape=(20, 22, 18), semi=(8.0, 9.0, 7.0), fwhm=2.0)
    d = tmp_path / "python_temp"
    d.mkdir()
    adj = _obj(A.from_csr(st.offsets, st.indices))
    for name, val in (("num_voxel", st.V), ("num_subjects", st.n), ("raw_nonzero_corr", st.Y.T.copy()),
                      ("pred_x", st.pred_x), ("adjac", adj), ("ancova", 0), ("optstfce", np.array([2.0, 0.5, 26]))):
        np.save(d / f"{name}.npy", val, allow_pickle=True)
    cwd = os.getcwd()
    os.chdir(tmp_path)
    try:
        os.makedirs("output", exist_ok=True)
        opts = SimpleNamespace(range=[0, 2], seed=[3], specifyvars=None, exchangeblock=None, batch=4)
        randomise.voxel_regress_run(opts)
        X = st.design()
        lines = open("output/perm_Tstat/perm_tstat_con1_TFCE_maxVoxel.csv").read().split()
        assert len(lines) == 6
        for p in range(3):
            perm = np.random.RandomState(3 + p).permutation(st.n)
            t = oracle.tval_fp64(X[perm], st.Y)[1].astype(np.float32)
            for si, s in enumerate((1.0, -1.0)):
                ref = oracle.tfce_max_batch(st.offsets, st.indices, t, 2.0, 0.5, sign=s)[0]
                assert abs(float(lines[2 * p + si]) - ref) <= 1e-3 * abs(ref) + 1e-4
        # F-test branch (ancova): twice the permutations, sqrt(max(F,0)) swept with one sign
        np.save(d / "ancova.npy", 1)
        randomise.voxel_regress_run(opts)
        lines = open("output/perm_Tstat/perm_fstat_TFCE_maxVoxel.csv").read().split()
        assert len(lines) == 5
        for p in range(5):
            perm = np.random.RandomState(3 + p).permutation(st.n)
            with np.errstate(all="ignore"):
                F = oracle.calcF(X[perm], st.Y.astype(np.float64), st.n, X.shape[1])
            f = np.sqrt(np.maximum(F, 0)).astype(np.float32)
            ref = oracle.tfce_max_batch(st.offsets, st.indices, f, 2.0, 0.5)[0]
            assert abs(float(lines[p]) - ref) <= 1e-3 * abs(ref) + 1e-4
    finally:
        os.chdir(cwd)


def test_mmr_lr_run(tmp_path):
    v, f = synth.icosphere(3)
    off, idx = A.mesh_csr(f, v.shape[0])
    rng = np.random.default_rng(6)
    n = 40
    data = synth.surface_data(rng, n, off, idx, 3)
    pred_x = rng.standard_normal((n, 2))
    d = tmp_path / "tmi_temp"
    d.mkdir()
    np.save(d / "2_adjacency_temp.npy", _obj(A.from_csr(off, idx)), allow_pickle=True)
    np.save(d / "2_mask_temp.npy", np.ones(v.shape[0], np.float32))
    np.save(d / "2_data_temp.npy", data)
    np.save(d / "2_vdensity_temp.npy", np.float32(1.0))
    out = tmp_path / "out"
    out.mkdir()
    cwd = os.getcwd()
    os.chdir(tmp_path)
    try:
        randomise.mmr_lr_run(2, (4, 6), 1000, str(out), 2.0, 1.0, pred_x=pred_x, batch=2)
        X = np.column_stack([np.ones(n), pred_x])
        for c in (1, 2):
            lines = open(out / f"perm_maxTFCE_surf2_tcon{c}.csv").read().split()
            assert len(lines) == 6
            for j, p in enumerate(range(4, 7)):
                perm = np.random.RandomState(p + 1000).permutation(n)
                t = oracle.tval_fp64(X[perm], data)[c].astype(np.float32)
                for si, s in enumerate((1.0, -1.0)):
                    ref = oracle.tfce_max_batch(off, idx, t, 2.0, 1.0, sign=s)[0]
                    assert abs(float(lines[2 * j + si]) - ref) <= 1e-3 * abs(ref) + 1e-5
    finally:
        os.chdir(cwd)
