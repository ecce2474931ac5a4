"""In-memory multisurface (mmr) bodies on the GPU: tm_func.calculate_tfce,
calc_mixed_tfce and calculate_mediation_tfce drop-ins against the reference's
own outputs (golden vectors), the batched driver (randomise.mmr_run) against
the oracle, and the grouped-threshold engine at the multimodal study's full
size (20 icospheres of levels 5-7 and a ~120k-voxel skeleton, n = 350).

Tolerances: the sweep of the reference's own float32 t is bit-identical up to
the threshold weight's rounding (correctly rounded T^H here, the host libm's
powf there: <= 1e-6 relative); the drop-ins compute t with the FP32 GLM
(~1e-6 of the reference's FP64 t), which can move a vertex across a
threshold, so maps are compared through their per-surface maxima (relative
<= 1e-3, median <= 1e-4) and the bulk of the vertices (99% within 1e-4 of
the map's max); the engines use the split-BF16 GLM (~3e-5).
"""
import os

import numpy as np
import pytest

from oracle import oracle
from tests.mmr_case import csv_values, mmr_case
from tfce_mediation_gb300 import adjacency as A
from tfce_mediation_gb300 import engine as E
from tfce_mediation_gb300 import synth
from tfce_mediation_gb300 import tfce as T
from tfce_mediation_gb300 import tm_func

pytestmark = pytest.mark.gpu


def _assert_maxima(got, ref, med=1e-4, mx=1e-3):
    got, ref = np.asarray(got, np.float64), np.asarray(ref, np.float64)
    rel = np.abs(got - ref) / np.maximum(np.abs(ref), 1e-12)
    print("maxima: median", np.median(rel), "max", rel.max())
    assert np.median(rel) <= med, np.median(rel)
    assert rel.max() <= mx, rel.max()


def _assert_maps(got, ref, pos):
    got, ref = np.asarray(got, np.float64), np.asarray(ref, np.float64)
    _assert_maxima(oracle.surface_maxima(got, pos), oracle.surface_maxima(ref, pos))
    scale = np.maximum(np.abs(ref).max(axis=-1, keepdims=True), 1e-12)
    close = np.abs(got - ref) <= 1e-4 * scale
    assert close.mean() >= 0.99, close.mean()


@pytest.fixture(scope="module")
def case(golden):
    c = mmr_case(golden)
    c["op"] = T.CreateAdjSet(2.0, 1.0, tm_func.merge_adjacency_array(range(3), c["adjs"]))
    return c


def test_grouped_sweep_of_reference_t_is_bitwise(golden, case):
    """The reference's own float32 t through the one-launch study sweep:
    every surface's map equals the reference's merged-image sweep."""
    import torch
    study = tm_func._study_for([case["op"]], np.zeros(3, np.int32), case["masks"], tm_func.create_full_mask)
    for tag in ("obs", "vd", "perm"):
        t = torch.from_numpy(np.ascontiguousarray(golden[f"mmr_calc_t_{tag}"])).cuda()
        vd = case["vd"] if tag == "vd" else 1
        mx, maps = study.sweep(t, t.shape[0], 2, vd, want_maps=True)
        for s, key in enumerate(("pos", "neg")):
            ref = golden[f"mmr_calc_{key}_{tag}"]
            np.testing.assert_allclose(maps[:, s], ref, rtol=1e-6, atol=1e-12 * np.abs(ref).max(), err_msg=tag)
            np.testing.assert_allclose(mx[:, s], oracle.surface_maxima(ref, case["pos"]), rtol=1e-6)


@pytest.mark.parametrize("tag", ["obs", "vd", "perm"])
def test_calculate_tfce_dropin(golden, case, tag):
    vd = case["vd"] if tag == "vd" else 1
    x = case["x"][case["perm"]] if tag == "perm" else case["x"]
    tv, tp, tn = tm_func.calculate_tfce(case["y"], case["masks"], x, case["op"], vd, case["pos"], case["full"])
    np.testing.assert_allclose(tv, golden[f"mmr_calc_t_{tag}"], rtol=2e-5, atol=2e-5)
    _assert_maps(tp, golden[f"mmr_calc_pos_{tag}"], case["pos"])
    _assert_maps(tn, golden[f"mmr_calc_neg_{tag}"], case["pos"])


def test_calc_mixed_tfce_dropin(golden, case):
    ops = [T.CreateAdjSet(H, E_, tm_func.merge_adjacency_array(np.arange(3)[sel], case["adjs"][sel]))
           for (H, E_), sel in zip(golden["mmr_mixed_settings"], (golden["mmr_mixed_assign"] == 0,
                                                                  golden["mmr_mixed_assign"] == 1))]
    a, b, c = tm_func.calc_mixed_tfce(golden["mmr_mixed_assign"], case["y"], case["masks"], case["pos"], 1, case["x"],
                                      ops)
    assert a is b is c  # one array, as the reference returns it
    _assert_maps(c[None], golden["mmr_mixed_obs"][None], case["pos"])


def test_calculate_mediation_tfce_dropin(golden, case):
    z, tz = tm_func.calculate_mediation_tfce("M", case["y"], case["masks"], golden["mmr_med_x"], golden["mmr_med_dy"],
                                             case["op"], 1, case["pos"], case["full"])
    np.testing.assert_allclose(z, golden["mmr_med_z"], rtol=1e-4, atol=1e-4)
    _assert_maps(tz[None], golden["mmr_med_tfce"][None], case["pos"])


def test_randomised_calls_write_the_reference_csv(golden, case, tmp_path, monkeypatch):
    """The randomised calls with the clock replaced by the constant the
    golden run used: the same permutations, the same CSV files and lines."""
    monkeypatch.setattr(tm_func, "time", lambda: 1700000000.25)
    monkeypatch.chdir(tmp_path)
    ops = [T.CreateAdjSet(H, E_, tm_func.merge_adjacency_array(np.arange(3)[sel], case["adjs"][sel]))
           for (H, E_), sel in zip(golden["mmr_mixed_settings"], (golden["mmr_mixed_assign"] == 0,
                                                                  golden["mmr_mixed_assign"] == 1))]
    for kind in ("calc", "mixed", "med"):
        os.makedirs(kind)
        os.chdir(kind)
        for pn in (0, 1):
            if kind == "calc":
                tm_func.calculate_tfce(case["y"], case["masks"], case["x"], case["op"], 1, case["pos"], case["full"],
                                       perm_number=pn, randomise=True)
            elif kind == "mixed":
                tm_func.calc_mixed_tfce(golden["mmr_mixed_assign"], case["y"], case["masks"], case["pos"], 1,
                                        case["x"], ops, perm_number=pn, randomise=True)
            else:
                tm_func.calculate_mediation_tfce("M", case["y"], case["masks"], golden["mmr_med_x"],
                                                 golden["mmr_med_dy"], case["op"], 1, case["pos"], case["full"],
                                                 perm_number=pn, randomise=True)
        got, ref = [], []
        for s in range(3):
            if kind == "med":
                got.append(np.loadtxt(f"perm_maxTFCE_surf{s}_M_zstat.csv"))
                ref.append(csv_values(golden[f"mmr_csv_med_s{s}"]))
                continue
            for c in (1, 2):
                got.append(np.loadtxt(f"perm_maxTFCE_surf{s}_tcon{c}.csv"))
                ref.append(csv_values(golden[f"mmr_csv_{kind}_s{s}_c{c}"]))
        _assert_maxima(np.concatenate(got), np.concatenate(ref), med=2e-4, mx=2e-3)
        os.chdir("..")


def test_mmr_run_batched_driver(golden, case, tmp_path, monkeypatch):
    """The batched driver from a TMI file: permutation maxima of the seeded
    stream against the oracle's calculate_tfce / calc_mixed_tfce, and the
    observed branch's maps against the reference's."""
    from tfce_mediation_gb300 import randomise as R
    from tfce_mediation_gb300 import tmi
    monkeypatch.chdir(tmp_path)
    tmi.write_tm_filetype("study", image_array=case["y"].T, masking_array=list(case["masks"]),
                          adjacency_array=list(case["adjs"]), checkname=False)
    np.savetxt("x0.csv", case["x"][:, 0], delimiter=",")
    np.savetxt("x1.csv", case["x"][:, 1], delimiter=",")
    n = case["y"].shape[0]
    perms = np.stack([np.random.RandomState(7 + p).permutation(n) for p in range(6)])
    for mixed in (False, True):
        args = ["-i_tmi", "study.tmi", "-i", "x0.csv", "x1.csv", "-p", "0", "5", "--seed", "7", "--noweight",
                "-i_name", "mixed" if mixed else "calc", "--batch", "4"]
        if mixed:
            args += ["-st", "0", "0", "1", "--tfce", "2", "1", "2", "0.5"]
        opts = R.mmr_parser().parse_args(args)
        got = R.mmr_run(opts)  # (P, C, 2, S)
        ref = np.zeros_like(got)
        for p in range(perms.shape[0]):
            if mixed:
                _, tp, tn = oracle.calc_mixed_tfce([0, 0, 1], case["y"], case["masks"], case["adjs"],
                                                   [(2.0, 1.0), (2.0, 0.5)], case["x"], 1, perm=perms[p])
            else:
                _, tp, tn = oracle.calculate_tfce(case["y"], case["masks"], case["x"], case["adjs"], 2.0, 1.0, 1,
                                                  perm=perms[p])
            ref[p, :, 0] = oracle.surface_maxima(tp, case["pos"])
            ref[p, :, 1] = oracle.surface_maxima(tn, case["pos"])
        _assert_maxima(got, ref)
        name = "mixed" if mixed else "calc"
        csv = np.loadtxt(f"output_{name}/output_stats_{name}.tmi/perm_maxTFCE_surf2_tcon1.csv")
        np.testing.assert_allclose(csv, got[:, 0, :, 2].reshape(-1), rtol=1e-6, atol=1e-6)
    opts = R.mmr_parser().parse_args(["-i_tmi", "study.tmi", "-i", "x0.csv", "x1.csv", "--noweight",
                                      "-i_name", "obs"])
    out = R.mmr_run(opts)
    _assert_maps(out[:, 2:4].T, golden["mmr_calc_pos_obs"], case["pos"])
    _assert_maps(out[:, 4:6].T, golden["mmr_calc_neg_obs"], case["pos"])
    back = tmi.read_tm_filetype("output_obs/stats_obs.tmi", verbose=False)
    np.testing.assert_allclose(back[1][0], out.astype(np.float32), rtol=1e-6)


def _group_maxima_oracle(st, X, perm, groups, contrasts):
    """Per-segment maxima of one permutation with grouped threshold tables
    (each group's segments are one contiguous span here): FP64 t, every group
    swept as one merged image, each segment scaled by its own max / 100."""
    t = oracle.tval_fp64(X[perm], st.Y)
    S = len(st.segments) - 1
    out = np.zeros((len(contrasts), 2, S))
    for g in np.unique(groups):
        segs = np.flatnonzero(groups == g)
        v0, v1 = st.segments[segs[0]], st.segments[segs[-1] + 1]
        off = st.offsets[v0:v1 + 1] - st.offsets[v0]
        idx = st.indices[st.offsets[v0]:st.offsets[v1]] - v0
        H, E_ = float(st.H[segs[0]]), float(st.E[segs[0]])
        for ci, c in enumerate(contrasts):
            img = t[c, v0:v1].astype(np.float32)
            for si, sgn in enumerate((1.0, -1.0)):
                im = img * np.float32(sgn)
                e = oracle.tfce(off, idx, im, H, E_)
                for s in segs:
                    a, b = st.segments[s] - v0, st.segments[s + 1] - v0
                    out[ci, si, s] = np.max(e[a:b] * (im[a:b].max() / np.float32(100)))
    return out


def test_multimodal_study_full_size():
    """The multimodal study at its specified size: 20 icospheres of levels
    5-7 (6 x 163,842 + 7 x 40,962 + 7 x 10,242 vertices) and a ~120k-voxel
    skeleton, n = 350, about 1.4M elements; the icospheres are one TFCE
    setting (H=2, E=1, one merged threshold table, calc_mixed_tfce's group 0),
    the skeleton another (H=2, E=0.5); per-surface maxima of a few seeded
    permutations against the oracle."""
    st = synth.config4_mmr()
    S = len(st.segments) - 1
    groups = np.array([0] * (S - 1) + [1], np.int32)
    eng = E.PermutationEngine(st.Y, st.pred_x, (st.offsets, st.indices), st.segments, st.H, st.E,
                              threshold_groups=groups, batch=4)
    perms = E.permutations(st.n, 5, 0, 3)
    got = eng.run(perms=perms)  # (P, C, 2, S)
    X = st.design()
    ref = np.stack([_group_maxima_oracle(st, X, perms[p], groups, (1, 2)) for p in range(perms.shape[0])])
    _assert_maxima(got, ref)
    # the study-wide value per permutation: max over surfaces
    _assert_maxima(got.max(axis=-1), ref.max(axis=-1))


def test_mmr_lr_from_tmi_equals_per_surface_jobs(golden, case, tmp_path, monkeypatch):
    """mmr-lr straight from the TMI file (all surfaces in one launch) writes
    the same per-surface CSV values as the per-surface jobs that read the
    tmi_temp/ hand-off, on the same seeded permutations."""
    from tfce_mediation_gb300 import randomise as R
    from tfce_mediation_gb300 import tmi
    monkeypatch.chdir(tmp_path)
    tmi.write_tm_filetype("study", image_array=case["y"].T, masking_array=list(case["masks"]),
                          adjacency_array=list(case["adjs"]), checkname=False)
    got = R.mmr_lr_tmi_run("study.tmi", (0, 7), 11, "out_tmi", tfce=(2.0, 1.0), pred_x=case["x"], noweight=True,
                           batch=4)
    os.makedirs("tmi_temp")
    os.makedirs("out_jobs")
    pos = case["pos"]
    for s in range(3):
        m = np.asarray(case["masks"][s])
        mask = m[:, 0, 0] if m.shape[2] == 1 else m[m]
        np.save(f"tmi_temp/{s}_mask_temp.npy", mask)
        np.save(f"tmi_temp/{s}_adjacency_temp.npy", case["adjs"][s], allow_pickle=True)
        np.save(f"tmi_temp/{s}_data_temp.npy", np.ascontiguousarray(case["y"][:, pos[s]:pos[s + 1]], np.float32))
        np.save(f"tmi_temp/{s}_vdensity_temp.npy", np.array([1.0], np.float32))
        R.mmr_lr_run(s, (0, 7), 11, "out_jobs", 2.0, 1.0, pred_x=case["x"], batch=4)
    for s in range(3):
        for c in (1, 2):
            a = np.loadtxt(f"out_tmi/perm_maxTFCE_surf{s}_tcon{c}.csv")
            b = np.loadtxt(f"out_jobs/perm_maxTFCE_surf{s}_tcon{c}.csv")
            np.testing.assert_allclose(a, b, rtol=1e-6, atol=1e-6, err_msg=f"surface {s} contrast {c}")
    assert got.shape == (8, 2, 2, 3)
