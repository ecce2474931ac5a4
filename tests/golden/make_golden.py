"""Generate the golden vectors in tests/golden/ by running the reference itself.

Run on a machine that holds a reference checkout (``$TFCE_REFERENCE_ROOT``,
else ``reference`` beside the repository directory) after
``python oracle/build_ref.py``:

    python tests/golden/make_golden.py

It imports the reference's compiled operator modules (``tfce``, ``cynumstats``
built into oracle/_ref/) and its unmodified ``pyfunc.py`` / ``tm_func.py`` /
``tm_io.py`` (nibabel and matplotlib, absent here, are replaced by empty stub
modules; none of the functions recorded touch them), calls them on small seeded
inputs and stores inputs and outputs as compressed .npz fixtures.  The fixtures
are what the tests compare against; the reference is not needed afterwards.
"""
from __future__ import annotations

import importlib.util
import os
import sys
import tempfile
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle.build_ref import ref_root  # noqa: E402

REF = ref_root()


def _stub(name):
    m = types.ModuleType(name)
    sys.modules[name] = m
    return m


def load_reference():
    for name in ["nibabel", "nibabel.freesurfer", "nibabel.freesurfer.mghformat", "matplotlib",
                 "matplotlib.pyplot", "matplotlib.colors", "matplotlib.patches", "matplotlib.cm"]:
        _stub(name)
    sys.modules["matplotlib"].use = lambda *a, **k: None
    sys.path.insert(0, os.path.join(ROOT, "oracle", "_ref"))
    import tfce_mediation  # the oracle/_ref package holding the compiled modules
    from tfce_mediation import cynumstats, tfce  # noqa: F401
    mods = {}
    for name in ["pyfunc", "tm_io", "tm_func"]:
        path = os.path.join(REF, "tfce_mediation", f"{name}.py")
        spec = importlib.util.spec_from_file_location(f"tfce_mediation.{name}", path)
        mod = importlib.util.module_from_spec(spec)
        sys.modules[f"tfce_mediation.{name}"] = mod
        setattr(tfce_mediation, name, mod)
        try:
            spec.loader.exec_module(mod)
        except Exception as exc:  # tm_io needs more of nibabel at import time
            print(f"note: {name} not importable ({exc!r})")
            sys.modules.pop(f"tfce_mediation.{name}", None)
            continue
        mods[name] = mod
    mods["tfce"] = sys.modules["tfce_mediation.tfce"]
    mods["cynumstats"] = sys.modules["tfce_mediation.cynumstats"]
    return mods


class _OldNumpyArray(types.ModuleType):
    """numpy as seen by code written for numpy < 1.24: np.array of ragged lists
    gives an object array (pyfunc.create_adjac_voxel relies on it) instead of
    raising.  Everything else is numpy itself."""

    def __init__(self):
        super().__init__("numpy_compat")

    def __getattr__(self, name):
        return getattr(np, name)

    @staticmethod
    def argwhere(a):
        # int() of a one-element array row (tm_func.calc_mixed_tfce) worked on
        # older numpy; rows of a 1-D argument come back as plain indices
        r = np.argwhere(a)
        return r.ravel() if np.ndim(a) == 1 else r

    @staticmethod
    def array(obj, *a, **k):
        try:
            return np.array(obj, *a, **k)
        except ValueError:
            out = np.empty(len(obj), dtype=object)
            for i, x in enumerate(obj):
                out[i] = x
            return out


def main():
    from tfce_mediation_gb300 import adjacency as A
    from tfce_mediation_gb300 import synth

    R = load_reference()
    tfce, cyn, pyfunc = R["tfce"], R["cynumstats"], R["pyfunc"]
    pyfunc.np = _OldNumpyArray()
    rng = np.random.default_rng(20261203)
    out = {}

    # --- adjacency builders -------------------------------------------------
    v, f = synth.icosphere(2)
    ref_adj = pyfunc.create_adjac_vertex(v, f)
    off, idx = A.to_csr([sorted(s) for s in ref_adj])
    out["adj_mesh_faces"] = f.astype(np.int32)
    out["adj_mesh_nv"] = np.int32(v.shape[0])
    out["adj_mesh_off"], out["adj_mesh_idx"] = off, idx
    mask = np.zeros((7, 6, 5), bool)
    mask[1:6, 1:5, 1:4] = True
    mask[0, 0, 0] = True
    mask[3, 0, 2] = True
    mask[6, 5, 4] = True
    out["vox_mask"] = mask
    for dirtype in (6, 26):
        nv = int(mask.sum())
        adj = pyfunc.create_adjac_voxel(mask, mask.astype(np.float32), nv, dirtype=dirtype)
        o, i = A.to_csr([list(a) for a in adj])
        out[f"vox{dirtype}_off"], out[f"vox{dirtype}_idx"] = o, i
    try:
        # the tool imports the geodesic extension at module level; it is not
        # used by create_adjac_voxel
        if "tfce_mediation.adjacency" not in sys.modules:
            _stub("tfce_mediation.adjacency").compute = None
        spec = importlib.util.spec_from_file_location(
            "tm_mmr_adj", os.path.join(REF, "tfce_mediation", "tools", "tm_mulitmodality_adjacency.py"))
        mmr_adj = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mmr_adj)
        for dirtype in (6, 26):
            adj = mmr_adj.create_adjac_voxel(mask, dirtype=dirtype)
            o, i = A.to_csr([sorted(a) for a in adj])
            out[f"voxmmr{dirtype}_off"], out[f"voxmmr{dirtype}_idx"] = o, i
    except Exception as exc:
        print(f"note: mmr voxel adjacency not recorded ({exc!r})")

    # --- TFCE sweeps on a level-3 icosphere ---------------------------------
    v3, f3 = synth.icosphere(3)
    off3, idx3 = A.mesh_csr(f3, v3.shape[0])
    adj3 = A.from_csr(off3, idx3)
    S = synth.smoothing_matrix(off3, idx3)
    maps = []
    for _ in range(4):
        m = rng.standard_normal(v3.shape[0]).astype(np.float32)
        for _ in range(3):
            m = (S @ m).astype(np.float32)
        maps.append(m * np.float32(4.0))
    maps.append(np.round(maps[0] * 2) / 2)  # ties
    maps.append(-np.abs(maps[1]))  # all <= 0
    maps = np.stack(maps).astype(np.float32)
    out["sweep_off"], out["sweep_idx"], out["sweep_maps"] = off3, idx3, maps
    params = [(2.0, 1.0), (2.0, 0.5), (1.0, 0.67), (2.0, 2.0), (1.5, 0.75)]
    out["sweep_params"] = np.array(params, np.float32)
    res = np.zeros((len(params), maps.shape[0], maps.shape[1]), np.float32)
    for pi, (H, E) in enumerate(params):
        op = tfce.CreateAdjSet(H, E, adj3)
        for mi in range(maps.shape[0]):
            if maps[mi].max() == 0:
                continue  # the reference never returns on a map whose maximum is 0
            e = np.zeros(maps.shape[1], np.float32)
            op.run(maps[mi].copy(), e)
            res[pi, mi] = e
    out["sweep_enhn"] = res
    # accumulation into a non-zero enhn
    op = tfce.CreateAdjSet(2.0, 1.0, adj3)
    e0 = rng.standard_normal(maps.shape[1]).astype(np.float32)
    e = e0.copy()
    op.run(maps[2].copy(), e)
    out["sweep_accum_in"], out["sweep_accum_out"] = e0, e

    # --- GLM helpers ---------------------------------------------------------
    n, V = 40, 300
    y = rng.standard_normal((n, V)).astype(np.float32)
    x = np.column_stack([rng.integers(0, 2, n), rng.standard_normal(n), rng.standard_normal(n)])
    X = np.column_stack([np.ones(n), x])
    invXX = np.linalg.inv(X.T @ X)
    out["glm_y"], out["glm_x"] = y, x
    out["glm_tval_int"] = cyn.tval_int(X, invXX, y, n, X.shape[1], V)
    b, se = cyn.calc_beta_se(x[:, 0], y, n, V)
    out["glm_cbs_beta"], out["glm_cbs_se"] = b, se
    out["glm_lstsqr"] = cyn.cy_lin_lstsqr_mat(X, y)
    out["glm_calcF"] = cyn.calcF(X, y, n, X.shape[1])
    out["glm_resid_covars"] = cyn.resid_covars(X[:, :2], y.T)
    a, rss = cyn.cy_lin_lstsqr_mat_residual(X, y)
    out["glm_lsr_a"], out["glm_lsr_rss"] = a, rss
    sig2 = rng.uniform(0.5, 2.0, V)
    out["glm_sig2"] = sig2
    out["glm_se_of_slope"] = cyn.se_of_slope(V, invXX, sig2, X.shape[1])

    # --- Sobel z ---------------------------------------------------------------
    mx = rng.integers(0, 2, n).astype(np.float64)
    dy = rng.standard_normal(n) + 0.5 * mx
    my = (y + 0.3 * mx[:, None] + 0.2 * dy[:, None]).astype(np.float32)
    out["sobel_x"], out["sobel_dy"], out["sobel_y"] = mx, dy, my
    for mt in ("I", "M", "Y"):
        for alg in ("aroian", "sobel", "goodman"):
            with np.errstate(all="ignore"):
                out[f"sobel_{mt}_{alg}"] = pyfunc.calc_sobelz(mt, mx, dy, my, n, V, alg=alg)

    # --- per-permutation maxima (CSV) ----------------------------------------
    Vh = off3.shape[0] - 1
    lh = tfce.CreateAdjSet(2.0, 1.0, adj3)
    rh = tfce.CreateAdjSet(2.0, 1.0, adj3)
    mask_lh = np.ones(Vh, bool)
    mask_rh = np.ones(Vh, bool)
    mask_rh[: Vh // 5] = False
    nmask = int(mask_lh.sum())
    stat = np.concatenate([maps[0], maps[1][mask_rh]]).astype(np.float64)
    vd = A.vertex_density(adj3)
    with tempfile.TemporaryDirectory() as td:
        cwd = os.getcwd()
        os.chdir(td)
        try:
            pyfunc.write_perm_maxTFCE_vertex("tstat_con1", stat, nmask, mask_lh, mask_rh, lh, rh)
            pyfunc.write_perm_maxTFCE_vertex("tstat_con1", -stat, nmask, mask_lh, mask_rh, lh, rh)
            pyfunc.write_perm_maxTFCE_vertex("tstat_con2", stat, nmask, mask_lh, mask_rh, lh, rh, vd, vd)
            pyfunc.write_perm_maxTFCE_voxel("tstat_con1", maps[3].astype(np.float64), lh)
            out["perm_csv_vertex1"] = np.array(open("perm_tstat_con1_TFCE_maxVertex.csv").read())
            out["perm_csv_vertex2"] = np.array(open("perm_tstat_con2_TFCE_maxVertex.csv").read())
            out["perm_csv_voxel1"] = np.array(open("perm_tstat_con1_TFCE_maxVoxel.csv").read())
        finally:
            os.chdir(cwd)
    out["perm_stat"], out["perm_mask_rh"], out["perm_vd"] = stat, mask_rh, vd

    # --- FWER lookups -----------------------------------------------------------
    null = np.round(rng.gamma(3.0, 50.0, 200), 4)
    img = np.concatenate([rng.gamma(3.0, 60.0, 500), np.zeros(20), null[:10], [1e6, -1.0]])
    out["fwe_null"], out["fwe_img"] = null, img
    srt = np.sort(null)
    p_array = np.arange(len(srt)) / len(srt)
    # calculate_fweP_vertex.find_nearest (restated here only to record the
    # reference module's answer; the module itself needs nibabel at run time)
    spec = importlib.util.spec_from_file_location(
        "fwep_vertex", os.path.join(REF, "tfce_mediation", "tmanalysis", "calculate_fweP_vertex.py"))
    fwepv = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(fwepv)
    out["fwe_vertex"] = np.array([fwepv.find_nearest(srt, k, p_array) if k > 0 else 0.0 for k in img])
    if "tm_func" in R:
        out["fwe_nearest"] = np.array([R["tm_func"].find_nearest(srt, k, p_array) for k in img])
    else:
        out["fwe_nearest"] = np.array([pyfunc.find_nearest(srt, k, p_array) for k in img])

    # --- apply_mfwer -------------------------------------------------------------
    if "tm_func" in R:
        tmf = R["tm_func"]
        pos = [0, 40, 100, 130]
        nperm, ncon = 50, 2
        images = rng.gamma(2.0, 30.0, (130, 2 * ncon))
        images[rng.random(images.shape) < 0.2] = 0.0
        with tempfile.TemporaryDirectory() as td:
            cwd = os.getcwd()
            os.chdir(td)
            try:
                os.mkdir("output_study")
                perm = {}
                for s in range(3):
                    for c in range(ncon):
                        vals = rng.gamma(2.0 + s, 40.0, nperm)
                        perm[(s, c)] = vals
                        np.savetxt(f"output_study/perm_maxTFCE_surf{s}_tcon{c + 1}.csv", vals, fmt="%f")
                for w in (None, "logmasksize"):
                    with np.errstate(all="ignore"):
                        p, q = tmf.apply_mfwer([images], ncon, range(3), nperm, 3, "study", pos,
                                               [0, 1], [2, 3], weight=w)
                    out[f"mfwer_pos_{w}"], out[f"mfwer_neg_{w}"] = p, q
                out["mfwer_perm"] = np.stack([np.loadtxt(f"output_study/perm_maxTFCE_surf{s}_tcon{c + 1}.csv")
                                              for s in range(3) for c in range(ncon)])
            finally:
                os.chdir(cwd)
        out["mfwer_images"], out["mfwer_pos_array"] = images, np.array(pos)

        # low_ram_calculate_tfce, observed (not randomised)
        nl = 30
        yl = rng.standard_normal((nl, Vh)).astype(np.float32)
        for _ in range(3):
            yl = (S @ yl.T).T.astype(np.float32)
        xl = np.column_stack([rng.integers(0, 2, nl), rng.standard_normal(nl)])
        maskl = np.ones(Vh, np.float32)
        tv, tp, tn = tmf.low_ram_calculate_tfce(yl, maskl, xl, tfce.CreateAdjSet(2.0, 1.0, adj3), 1)
        out["lr_y"], out["lr_x"], out["lr_t"], out["lr_pos"], out["lr_neg"] = yl, xl, tv, tp, tn

    # glm_typeI (tm-models GLM): drop-one F per exogenous variable, model F
    # and t, observed and with a fixed permutation of the design rows
    nt, Vt = 60, 40
    yt = rng.standard_normal((nt, Vt)).astype(np.float32) + 2.0
    fac = rng.integers(0, 3, nt)
    ex0 = np.column_stack([(fac == 1), (fac == 2)]).astype(np.float64)
    ex1 = rng.standard_normal(nt)
    cov = rng.standard_normal((nt, 1))
    yt[:, :10] += (0.8 * ex1)[:, None].astype(np.float32)
    yt[:, 10:20] += (0.6 * ex0[:, 0])[:, None].astype(np.float32)
    permt = np.random.RandomState(77).permutation(nt)
    for tag, ra in (("obs", None), ("perm", permt)):
        Fm, Fv, Tv = pyfunc.glm_typeI(yt, [ex0, ex1], dmy_covariates=cov, output_fvalues=True,
                                  output_tvalues=True, verbose=False, rand_array=ra)
        out[f"typeI_F_{tag}"], out[f"typeI_Fvar_{tag}"], out[f"typeI_T_{tag}"] = Fm, np.asarray(Fv), Tv
    out["typeI_y"], out["typeI_ex0"], out["typeI_ex1"] = yt, ex0, ex1
    out["typeI_cov"], out["typeI_perm"] = cov, permt

    # glm_cosinor (tm-models cosinor): observed and permuted statistics with
    # two periods, one exogenous variable and a covariate; and the fit-only form
    nc, Vc = 48, 30
    tcos = rng.uniform(0.0, 48.0, nc)
    yc = rng.standard_normal((nc, Vc)).astype(np.float32) + 5.0
    yc[:, :12] += (1.5 * np.cos(2.0 * np.pi * (tcos - 3.0) / 24.0))[:, None].astype(np.float32)
    yc[:, 12:18] += (0.9 * np.sin(2.0 * np.pi * tcos / 12.0))[:, None].astype(np.float32)
    exc = rng.standard_normal(nc)
    covc = rng.standard_normal((nc, 1))
    permc = np.random.RandomState(78).permutation(nc)
    names = ("R2", "MESOR", "SE_MESOR", "AMP", "SE_AMP", "ACRO", "SE_ACRO", "F", "tMESOR", "tAMP", "tACRO",
             "tEXOG")
    for tag, ra in (("obs", None), ("perm", permc)):
        res = pyfunc.glm_cosinor(yc, tcos, exog=[exc], dmy_covariates=covc, rand_array=ra, period=[24.0, 12.0],
                                 calc_MESOR=ra is None)
        for name, val in zip(names, res):
            if val is not None:
                out[f"cos_{name}_{tag}"] = np.asarray(val)
    fit = pyfunc.glm_cosinor(yc, tcos, period=[24.0, 12.0], output_fit_only=True)
    out["cos_fit_MESOR"], out["cos_fit_AMP"], out["cos_fit_ACRO"] = (np.asarray(v) for v in fit)
    out["cos_y"], out["cos_t"], out["cos_ex"], out["cos_cov"], out["cos_perm"] = yc, tcos, exc, covc, permc

    # reg_rm_ancova_one_bs_factor / _two_bs_factor (tm-models RM-ANCOVA), short
    # data format, observed and permuted.  A permuted call draws its row
    # shuffle from the global RNG after rand_array; the same draws are
    # replayed here and stored ("rm*_shuffle").  The reference shuffles the
    # caller's array in place (its long form is a view), so every call gets
    # its own copy of the data.
    def seeded_call(fn, seed, n_subj, n_long, *args, **kw):
        np.random.seed(seed)
        ra = np.random.permutation(n_subj)
        res = fn(*args, rand_array=ra, **kw)
        np.random.seed(seed)
        np.random.permutation(n_subj)
        return res, ra, np.random.permutation(n_long)

    n1, s1, V1 = 24, 3, 20
    g1 = rng.integers(0, 2, n1)
    f1 = pyfunc.dummy_code(g1)
    subj1 = pyfunc.dummy_code(np.arange(n1), demean=False)
    cov1 = rng.standard_normal((n1, 1))
    d1 = rng.standard_normal((s1, n1, V1)).astype(np.float32) + 3.0
    d1 += (0.7 * rng.standard_normal(n1))[None, :, None].astype(np.float32)  # subject effects
    d1[2, :, :6] += (0.9 * g1)[:, None].astype(np.float32)  # group x time
    d1[1:, :, 6:10] += np.float32(0.6)  # time
    for tag, cv in (("nocov", None), ("cov", cov1)):
        res = pyfunc.reg_rm_ancova_one_bs_factor(d1.copy(), f1, subj1, dmy_covariates=cv, verbose=False)
        out[f"rm1_obs_{tag}"] = np.asarray(res)
        res, ra, sh = seeded_call(pyfunc.reg_rm_ancova_one_bs_factor, 91, n1, n1 * s1, d1.copy(), f1, subj1,
                                  dmy_covariates=cv, verbose=False)
        out[f"rm1_perm_{tag}"], out[f"rm1_ra_{tag}"], out[f"rm1_shuffle_{tag}"] = np.asarray(res), ra, sh
    out["rm1_data"], out["rm1_f1"], out["rm1_subj"], out["rm1_cov"] = d1, f1, subj1, cov1
    # the caller's array after one permuted call (shuffled in place)
    d_after = d1.copy()
    seeded_call(pyfunc.reg_rm_ancova_one_bs_factor, 93, n1, n1 * s1, d_after, f1, subj1, verbose=False)
    out["rm1_after_perm"] = d_after
    np.random.seed(93)
    np.random.permutation(n1)
    out["rm1_after_shuffle"] = np.random.permutation(n1 * s1)

    n2, s2, V2 = 30, 3, 16
    ga, gb = rng.integers(0, 2, n2), rng.integers(0, 3, n2)
    fa2, fb2 = pyfunc.dummy_code(ga), pyfunc.dummy_code(gb)
    subj2 = pyfunc.dummy_code(np.arange(n2), demean=False)
    cov2 = rng.standard_normal((n2, 1))
    d2 = rng.standard_normal((s2, n2, V2)).astype(np.float32) + 2.0
    d2 += (0.5 * rng.standard_normal(n2))[None, :, None].astype(np.float32)
    d2[:, :, :5] += (0.8 * (gb == 2))[None, :, None].astype(np.float32)
    d2[2, :, 5:9] += (0.9 * ga)[:, None].astype(np.float32)
    for tag, cv in (("nocov", None), ("cov", cov2)):
        res = pyfunc.reg_rm_ancova_two_bs_factor(d2.copy(), fa2, fb2, subj2, dmy_covariates=cv, verbose=False)
        out[f"rm2_obs_{tag}"] = np.asarray(res)
        res, ra, sh = seeded_call(pyfunc.reg_rm_ancova_two_bs_factor, 92, n2, n2 * s2, d2.copy(), fa2, fb2,
                                  subj2,
                                  dmy_covariates=cv, verbose=False)
        out[f"rm2_perm_{tag}"], out[f"rm2_ra_{tag}"], out[f"rm2_shuffle_{tag}"] = np.asarray(res), ra, sh
    out["rm2_data"], out["rm2_fa"], out["rm2_fb"], out["rm2_subj"], out["rm2_cov"] = d2, fa2, fb2, subj2, cov2

    # wider RM-ANCOVA and cosinor shapes: a three-level factor, two covariates,
    # four intervals; cosinor with two exogenous variables (one of two columns)
    rw = np.random.default_rng(79)
    n3, s3, V3 = 30, 4, 12
    g3 = rw.integers(0, 3, n3)
    f3 = pyfunc.dummy_code(g3)
    subj3 = pyfunc.dummy_code(np.arange(n3), demean=False)
    cov3 = rw.standard_normal((n3, 2))
    d3 = rw.standard_normal((s3, n3, V3)).astype(np.float32) + 1.0
    d3 += (0.5 * rw.standard_normal(n3))[None, :, None].astype(np.float32)
    d3[3, :, :4] += (0.8 * (g3 == 2))[:, None].astype(np.float32)
    out["rm3_obs"] = np.asarray(pyfunc.reg_rm_ancova_one_bs_factor(d3.copy(), f3, subj3, dmy_covariates=cov3,
                                                                  verbose=False))
    res, ra, sh = seeded_call(pyfunc.reg_rm_ancova_one_bs_factor, 94, n3, n3 * s3, d3.copy(), f3, subj3,
                              dmy_covariates=cov3, verbose=False)
    out["rm3_perm"], out["rm3_ra"], out["rm3_shuffle"] = np.asarray(res), ra, sh
    out["rm3_data"], out["rm3_f1"], out["rm3_subj"], out["rm3_cov"] = d3, f3, subj3, cov3
    nw, Vw = 40, 15
    tw = rw.uniform(0.0, 24.0, nw)
    yw = rw.standard_normal((nw, Vw)).astype(np.float32) + 3.0
    yw[:, :5] += (np.cos(2.0 * np.pi * tw / 24.0))[:, None].astype(np.float32)
    exw = [rw.standard_normal((nw, 2)), rw.standard_normal(nw)]
    permw = np.random.RandomState(80).permutation(nw)
    for tag, ra_ in (("obs", None), ("perm", permw)):
        r = pyfunc.glm_cosinor(yw, tw, exog=exw, rand_array=ra_, period=[24.0, 8.0])
        for name, val in zip(names, r):
            if val is not None:
                out[f"cosw_{name}_{tag}"] = np.asarray(val)
    out["cosw_y"], out["cosw_t"], out["cosw_ex0"], out["cosw_ex1"], out["cosw_perm"] = yw, tw, exw[0], exw[1], permw

    # calc_gd_fwhm (geodesic FWHM smoothing): vertex pairs of a level-3
    # icosphere within a radius (chord lengths standing in for geodesic
    # distances), plus a repeated pair and a self pair
    rg = np.random.default_rng(77)
    vg, _ = synth.icosphere(3)
    dd = np.linalg.norm(vg[:, None, :] - vg[None, :, :], axis=2)
    ii, jj = np.nonzero((dd < 0.35) & (np.arange(len(vg))[:, None] < np.arange(len(vg))[None, :]))
    order = rg.permutation(len(ii))
    pairs = np.column_stack([ii[order], jj[order]])
    pairs = np.concatenate([pairs, pairs[:3], [[5, 5]]]).astype(np.int32)
    dist = np.linalg.norm(vg[pairs[:, 0]] - vg[pairs[:, 1]], axis=1).astype(np.float32)
    dist[-1] = np.float32(0.0)
    out["gd_pairs"], out["gd_dist"] = pairs, dist
    for k, sg in enumerate((0.02, 0.005)):
        img = (rg.standard_normal(len(vg)) * 2.0 + 1.0).astype(np.float32)
        out[f"gd_data{k}"], out[f"gd_sigma{k}"] = img, np.float64(sg)
        out[f"gd_out{k}"] = cyn.calc_gd_fwhm(np.ascontiguousarray(pairs), np.ascontiguousarray(dist), img.copy(), sg)

    # in-memory multisurface (mmr) bodies of tm_func: calculate_tfce (one sweep
    # over the merged adjacency of all surfaces, each surface scaled by its own
    # max), calc_mixed_tfce (one merged sweep per TFCE setting) and
    # calculate_mediation_tfce, observed and randomised.  Three surfaces: an
    # icosphere-3 mesh (full mask), an icosphere-2 mesh with masked-out
    # vertices and a small voxel volume (26-neighbour mmr lists).  The
    # randomised calls seed from the clock (tm_func.py:57); the module's
    # `time` is replaced by a constant so the seeds, and the CSV lines they
    # give, are reproducible.
    if "tm_func" in R:
        tmf = R["tm_func"]
        rm = np.random.default_rng(81)
        va, fa = synth.icosphere(3)
        vb, fb = synth.icosphere(2)
        oa, ia = A.mesh_csr(fa, va.shape[0])
        ob, ib = A.mesh_csr(fb, vb.shape[0])
        vol = np.zeros((7, 6, 5), bool)
        vol[1:6, 1:5, 1:4] = True
        vol[0, 0, 0] = True
        vol[3, 3, 4] = True
        adj_vol = A.create_adjac_voxel_mmr(vol, 26)
        mask_b = np.ones(vb.shape[0], bool)
        mask_b[rm.choice(vb.shape[0], 30, replace=False)] = False
        masks = np.empty(3, dtype=object)
        masks[0] = np.ones((va.shape[0], 1, 1), bool)
        masks[1] = mask_b[:, None, None]
        masks[2] = vol
        def obj_lists(lists):  # adjacency sets as the TMI reader returns them: object arrays of lists
            o = np.empty(len(lists), dtype=object)
            for i_, a_ in enumerate(lists):
                o[i_] = list(a_)
            return o

        adjs = np.empty(3, dtype=object)
        adjs[0] = obj_lists(A.from_csr(oa, ia))
        adjs[1] = obj_lists(A.from_csr(ob, ib))
        adjs[2] = obj_lists([sorted(a) for a in adj_vol])
        nm = 36
        Sa, Sb = synth.smoothing_matrix(oa, ia), synth.smoothing_matrix(ob, ib)
        ya = rm.standard_normal((va.shape[0], nm)).astype(np.float32)
        yb = rm.standard_normal((vb.shape[0], nm)).astype(np.float32)
        for _ in range(3):
            ya, yb = (Sa @ ya).astype(np.float32), (Sb @ yb).astype(np.float32)
        yv = rm.standard_normal((int(vol.sum()), nm)).astype(np.float32)
        xm = np.column_stack([np.repeat([0.0, 1.0], nm // 2), rm.standard_normal(nm)])
        ym = np.concatenate([ya, yb[mask_b], yv]).T.astype(np.float32)
        ym[:, :120] += (0.9 * xm[:, 0])[:, None].astype(np.float32)
        ym[:, 650:690] -= (0.7 * xm[:, 1])[:, None].astype(np.float32)
        pos = tmf.create_position_array(masks)
        full = tmf.create_full_mask(masks)
        vd = []
        for i in range(3):
            deg = np.array([len(a) for a in adjs[i]], np.float64)
            if masks[i].shape[2] == 1:
                deg = deg[masks[i][:, 0, 0]]
            vd = np.hstack((vd, np.array(1 - deg / deg.max() + deg.mean() / deg.max(), np.float32)))
        out["mmr_y"], out["mmr_x"], out["mmr_pos"], out["mmr_full"], out["mmr_vd"] = ym, xm, np.array(pos), full, vd
        out["mmr_mask_b"], out["mmr_vol"] = mask_b, vol
        out["mmr_adj_vol_off"], out["mmr_adj_vol_idx"] = A.to_csr(adjs[2])
        op = tfce.CreateAdjSet(2.0, 1.0, tmf.merge_adjacency_array(range(3), adjs))
        permm = np.random.RandomState(83).permutation(nm)
        out["mmr_perm"] = permm
        for tag, vdx, px in (("obs", 1, xm), ("vd", vd, xm), ("perm", 1, xm[permm])):
            tv, tp, tn = tmf.calculate_tfce(ym, masks, px, op, vdx, pos, full)
            out[f"mmr_calc_t_{tag}"], out[f"mmr_calc_pos_{tag}"], out[f"mmr_calc_neg_{tag}"] = tv, tp, tn
        tmf.np = _OldNumpyArray()
        assign = np.array([0, 0, 1])
        settings = [(2.0, 1.0), (2.0, 0.5)]
        ops = []
        for i in range(2):
            sel = assign == i
            ops.append(tfce.CreateAdjSet(settings[i][0], settings[i][1],
                                         tmf.merge_adjacency_array(np.arange(3)[sel], adjs[sel])))
        out["mmr_mixed_assign"], out["mmr_mixed_settings"] = assign, np.array(settings)
        res = tmf.calc_mixed_tfce(assign, ym, masks, pos, 1, xm, ops)
        out["mmr_mixed_obs"] = np.asarray(res[2])  # the reference returns one array three times
        xb, dyb = xm[:, 0], (0.5 * xm[:, 0] + rm.standard_normal(nm))
        out["mmr_med_x"], out["mmr_med_dy"] = xb, dyb
        with np.errstate(all="ignore"):
            z, tz = tmf.calculate_mediation_tfce("M", ym, masks, xb, dyb, op, 1, pos, full)
        out["mmr_med_z"], out["mmr_med_tfce"] = z, tz
        tmf.time = lambda: 1700000000.25  # str(...)[-6:] = '000.25' -> seed = perm_number + 25
        out["mmr_time_seed_offset"] = np.int64(25)
        with tempfile.TemporaryDirectory() as td:
            cwd = os.getcwd()
            os.chdir(td)
            try:
                for pn in (0, 1):
                    tmf.calculate_tfce(ym, masks, xm, op, 1, pos, full, perm_number=pn, randomise=True)
                for s_ in range(3):
                    for c in (1, 2):
                        out[f"mmr_csv_calc_s{s_}_c{c}"] = np.array(open(f"perm_maxTFCE_surf{s_}_tcon{c}.csv").read())
                        os.remove(f"perm_maxTFCE_surf{s_}_tcon{c}.csv")
                for pn in (0, 1):
                    tmf.calc_mixed_tfce(assign, ym, masks, pos, 1, xm, ops, perm_number=pn, randomise=True)
                for s_ in range(3):
                    for c in (1, 2):
                        out[f"mmr_csv_mixed_s{s_}_c{c}"] = np.array(open(f"perm_maxTFCE_surf{s_}_tcon{c}.csv").read())
                with np.errstate(all="ignore"):
                    for pn in (0, 1):
                        tmf.calculate_mediation_tfce("M", ym, masks, xb, dyb, op, 1, pos, full, perm_number=pn,
                                                     randomise=True)
                for s_ in range(3):
                    out[f"mmr_csv_med_s{s_}"] = np.array(open(f"perm_maxTFCE_surf{s_}_M_zstat.csv").read())
            finally:
                os.chdir(cwd)

    path = os.path.join(HERE, "reference_vectors.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path} ({os.path.getsize(path)} bytes, {len(out)} arrays)")


if __name__ == "__main__":
    main()
