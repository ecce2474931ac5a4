"""Pin the oracle (and the host-side builders) to the reference's own outputs.

tests/golden/reference_vectors.npz was produced by tests/golden/make_golden.py
from the reference's compiled modules and unmodified Python; every oracle
function used by the GPU parity tests is checked against it here, on CPU.
When oracle/_ref (the reference sweep compiled from a reference checkout) is
present, the oracle sweep is also compared against it directly.
"""
import numpy as np
import pytest

from oracle import oracle
from tfce_mediation_gb300 import adjacency as A
from tfce_mediation_gb300 import synth


def test_sweep_matches_reference_bitwise(golden):
    maps, params = golden["sweep_maps"], golden["sweep_params"]
    for pi, (H, E) in enumerate(params):
        for mi in range(maps.shape[0]):
            if maps[mi].max() == 0:
                continue
            e = oracle.tfce(golden["sweep_off"], golden["sweep_idx"], maps[mi], float(H), float(E))
            np.testing.assert_array_equal(e, golden["sweep_enhn"][pi, mi], err_msg=f"H={H} E={E} map {mi}")


def test_sweep_accumulates_into_enhn(golden):
    e = golden["sweep_accum_in"].copy()
    oracle.tfce(golden["sweep_off"], golden["sweep_idx"], golden["sweep_maps"][2], 2.0, 1.0, enhn=e)
    np.testing.assert_array_equal(e, golden["sweep_accum_out"])


def test_sweep_all_nonpositive_map_is_zero(golden):
    m = golden["sweep_maps"][5]
    assert m.max() <= 0
    e = oracle.tfce(golden["sweep_off"], golden["sweep_idx"], m, 2.0, 1.0)
    assert not e.any()


def test_threshold_table_recurrence():
    T = oracle.threshold_table(4.2)
    assert T[0] == np.float32(4.2)
    dT = np.float32(4.2) / np.float32(100)
    for a, b in zip(T[:-1], T[1:]):
        assert b == np.float32(a - dT)
    assert T[-1] >= 0 and np.float32(T[-1] - dT) < 0
    assert len(T) in (100, 101)
    assert len(oracle.threshold_table(0.0)) == 0
    assert len(oracle.threshold_table(-1.0)) == 0


def test_labels_are_consistent_partitions(golden):
    m = golden["sweep_maps"][0]
    enhn, labels, extents = oracle.tfce_labels(golden["sweep_off"], golden["sweep_idx"], m, 2.0, 1.0)
    assert labels.shape[0] == len(oracle.threshold_table(float(m.max())))
    for s in range(labels.shape[0]):
        lab = labels[s]
        act = lab >= 0
        _, inv, cnt = np.unique(lab[act], return_inverse=True, return_counts=True)
        np.testing.assert_array_equal(extents[s][act], cnt[inv])
    np.testing.assert_array_equal(enhn, golden["sweep_enhn"][0, 0])


def test_sweep_against_reference_build(golden):
    if oracle.ref_lib() is None:
        pytest.skip("oracle/_ref not built (no reference checkout here)")
    st = synth.config1()
    t = oracle.tval_fp64(st.design(), st.Y)
    for c in (1, 2):
        for s in (1, -1):
            img = (s * t[c]).astype(np.float32)
            for H, E in ((2.0, 1.0), (2.0, 0.5), (1.0, 0.67)):
                a = oracle.tfce(st.offsets, st.indices, img, H, E)
                b = oracle.ref_tfce(st.offsets, st.indices, img, H, E)
                np.testing.assert_array_equal(a, b)


def test_glm_helpers(golden):
    y, x = golden["glm_y"], golden["glm_x"]
    n, V = y.shape
    X = np.column_stack([np.ones(n), x])
    invXX = np.linalg.inv(X.T @ X)
    np.testing.assert_array_equal(oracle.tval_int_ref(X, invXX, y, n, X.shape[1]), golden["glm_tval_int"])
    np.testing.assert_allclose(oracle.tval_fp64(X, y), golden["glm_tval_int"], rtol=1e-6, atol=1e-6)
    b, se = oracle.calc_beta_se(x[:, 0], y, n)
    np.testing.assert_array_equal(b, golden["glm_cbs_beta"])
    np.testing.assert_array_equal(se, golden["glm_cbs_se"])
    np.testing.assert_array_equal(oracle.lstsqr_mat(X, y), golden["glm_lstsqr"])
    np.testing.assert_allclose(oracle.calcF(X, y, n, X.shape[1]), golden["glm_calcF"], rtol=1e-12)
    np.testing.assert_allclose(oracle.resid_covars(X[:, :2], y.T), golden["glm_resid_covars"], rtol=1e-12,
                               atol=1e-12)


def test_sobel(golden):
    n = golden["sobel_x"].shape[0]
    for mt in ("I", "M", "Y"):
        for alg in ("aroian", "sobel", "goodman"):
            with np.errstate(all="ignore"):
                z = oracle.calc_sobelz(mt, golden["sobel_x"], golden["sobel_dy"], golden["sobel_y"], n, alg)
            np.testing.assert_allclose(z, golden[f"sobel_{mt}_{alg}"], rtol=1e-12, equal_nan=True)


def test_perm_max_csv(golden):
    """write_perm_maxTFCE_vertex/voxel values, formatted as the reference formats them."""
    off, idx = golden["sweep_off"], golden["sweep_idx"]
    stat, mask_rh, vd = golden["perm_stat"], golden["perm_mask_rh"], golden["perm_vd"]
    Vh = off.shape[0] - 1
    nl = Vh

    def full(sign, vdens=None):
        lh = np.zeros(Vh, np.float32)
        rh = np.zeros(Vh, np.float32)
        lh[:] = sign * stat[:nl]
        rh[mask_rh] = sign * stat[nl:]
        segs = [(off, idx, 0, Vh)]
        v = []
        for arr in (lh, rh):
            e = oracle.tfce(off, idx, arr, 2.0, 1.0)
            val = e * (arr[np.isfinite(arr)].max() / np.float32(100))
            if vdens is not None:
                val = val * vdens
            v.append(val.max())
        return max(v)

    lines1 = "%.4f\n%.4f\n" % (full(1), full(-1))
    assert lines1 == str(golden["perm_csv_vertex1"])
    assert "%.4f\n" % full(1, vd) == str(golden["perm_csv_vertex2"])
    m3 = golden["sweep_maps"][3].astype(np.float64).astype(np.float32)
    vox = oracle.tfce_max_batch(off, idx, m3, 2.0, 1.0)[0]
    assert "%1.4f\n" % vox == str(golden["perm_csv_voxel1"])


def test_fwer_lookups(golden):
    null, img = golden["fwe_null"], golden["fwe_img"]
    np.testing.assert_array_equal(oracle.fwep_vertex(img, null), golden["fwe_vertex"])
    srt = np.sort(null)
    p_array = np.arange(len(srt)) / len(srt)
    np.testing.assert_array_equal(np.array([oracle.find_nearest(srt, k, p_array) for k in img]),
                                  golden["fwe_nearest"])


@pytest.mark.parametrize("weight", [None, "logmasksize"])
def test_apply_mfwer(golden, weight):
    images = golden["mfwer_images"]
    perm = golden["mfwer_perm"]
    pos = list(golden["mfwer_pos_array"])
    pm = {}
    k = 0
    for s in range(3):
        for c in range(2):
            pm[(s, c)] = perm[k]
            k += 1
    p, q = oracle.apply_mfwer(images[:, [0, 1]], images[:, [2, 3]], pm, pos, weight=weight)
    np.testing.assert_array_equal(p, golden[f"mfwer_pos_{weight}"])
    np.testing.assert_array_equal(q, golden[f"mfwer_neg_{weight}"])


# ---- host-side builders of the product against the reference's builders ----
def test_mesh_adjacency_builder(golden):
    off, idx = A.mesh_csr(golden["adj_mesh_faces"], int(golden["adj_mesh_nv"]))
    np.testing.assert_array_equal(off, golden["adj_mesh_off"])
    np.testing.assert_array_equal(idx, golden["adj_mesh_idx"])


@pytest.mark.parametrize("dirtype", [6, 26])
def test_voxel_adjacency_builders(golden, dirtype):
    mask = golden["vox_mask"]
    off, idx = A.voxel_csr(mask, dirtype, "pyfunc")
    np.testing.assert_array_equal(off, golden[f"vox{dirtype}_off"])
    np.testing.assert_array_equal(idx, golden[f"vox{dirtype}_idx"])
    off, idx = A.voxel_csr(mask, dirtype, "mmr")
    np.testing.assert_array_equal(off, golden[f"voxmmr{dirtype}_off"])
    np.testing.assert_array_equal(idx, golden[f"voxmmr{dirtype}_idx"])


@pytest.mark.parametrize("tag", ["obs", "perm"])
def test_glm_typeI(golden, tag):
    """The FP64 restatement of glm_typeI against the reference's own outputs
    (model F, drop-one F per variable, t with float32 SE)."""
    ra = None if tag == "obs" else golden["typeI_perm"]
    F, Fv, T = oracle.glm_typeI(golden["typeI_y"], [golden["typeI_ex0"], golden["typeI_ex1"]],
                                dmy_covariates=golden["typeI_cov"], rand_array=ra)
    np.testing.assert_allclose(F, golden[f"typeI_F_{tag}"], rtol=1e-9)
    np.testing.assert_allclose(Fv, golden[f"typeI_Fvar_{tag}"], rtol=1e-8, atol=1e-10)
    np.testing.assert_allclose(T, golden[f"typeI_T_{tag}"], rtol=1e-12)


def test_partial_f_is_glm_typeI_drop_one(golden):
    y = golden["typeI_y"]
    n = y.shape[0]
    X = np.column_stack([np.ones(n), golden["typeI_ex0"], golden["typeI_ex1"], golden["typeI_cov"]])
    Fv = oracle.partial_f_fp64(X, y, [(1, 2), (3, 1)])
    np.testing.assert_allclose(Fv, golden["typeI_Fvar_obs"], rtol=1e-8, atol=1e-10)


_COS_NAMES = ("R2", "MESOR", "SE_MESOR", "AMP", "SE_AMP", "ACRO", "SE_ACRO", "F", "tMESOR", "tAMP", "tACRO",
              "tEXOG")


@pytest.mark.parametrize("tag", ["obs", "perm"])
def test_glm_cosinor(golden, tag):
    """The FP64 restatement of glm_cosinor against the reference's own 12-tuple
    (two periods, one exogenous variable, one covariate; the permuted call
    skips the quadrant rule and R2, as the reference does)."""
    ra = None if tag == "obs" else golden["cos_perm"]
    res = oracle.glm_cosinor(golden["cos_y"], golden["cos_t"], exog=[golden["cos_ex"]],
                             dmy_covariates=golden["cos_cov"], rand_array=ra, period=[24.0, 12.0],
                             calc_MESOR=ra is None)
    for name, val in zip(_COS_NAMES, res):
        key = f"cos_{name}_{tag}"
        if key not in golden:
            assert val is None, name
            continue
        np.testing.assert_allclose(val, golden[key], rtol=1e-9, atol=1e-12, err_msg=name)


def test_glm_cosinor_fit_only(golden):
    mesor, amp, acro = oracle.glm_cosinor(golden["cos_y"], golden["cos_t"], period=[24.0, 12.0],
                                          output_fit_only=True)
    np.testing.assert_allclose(mesor, golden["cos_fit_MESOR"], rtol=1e-12)
    np.testing.assert_allclose(amp, golden["cos_fit_AMP"], rtol=1e-12)
    np.testing.assert_allclose(acro, golden["cos_fit_ACRO"], rtol=1e-12)


def test_cosinor_program_forms(golden):
    """The closed forms of the tensor-core epilogue's cosinor rows (model F as
    the Wald partial F of every column after the intercept; amplitude and
    acrophase t without trigonometry) against the restatement, FP64."""
    y = np.asarray(golden["cos_y"], np.float64)
    X = oracle.cosinor_design(golden["cos_t"], [24.0, 12.0], [golden["cos_ex"]], golden["cos_cov"])
    X = X[golden["cos_perm"]]
    n, k = X.shape
    inv = np.linalg.inv(X.T @ X)
    b = inv @ X.T @ y
    rss = np.sum((y - X @ b) ** 2, 0)
    sigma = np.sqrt(rss / (n - k))
    res = oracle.glm_cosinor(golden["cos_y"], golden["cos_t"], exog=[golden["cos_ex"]],
                             dmy_covariates=golden["cos_cov"], rand_array=golden["cos_perm"],
                             period=[24.0, 12.0], calc_MESOR=False)
    S = slice(1, k)
    Fw = np.einsum("iv,ij,jv->v", b[S], np.linalg.inv(inv[S, S]), b[S]) / (k - 1) / (rss / (n - k))
    # the reference's SS_Total is a float32 sum: its rounding, amplified by the
    # SS_Total - RSS cancellation, moves its F by ~5e-6 relative here
    np.testing.assert_allclose(Fw, res[7], rtol=3e-5)
    for i in range(2):
        c, s = 1 + 2 * i, 2 + 2 * i
        a2 = b[c] ** 2 + b[s] ** 2
        cr = 2 * inv[c, s] * np.abs(b[c] * b[s])
        t_amp = a2 / (sigma * np.sqrt(inv[c, c] * b[c] ** 2 - cr + inv[s, s] * b[s] ** 2))
        t_acro = a2 / (sigma * np.sqrt(inv[c, c] * b[s] ** 2 + cr + inv[s, s] * b[c] ** 2))
        np.testing.assert_allclose(t_amp, res[9][i], rtol=1e-10)
        np.testing.assert_allclose(t_acro, res[10][i], rtol=1e-10)


@pytest.mark.parametrize("tag", ["nocov", "cov"])
@pytest.mark.parametrize("kind", ["obs", "perm"])
def test_rm_ancova_one(golden, tag, kind):
    """The FP64 restatement of reg_rm_ancova_one_bs_factor against the
    reference's (F_a, F_s, F_sa); the permuted call replays the reference's
    global-RNG row shuffle."""
    cov = golden["rm1_cov"] if tag == "cov" else None
    kw = {} if kind == "obs" else dict(rand_array=golden[f"rm1_ra_{tag}"], shuffle=golden[f"rm1_shuffle_{tag}"])
    got = oracle.rm_ancova_one(golden["rm1_data"], golden["rm1_f1"], golden["rm1_subj"], dmy_covariates=cov, **kw)
    np.testing.assert_allclose(np.asarray(got), golden[f"rm1_{kind}_{tag}"], rtol=1e-9)


@pytest.mark.parametrize("tag", ["nocov", "cov"])
@pytest.mark.parametrize("kind", ["obs", "perm"])
def test_rm_ancova_two(golden, tag, kind):
    cov = golden["rm2_cov"] if tag == "cov" else None
    kw = {} if kind == "obs" else dict(rand_array=golden[f"rm2_ra_{tag}"], shuffle=golden[f"rm2_shuffle_{tag}"])
    got = oracle.rm_ancova_two(golden["rm2_data"], golden["rm2_fa"], golden["rm2_fb"], golden["rm2_subj"],
                               dmy_covariates=cov, **kw)
    np.testing.assert_allclose(np.asarray(got), golden[f"rm2_{kind}_{tag}"], rtol=1e-9)


def test_rm_ancova_shuffles_caller_data_in_place(golden):
    """A permuted reg_rm_ancova_* call leaves the caller's short-format array
    shuffled: its long form is a view, and np.random.shuffle acts on it."""
    d = golden["rm1_data"]
    s, n, V = d.shape
    want = d.reshape(s * n, V)[golden["rm1_after_shuffle"]].reshape(s, n, V)
    np.testing.assert_array_equal(golden["rm1_after_perm"], want)


@pytest.mark.parametrize("k", [0, 1])
def test_calc_gd_fwhm(golden, k):
    """The restatement of calc_gd_fwhm (float32 accumulation in pair order,
    powf / expf weights) against the reference's own output, bit for bit."""
    got = oracle.calc_gd_fwhm(golden["gd_pairs"], golden["gd_dist"], golden[f"gd_data{k}"],
                              float(golden[f"gd_sigma{k}"]))
    np.testing.assert_array_equal(got, golden[f"gd_out{k}"])


@pytest.mark.parametrize("kind", ["obs", "perm"])
def test_rm_ancova_one_wider(golden, kind):
    """Three-level factor, two covariates, four intervals."""
    kw = {} if kind == "obs" else dict(rand_array=golden["rm3_ra"], shuffle=golden["rm3_shuffle"])
    got = oracle.rm_ancova_one(golden["rm3_data"], golden["rm3_f1"], golden["rm3_subj"],
                               dmy_covariates=golden["rm3_cov"], **kw)
    np.testing.assert_allclose(np.asarray(got), golden[f"rm3_{kind}"], rtol=1e-9)


@pytest.mark.parametrize("tag", ["obs", "perm"])
def test_glm_cosinor_two_exog(golden, tag):
    """Two periods, two exogenous variables (one of two columns), no covariate,
    calc_MESOR default."""
    ra = None if tag == "obs" else golden["cosw_perm"]
    res = oracle.glm_cosinor(golden["cosw_y"], golden["cosw_t"], exog=[golden["cosw_ex0"], golden["cosw_ex1"]],
                             rand_array=ra, period=[24.0, 8.0])
    for name, val in zip(_COS_NAMES, res):
        key = f"cosw_{name}_{tag}"
        if key not in golden:
            assert val is None, name
            continue
        np.testing.assert_allclose(val, golden[key], rtol=1e-9, atol=1e-12, err_msg=name)


# --- in-memory multisurface bodies (tm_func.calculate_tfce & co.) ----------
def _mmr():
    from tests.mmr_case import mmr_case
    return mmr_case


@pytest.mark.parametrize("tag", ["obs", "vd", "perm"])
def test_mmr_calculate_tfce(golden, tag):
    case = _mmr()(golden)
    vd = case["vd"] if tag == "vd" else 1
    perm = case["perm"] if tag == "perm" else None
    tv, tp, tn = oracle.calculate_tfce(case["y"], case["masks"], case["x"], case["adjs"], 2.0, 1.0, vd, perm=perm)
    np.testing.assert_allclose(tv, golden[f"mmr_calc_t_{tag}"], rtol=1e-6, atol=1e-6)
    # the same float32 t -> the sweep and scaling are the reference's arithmetic
    t_ref = golden[f"mmr_calc_t_{tag}"]
    np.testing.assert_array_equal(tv, t_ref)
    np.testing.assert_array_equal(tp, golden[f"mmr_calc_pos_{tag}"])
    np.testing.assert_array_equal(tn, golden[f"mmr_calc_neg_{tag}"])


def test_mmr_global_thresholds_differ_from_per_surface(golden):
    """One merged sweep (global dT) differs from sweeping each surface on its
    own, so the restatement must not be the per-surface one."""
    case = _mmr()(golden)
    _, tp, _ = oracle.calculate_tfce(case["y"], case["masks"], case["x"], case["adjs"], 2.0, 1.0, 1)
    pos = case["pos"]
    # surface 1 swept alone on its induced lists
    off, idx = A.induced_csr(A.to_csr(list(case["adjs"][1])), case["masks"][1][:, 0, 0])
    t1 = oracle.calculate_tfce(case["y"], case["masks"], case["x"], case["adjs"], 2.0, 1.0, 1)[0][0, pos[1]:pos[2]]
    alone = oracle.tfce(off, idx, t1, 2.0, 1.0) * (t1.max() / np.float32(100))
    assert not np.array_equal(alone, tp[0, pos[1]:pos[2]])


def test_mmr_calc_mixed_tfce(golden):
    case = _mmr()(golden)
    settings = [tuple(s) for s in golden["mmr_mixed_settings"]]
    _, _, tn = oracle.calc_mixed_tfce(golden["mmr_mixed_assign"], case["y"], case["masks"], case["adjs"], settings,
                                      case["x"], 1)
    # the reference hands back one array three times, holding the negative maps
    np.testing.assert_array_equal(tn.astype(np.float64), golden["mmr_mixed_obs"])


def test_mmr_calculate_mediation_tfce(golden):
    case = _mmr()(golden)
    z, tz = oracle.calculate_mediation_tfce("M", case["y"], case["masks"], golden["mmr_med_x"], golden["mmr_med_dy"],
                                            case["adjs"], 2.0, 1.0, 1)
    np.testing.assert_allclose(z, golden["mmr_med_z"], rtol=2e-6, atol=2e-6)
    np.testing.assert_allclose(tz, golden["mmr_med_tfce"], rtol=2e-5, atol=1e-6)


def _replayed_perm(n, pn, offset):
    np.random.seed(pn + offset)
    return np.random.permutation(list(range(n)))


def test_mmr_randomised_csv_lines(golden):
    """The randomised calls (clock seed replaced by a constant): per surface
    and contrast, + then - maxima of every permutation, '%f'."""
    from tests.mmr_case import csv_values
    case = _mmr()(golden)
    off = int(golden["mmr_time_seed_offset"])
    n = case["y"].shape[0]
    got = {(s, c): [] for s in range(3) for c in (1, 2)}
    mixed = {(s, c): [] for s in range(3) for c in (1, 2)}
    settings = [tuple(s) for s in golden["mmr_mixed_settings"]]
    for pn in (0, 1):
        perm = _replayed_perm(n, pn, off)
        _, tp, tn = oracle.calculate_tfce(case["y"], case["masks"], case["x"], case["adjs"], 2.0, 1.0, 1, perm=perm)
        mp, mn = oracle.surface_maxima(tp, case["pos"]), oracle.surface_maxima(tn, case["pos"])
        _, tp2, tn2 = oracle.calc_mixed_tfce(golden["mmr_mixed_assign"], case["y"], case["masks"], case["adjs"],
                                             settings, case["x"], 1, perm=perm)
        mp2, mn2 = oracle.surface_maxima(tp2, case["pos"]), oracle.surface_maxima(tn2, case["pos"])
        for s in range(3):
            for c in (1, 2):
                got[(s, c)] += ["%f" % mp[c - 1, s], "%f" % mn[c - 1, s]]
                mixed[(s, c)] += ["%f" % mp2[c - 1, s], "%f" % mn2[c - 1, s]]
    for s in range(3):
        for c in (1, 2):
            assert got[(s, c)] == str(golden[f"mmr_csv_calc_s{s}_c{c}"]).split(), (s, c)
            assert mixed[(s, c)] == str(golden[f"mmr_csv_mixed_s{s}_c{c}"]).split(), (s, c)
    for s in range(3):
        vals = []
        for pn in (0, 1):
            perm = _replayed_perm(n, pn, off)
            _, tz = oracle.calculate_mediation_tfce("M", case["y"], case["masks"], golden["mmr_med_x"],
                                                    golden["mmr_med_dy"], case["adjs"], 2.0, 1.0, 1, perm=perm)
            vals.append(oracle.surface_maxima(tz, case["pos"])[s])
        np.testing.assert_allclose(vals, csv_values(golden[f"mmr_csv_med_s{s}"]), rtol=2e-5, atol=2e-6)
