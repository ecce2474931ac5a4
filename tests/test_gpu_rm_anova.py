"""tm-models repeated-measures ANCOVA on the GPU: the reg_rm_ancova_* drop-ins
against the reference's own outputs (golden vectors, incl. the in-place row
shuffle of a permuted call); the engine's F maps against the FP64 oracle for
permuted designs with the reference's cumulative row shuffles; the TFCE maxima
and the tm_models_randomise RM-ANCOVA driver against the oracle pipeline.

Bars: F |dF| <= 2e-4 * max(1, F) (effect sums of squares from split-BF16
betas, the reference's float32 SS_Total ~1e-5); per-permutation max-TFCE
relative error <= 1e-3 every value, median <= 1e-4."""
import numpy as np
import pytest

from oracle import oracle
from tfce_mediation_gb300 import adjacency as A
from tfce_mediation_gb300 import pyfunc, randomise, synth
from tfce_mediation_gb300 import rm_anova as R

pytestmark = pytest.mark.gpu


def _scaled(a, ref):
    return float(np.max(np.abs(np.asarray(a, np.float64) - ref) / np.maximum(1.0, np.abs(ref))))


def _golden_call(golden, two, tag, kind, seed):
    pre = "rm2" if two else "rm1"
    d = golden[f"{pre}_data"].copy()
    cov = golden[f"{pre}_cov"] if tag == "cov" else None
    ra = None
    if kind == "perm":
        np.random.seed(seed)
        ra = np.random.permutation(d.shape[1])
    if two:
        res = pyfunc.reg_rm_ancova_two_bs_factor(d, golden["rm2_fa"], golden["rm2_fb"], golden["rm2_subj"],
                                                 dmy_covariates=cov, verbose=False, rand_array=ra)
    else:
        res = pyfunc.reg_rm_ancova_one_bs_factor(d, golden["rm1_f1"], golden["rm1_subj"], dmy_covariates=cov,
                                                 verbose=False, rand_array=ra)
    return np.asarray(res), d


@pytest.mark.parametrize("two", [False, True])
@pytest.mark.parametrize("tag", ["nocov", "cov"])
@pytest.mark.parametrize("kind", ["obs", "perm"])
def test_rm_ancova_dropins_vs_reference(golden, two, tag, kind):
    got, _ = _golden_call(golden, two, tag, kind, 92 if two else 91)
    ref = golden[f"{'rm2' if two else 'rm1'}_{kind}_{tag}"]
    assert got.shape == ref.shape
    err = _scaled(got, ref)
    print("rm-ancova", two, tag, kind, err)
    assert err <= 2e-4, err


def test_rm_ancova_permuted_call_shuffles_caller_data(golden):
    d = golden["rm1_data"].copy()
    np.random.seed(93)
    ra = np.random.permutation(d.shape[1])
    pyfunc.reg_rm_ancova_one_bs_factor(d, golden["rm1_f1"], golden["rm1_subj"], verbose=False, rand_array=ra)
    np.testing.assert_array_equal(d, golden["rm1_after_perm"])


def test_rm_ancova_outputs_sig_and_residuals(golden):
    d = golden["rm1_data"]
    out = pyfunc.reg_rm_ancova_one_bs_factor(d.copy(), golden["rm1_f1"], golden["rm1_subj"], output_sig=True,
                                             verbose=False)
    assert len(out) == 6
    from scipy.stats import f as fdist
    n = d.shape[1]
    np.testing.assert_allclose(out[3], 1 - fdist.cdf(out[0], 1, n - 2), rtol=1e-6)
    F_a, F_s, F_sa, red = pyfunc.reg_rm_ancova_one_bs_factor(d.copy(), golden["rm1_f1"], golden["rm1_subj"],
                                                             output_reduced_residuals=True, verbose=False)
    s = d.shape[0]
    Y = d.reshape(s * n, -1).astype(np.float64)
    X = np.column_stack([np.ones(s * n), np.tile(golden["rm1_f1"], s)])
    want = Y - X @ np.linalg.lstsq(X, Y, rcond=None)[0]
    np.testing.assert_allclose(red, want, atol=2e-5)


def _surface_study(seed, n=40, s=3, level=4):
    rng = np.random.default_rng(seed)
    v, f = synth.icosphere(level)
    V = v.shape[0]
    off, idx = A.mesh_csr(f, V)
    S = synth.smoothing_matrix(off, idx)
    flat = rng.standard_normal((s * n, V))
    for _ in range(3):
        flat = (S @ flat.T).T
    d = flat.reshape(s, n, V) * 3.0
    g = rng.integers(0, 2, n)
    h = rng.integers(0, 3, n)
    d = d + 0.6 * rng.standard_normal(n)[None, :, None]
    d[s - 1, :, : V // 4] += (0.5 * g)[:, None]
    d[:, :, V // 2: V // 2 + V // 5] += (0.4 * (h == 1))[None, :, None]
    cov = rng.standard_normal((n, 1))
    subj = R.dummy_code(np.arange(n), demean=False)
    return d.astype(np.float32), R.dummy_code(g), R.dummy_code(h), subj, cov, off, idx


@pytest.mark.parametrize("two", [False, True])
def test_engine_fmaps_vs_fp64(two):
    d, fa, fb, subj, cov, off, idx = _surface_study(3)
    s, n, V = d.shape
    model = R.RMModel(n, s, fa, subj, dmy_factor2=fb if two else None, dmy_covariates=cov)
    eng = R.RMAncovaEngine(d.reshape(s * n, V), model)
    ras, cums = randomise.rm_permutations(n, n * s, 0, 10, 12)
    ras = [None] + list(ras)
    cums = np.concatenate([np.arange(n * s)[None], cums])
    got = eng.fmaps(ras, cums).cpu().numpy()
    eng.status()
    for p in (0, 1, 4, 10):
        kw = {} if ras[p] is None else dict(rand_array=ras[p], shuffle=cums[p])
        if two:
            ref = oracle.rm_ancova_two(d.astype(np.float64), fa, fb, subj, dmy_covariates=cov, **kw)
        else:
            ref = oracle.rm_ancova_one(d.astype(np.float64), fa, subj, dmy_covariates=cov, **kw)
        err = _scaled(got[p], np.asarray(ref))
        print("fmaps", two, p, err)
        assert err <= 2e-4, (p, err)


def test_engine_maxima_vs_oracle():
    d, fa, fb, subj, cov, off, idx = _surface_study(4)
    s, n, V = d.shape
    model = R.RMModel(n, s, fa, subj, dmy_covariates=cov)
    eng = R.RMAncovaEngine(d.reshape(s * n, V), model, (off, idx), H=2.0, E=1.0, batch=5)
    ras, cums = randomise.rm_permutations(n, n * s, 0, 8, 3)
    got = eng.maxima(list(ras), cums)[:, :, 0]  # (P, 3)
    ref = np.zeros_like(got)
    for p in range(len(ras)):
        F = oracle.rm_ancova_one(d.astype(np.float64), fa, subj, dmy_covariates=cov, rand_array=ras[p],
                                 shuffle=cums[p])
        for j in range(3):
            ref[p, j] = oracle.tfce_max_batch(off, idx, np.asarray(F[j], np.float32), 2.0, 1.0)[0]
    rel = np.abs(got - ref) / np.abs(ref)
    print("rm-ancova maxima: median", np.median(rel), "max", rel.max())
    assert np.median(rel) <= 1e-4
    assert rel.max() <= 1e-3


def test_tm_models_rmancova_driver_volume(tmp_path, monkeypatch):
    """tm_models_randomise -tfa drop-in on a small volume: CSV names and lines
    against the oracle pipeline on the same host-seeded permutations and
    cumulative row shuffles."""
    import argparse
    rng = np.random.default_rng(45)
    mask = np.zeros((9, 8, 7), bool)
    mask[1:8, 1:7, 1:6] = True
    off, idx = A.voxel_csr(mask, 26, "pyfunc")
    V, n, s = int(mask.sum()), 30, 2
    cells = rng.permutation(np.arange(n) % 4)  # every factor cell populated
    fa = R.dummy_code(cells % 2)
    fb = R.dummy_code(cells // 2)
    subj = R.dummy_code(np.arange(n), demean=False)
    data = rng.standard_normal((s, n, V)).astype(np.float32)
    data[1, :, :40] += (0.9 * (fa > 0))[:, None].astype(np.float32)
    d = tmp_path / "tmtemp_rmANCOVA2BS_volume"
    d.mkdir()
    np.save(d / "dmy_factor1.npy", fa)
    np.save(d / "dmy_factor2.npy", fb)
    np.save(d / "factors.npy", np.array(["grp", "x", "sex"]))
    np.save(d / "dmy_subjects.npy", subj)
    np.save(d / "dformat.npy", np.array(["short"]))
    np.save(d / "data.npy", data)
    np.save(d / "optstfce.npy", np.array([2.0, 0.5]))
    np.save(d / "dmy_covariates.npy", np.array(None, dtype=object), allow_pickle=True)
    adj = np.empty(V, dtype=object)
    for v in range(V):
        adj[v] = np.asarray(idx[off[v]:off[v + 1]], np.int64)
    np.save(d / "adjac.npy", adj, allow_pickle=True)
    monkeypatch.chdir(tmp_path)
    opts = argparse.Namespace(range=[2, 6], surface=None, exchangeblock=None, seed=[8], batch=3,
                              twobetweenssubjectfactor=True)
    randomise.tm_models_rmancova_run(opts)
    out = tmp_path / "output_rmANCOVA2BS_volume" / "perm_rmANCOVA2BS"
    names = ["grp", "sex", "grp.X.sex", "time", "grp.X.time", "sex.X.time", "grp.X.sex.X.time"]
    csv = [np.loadtxt(out / f"perm_Fstat_{nm}_TFCE_maxVoxel.csv") for nm in names]
    ras, cums = randomise.rm_permutations(n, n * s, 2, 7, 8)
    for p in range(5):
        F = oracle.rm_ancova_two(data.astype(np.float64), fa, fb, subj, rand_array=ras[p], shuffle=cums[p])
        for j in range(7):
            ref = oracle.tfce_max_batch(off, idx, np.asarray(F[j], np.float32), 2.0, 0.5)[0]
            assert abs(csv[j][p] - ref) <= 1e-3 * abs(ref) + 1e-3, (names[j], p, csv[j][p], ref)


def test_long_format_equals_short(golden):
    """'long' data (n*s rows, interval-major) gives the short-format F maps."""
    d = golden["rm2_data"]
    s, n, V = d.shape
    short = pyfunc.reg_rm_ancova_two_bs_factor(d.copy(), golden["rm2_fa"], golden["rm2_fb"], golden["rm2_subj"],
                                               dmy_covariates=golden["rm2_cov"], verbose=False)
    long_ = pyfunc.reg_rm_ancova_two_bs_factor(d.reshape(s * n, V).copy(), golden["rm2_fa"], golden["rm2_fb"],
                                               golden["rm2_subj"], dmy_covariates=golden["rm2_cov"],
                                               data_format="long", verbose=False)
    np.testing.assert_array_equal(np.asarray(short), np.asarray(long_))
