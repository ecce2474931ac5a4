"""tm-models cosinor on the GPU: the tensor-core GLM's programmed epilogue
(model F, amplitude / acrophase t, +/- t) against the FP64 oracle; the
glm_cosinor drop-in against the reference's own outputs (golden vectors); the
engine's programmed maps and the tm_models_randomise cosinor driver against
the oracle pipeline (FP64 glm_cosinor + C sweep).

Bars: programmed rows |d| <= 2e-4 * max(1, |x|) (split-BF16 betas, FP32
residuals); drop-in statistics |d| <= 1e-4 * max(1, |x|) (FP32 CUDA-core GLM;
the reference forms SS_Total in float32), acrophase angles |d| <= 1e-4 rad;
per-permutation max-TFCE relative error <= 1e-3 every value, median <= 1e-4."""
import numpy as np
import pytest

from oracle import oracle
from tfce_mediation_gb300 import engine as E
from tfce_mediation_gb300 import pyfunc
from tfce_mediation_gb300.glm import DesignBatch, glm_stat_tc
from tfce_mediation_gb300.randomise import cosinor_outputs

pytestmark = pytest.mark.gpu

_NAMES = ("R2", "MESOR", "SE_MESOR", "AMP", "SE_AMP", "ACRO", "SE_ACRO", "F", "tMESOR", "tAMP", "tACRO",
          "tEXOG")


def _scaled(a, ref):
    return float(np.max(np.abs(np.asarray(a, np.float64) - ref) / np.maximum(1.0, np.abs(ref))))


def _study(seed, n, V, n_per=2):
    rng = np.random.default_rng(seed)
    tv = rng.uniform(0.0, 48.0, n)
    Y = (6.0 + rng.standard_normal((n, V))).astype(np.float32)
    Y[:, :V // 5] += (1.2 * np.cos(2.0 * np.pi * (tv - 5.0) / 24.0))[:, None].astype(np.float32)
    if n_per > 1:
        Y[:, V // 5:V // 3] += (0.8 * np.sin(2.0 * np.pi * tv / 12.0))[:, None].astype(np.float32)
    ex = rng.standard_normal(n)
    cov = rng.standard_normal((n, 1))
    Y[:, -V // 6:] += (0.5 * ex)[:, None].astype(np.float32)
    return rng, tv, Y, ex, cov


@pytest.mark.parametrize("with_mesor", [False, True])
def test_program_rows_vs_fp64(with_mesor):
    """Model F, amplitude / acrophase t of two periods and +/- t of the exog
    column for 24 permuted designs; with an extra t row of the intercept the
    kernel runs the uncentred residual form."""
    rng, tv, Y, ex, cov = _study(5, 130, 4000)
    periods = [24.0, 12.0]
    X = pyfunc.cosinor_design(tv, periods, [ex], cov)
    outs = cosinor_outputs(2, 1, 1) + ([("t", 0)] if with_mesor else [])
    perms = np.stack([rng.permutation(130) for _ in range(24)])
    got = glm_stat_tc(Y, DesignBatch(X[perms]), "program", outputs=outs).cpu().numpy()
    for g in range(0, 24, 5):
        res = oracle.glm_cosinor(Y, tv, exog=[ex], dmy_covariates=cov, rand_array=perms[g], period=periods,
                                 calc_MESOR=True)
        F, tM, tA, tP, tE = res[7], res[8], res[9], res[10], res[11]
        assert _scaled(got[g, 0], F) <= 2e-4, _scaled(got[g, 0], F)
        for i in range(2):
            assert _scaled(got[g, 1 + 2 * i], tA[i]) <= 2e-4, ("amp", i, _scaled(got[g, 1 + 2 * i], tA[i]))
            assert _scaled(got[g, 2 + 2 * i], tP[i]) <= 2e-4, ("acro", i, _scaled(got[g, 2 + 2 * i], tP[i]))
        assert _scaled(got[g, 5], tE[0]) <= 2e-4
        np.testing.assert_array_equal(got[g, 6], -got[g, 5])
        if with_mesor:
            assert _scaled(got[g, 7], tM) <= 2e-4


def test_program_bad_rows_are_nan():
    """A row whose columns or weights fall outside the design yields NaN, the
    other rows are unaffected."""
    rng, tv, Y, ex, cov = _study(6, 64, 600, n_per=1)
    X = pyfunc.cosinor_design(tv, [24.0], [ex], cov)  # k = 5
    db = DesignBatch(X[None])
    good = glm_stat_tc(Y, db, "program", outputs=[("amp", 1)]).cpu().numpy()
    got = glm_stat_tc(Y, db, "program", outputs=[("amp", 4), ("amp", 1), ("f", 3, 4)]).cpu().numpy()
    assert np.all(np.isnan(got[0, 0])) and np.all(np.isnan(got[0, 2]))
    np.testing.assert_array_equal(got[0, 1], good[0, 0])


@pytest.mark.parametrize("tag", ["obs", "perm"])
def test_glm_cosinor_vs_reference(golden, tag):
    ra = None if tag == "obs" else golden["cos_perm"]
    res = pyfunc.glm_cosinor(golden["cos_y"], golden["cos_t"], exog=[golden["cos_ex"]],
                             dmy_covariates=golden["cos_cov"], rand_array=ra, period=[24.0, 12.0],
                             calc_MESOR=ra is None)
    for name, val in zip(_NAMES, res):
        key = f"cos_{name}_{tag}"
        if key not in golden:
            assert val is None, name
            continue
        ref = np.asarray(golden[key], np.float64)
        assert np.shape(val) == ref.shape, name
        err = _scaled(val, ref)
        assert err <= 1e-4, (name, err)


def test_glm_cosinor_fit_only(golden):
    mesor, amp, acro = pyfunc.glm_cosinor(golden["cos_y"], golden["cos_t"], period=[24.0, 12.0],
                                          output_fit_only=True)
    assert _scaled(mesor, golden["cos_fit_MESOR"]) <= 1e-5
    assert _scaled(amp, golden["cos_fit_AMP"]) <= 1e-4
    assert np.max(np.abs(acro - golden["cos_fit_ACRO"])) <= 1e-4


def test_engine_cosinor_maps_vs_oracle(config1):
    """PermutationEngine(outputs=...) maxima of every programmed map against the
    oracle's glm_cosinor maps swept by the C oracle, one sign each (the
    reference sweeps -t as its own map); also through the captured graphs."""
    st = config1
    n = st.n
    rng = np.random.default_rng(8)
    tv = rng.uniform(0.0, 24.0, n)
    Y = st.Y.copy()
    Y[:, : st.Y.shape[1] // 3] += (0.9 * np.cos(2.0 * np.pi * (tv - 2.0) / 24.0))[:, None].astype(np.float32)
    ex = st.pred_x[:, 1]
    X = pyfunc.cosinor_design(tv, [24.0], [ex])
    outs = cosinor_outputs(1, 1)
    eng = E.PermutationEngine(Y, X[:, 1:], (st.offsets, st.indices), st.segments, 2.0, 1.0, batch=8,
                              outputs=outs)
    perms = E.permutations(n, 17, 0, 12)
    got = eng.run(perms=perms)[:, :, 0, :]  # (P, C, S)
    np.testing.assert_allclose(eng.run_graph(perms=perms)[:, :, 0, :], got, rtol=1e-6)
    ref = np.zeros_like(got)
    for p in range(perms.shape[0]):
        res = oracle.glm_cosinor(Y, tv, exog=[ex], rand_array=perms[p], period=[24.0], calc_MESOR=False)
        maps = [res[7], res[9][0], res[10][0], res[11][0], -res[11][0]]
        for ci, m in enumerate(maps):
            img = m.astype(np.float32)
            for h in range(len(st.segments) - 1):
                v0, v1 = int(st.segments[h]), int(st.segments[h + 1])
                off = st.offsets[v0:v1 + 1] - st.offsets[v0]
                idx = st.indices[st.offsets[v0]:st.offsets[v1]] - v0
                ref[p, ci, h] = oracle.tfce_max_batch(off, idx, img[v0:v1], 2.0, 1.0)[0]
    rel = np.abs(got - ref) / np.abs(ref)
    print("cosinor maxima: median", np.median(rel), "max", rel.max())
    assert np.median(rel) <= 1e-4
    assert rel.max() <= 1e-3


def test_tm_models_cosinor_driver_volume(tmp_path, monkeypatch):
    """tm_models_randomise cosinor branch drop-in on a small volume: the CSV
    files and lines against the oracle pipeline on the same host-seeded
    permutations."""
    import argparse
    from tfce_mediation_gb300 import adjacency as A
    from tfce_mediation_gb300 import randomise
    rng = np.random.default_rng(44)
    mask = np.zeros((10, 9, 8), bool)
    mask[1:9, 1:8, 1:7] = True
    off, idx = A.voxel_csr(mask, 26, "pyfunc")
    V, n = int(mask.sum()), 48
    tv = rng.uniform(0.0, 24.0, n)
    ex = rng.standard_normal((n, 1))
    data = rng.standard_normal((n, V)).astype(np.float32)
    data[:, :80] += (1.0 * np.cos(2.0 * np.pi * tv / 24.0))[:, None].astype(np.float32)
    d = tmp_path / "tmtemp_cosinor_volume"
    d.mkdir()
    np.save(d / "time_var.npy", tv)
    np.save(d / "period.npy", np.array([24.0]))
    np.save(d / "exog_flat.npy", ex)
    np.save(d / "exog_shape.npy", np.array([1]))
    np.save(d / "varnames.npy", np.array(["age"]))
    np.save(d / "data.npy", data)
    np.save(d / "optstfce.npy", np.array([2.0, 0.5]))
    np.save(d / "dmy_covariates.npy", np.array(None, dtype=object), allow_pickle=True)
    adj = np.empty(V, dtype=object)
    for v in range(V):
        adj[v] = np.asarray(idx[off[v]:off[v + 1]], np.int64)
    np.save(d / "adjac.npy", adj, allow_pickle=True)
    monkeypatch.chdir(tmp_path)
    opts = argparse.Namespace(range=[0, 4], surface=None, exchangeblock=None, seed=[21], batch=4)
    randomise.tm_models_cosinor_run(opts)
    out = tmp_path / "output_cosinor_volume" / "perm_cosinor"
    csv = {nm: np.loadtxt(out / f"perm_{nm}_TFCE_maxVoxel.csv")
           for nm in ("Fstat_model", "Tstat_amplitude_24.00", "Tstat_acrophase_24.00", "Tstat_age")}
    assert csv["Tstat_age"].shape == (10,)
    for p in range(5):
        perm = np.random.RandomState(21 + p).permutation(n)
        res = oracle.glm_cosinor(data, tv, exog=[ex], rand_array=perm, period=[24.0], calc_MESOR=False)
        checks = [("Fstat_model", p, res[7]), ("Tstat_amplitude_24.00", p, res[9][0]),
                  ("Tstat_acrophase_24.00", p, res[10][0]), ("Tstat_age", 2 * p, res[11][0]),
                  ("Tstat_age", 2 * p + 1, -res[11][0])]
        for nm, row, m in checks:
            ref = oracle.tfce_max_batch(off, idx, m.astype(np.float32), 2.0, 0.5)[0]
            assert abs(csv[nm][row] - ref) <= 1e-3 * abs(ref) + 1e-3, (nm, p, csv[nm][row], ref)
