"""tm-models GLM (glm_typeI) on the GPU: the drop-one F per variable on the
tensor-core GLM (Wald form), the model F and t, against the reference's own
outputs (golden vectors) and the FP64 oracle; the engine's F mode against
the oracle pipeline.

Bars: drop-one F |dF| <= 2e-4 * max(1, F) (split-BF16 betas, FP32 residuals);
model F and t |d| <= 1e-4 * max(1, |x|) (FP32 CUDA-core GLM; the reference
forms SS_Total in float32); per-permutation max-TFCE of F maps: relative
error <= 1e-3 every value, median <= 1e-4."""
import numpy as np
import pytest

from oracle import oracle
from tfce_mediation_gb300 import engine as E
from tfce_mediation_gb300 import pyfunc
from tfce_mediation_gb300.glm import DesignBatch, glm_stat_tc

pytestmark = pytest.mark.gpu


def _scaled(a, ref):
    return float(np.max(np.abs(np.asarray(a, np.float64) - ref) / np.maximum(1.0, np.abs(ref))))


@pytest.mark.parametrize("tag", ["obs", "perm"])
def test_glm_typeI_vs_reference(golden, tag):
    ra = None if tag == "obs" else golden["typeI_perm"]
    F, Fv, T = pyfunc.glm_typeI(golden["typeI_y"], [golden["typeI_ex0"], golden["typeI_ex1"]],
                                dmy_covariates=golden["typeI_cov"], output_tvalues=True, verbose=False,
                                rand_array=ra)
    assert _scaled(F, golden[f"typeI_F_{tag}"]) <= 1e-4
    assert _scaled(Fv, golden[f"typeI_Fvar_{tag}"]) <= 2e-4, _scaled(Fv, golden[f"typeI_Fvar_{tag}"])
    assert _scaled(T, golden[f"typeI_T_{tag}"]) <= 1e-4


def test_glm_typeI_outputs_and_pvalues(golden):
    y = golden["typeI_y"]
    exog = [golden["typeI_ex0"], golden["typeI_ex1"]]
    out = pyfunc.glm_typeI(y, exog, dmy_covariates=golden["typeI_cov"], output_tvalues=True, output_pvalues=True,
                           verbose=False)
    assert len(out) == 6
    F, Fv, T, Pm, Pv, Pt = out
    from scipy.stats import f as fdist
    np.testing.assert_allclose(Pv[1], fdist.sf(Fv[1], 1, y.shape[0] - 5), rtol=1e-6)
    T1 = pyfunc.glm_typeI(y[:, 3], exog, dmy_covariates=golden["typeI_cov"], output_fvalues=False,
                          output_tvalues=True, verbose=False)
    np.testing.assert_allclose(T1, T[:, 3], rtol=2e-5, atol=1e-5)


@pytest.mark.parametrize("widths", [(1,), (2, 1), (1, 3, 1)])
def test_partial_f_modes_vs_fp64(widths):
    rng = np.random.default_rng(sum(widths) * 7)
    n, V, G = 150, 3000, 20
    Y = (4.0 + rng.standard_normal((n, V))).astype(np.float32)
    k = 1 + sum(widths)
    X = np.column_stack([np.ones(n), rng.standard_normal((n, k - 1))])
    Y[:, :500] += (0.5 * X[:, 1])[:, None].astype(np.float32)
    groups, s0 = [], 1
    for w in widths:
        groups.append((s0, w))
        s0 += w
    perms = np.stack([rng.permutation(n) for _ in range(G)])
    db = DesignBatch(X[perms])
    Fg = glm_stat_tc(Y, db, "f", groups=groups).cpu().numpy()
    R = glm_stat_tc(Y, db, "rss").cpu().numpy()
    for g in range(0, G, 3):
        Xg = X[perms[g]]
        ref = oracle.partial_f_fp64(Xg, Y, groups)
        assert _scaled(Fg[g], ref) <= 2e-4, _scaled(Fg[g], ref)
        a = np.linalg.lstsq(Xg, Y.astype(np.float64), rcond=None)[0]
        rss = np.sum((Y - Xg @ a) ** 2, axis=0)
        np.testing.assert_allclose(R[g], rss, rtol=1e-4)


def test_engine_f_mode_vs_oracle(config1):
    st = config1
    n = st.n
    # design [1, group, age]: F of the group column and of age (widths 1) and of both (width 2)
    groups = [(1, 1), (2, 1), (1, 2)]
    eng = E.PermutationEngine(st.Y, st.pred_x, (st.offsets, st.indices), st.segments, 2.0, 1.0, batch=8,
                              f_groups=groups)
    perms = E.permutations(n, 5, 0, 12)
    got = eng.run(perms=perms)[:, :, 0, :]  # (P, groups, S)
    got_g = eng.run_graph(perms=perms)[:, :, 0, :]
    np.testing.assert_array_equal(got, got_g)
    X = st.design()
    ref = np.zeros_like(got)
    for p in range(perms.shape[0]):
        Fm = oracle.partial_f_fp64(X[perms[p]], st.Y, groups)
        for gi in range(len(groups)):
            img = Fm[gi].astype(np.float32)
            ref[p, gi, 0] = oracle.tfce_max_batch(st.offsets, st.indices, img, 2.0, 1.0)[0]
    rel = np.abs(got - ref) / np.abs(ref)
    print("F-mode maxima: median", np.median(rel), "max", rel.max())
    assert np.median(rel) <= 1e-4
    assert rel.max() <= 1e-3


def test_tm_models_glm_driver_volume(tmp_path, monkeypatch):
    """tm_models_randomise GLM branch drop-in on a small volume: the CSV lines
    against the oracle pipeline (FP64 glm_typeI + C sweep) on the same
    host-seeded permutations."""
    import argparse
    from tfce_mediation_gb300 import adjacency as A
    from tfce_mediation_gb300 import randomise
    rng = np.random.default_rng(33)
    mask = np.zeros((10, 9, 8), bool)
    mask[1:9, 1:8, 1:7] = True
    off, idx = A.voxel_csr(mask, 26, "pyfunc")
    V, n = int(mask.sum()), 40
    fac = rng.integers(0, 2, n).astype(np.float64)
    age = rng.standard_normal(n)
    cov = rng.standard_normal((n, 1))
    data = rng.standard_normal((n, V)).astype(np.float32)
    data[:, :60] += (0.7 * age)[:, None].astype(np.float32)
    d = tmp_path / "tmtemp_GLM_volume"
    d.mkdir()
    np.save(d / "exog_flat.npy", np.column_stack([fac, age]))
    np.save(d / "exog_shape.npy", np.array([1, 1]))
    np.save(d / "varnames.npy", np.array(["group", "age"]))
    np.save(d / "gstat.npy", np.array("both"))
    np.save(d / "data.npy", data)
    np.save(d / "optstfce.npy", np.array([2.0, 0.5]))
    np.save(d / "dmy_covariates.npy", cov)
    adj = np.empty(V, dtype=object)
    for v in range(V):
        adj[v] = np.asarray(idx[off[v]:off[v + 1]], np.int64)
    np.save(d / "adjac.npy", adj, allow_pickle=True)
    monkeypatch.chdir(tmp_path)
    opts = argparse.Namespace(range=[0, 5], surface=None, exchangeblock=None, seed=[11], batch=4)
    randomise.tm_models_glm_run(opts)
    out = tmp_path / "output_GLM_volume" / "perm_GLM"
    F_csv = {nm: np.loadtxt(out / f"perm_Fstat_{nm}_TFCE_maxVoxel.csv") for nm in ("group", "age")}
    T_csv = [np.loadtxt(out / f"perm_Tstat_con{c}_TFCE_maxVoxel.csv") for c in (1, 2)]
    for p in range(6):
        perm = np.random.RandomState(11 + p).permutation(n)
        Fm, Fv, T = oracle.glm_typeI(data, [fac, age], dmy_covariates=cov, rand_array=perm)
        for j, nm in enumerate(("group", "age")):
            img = Fv[j].astype(np.float32)
            ref = oracle.tfce_max_batch(off, idx, img, 2.0, 0.5)[0]
            assert abs(F_csv[nm][p] - ref) <= 1e-3 * abs(ref) + 1e-3, (nm, p, F_csv[nm][p], ref)
        for c in (1, 2):
            for si, s in enumerate((1.0, -1.0)):
                ref = oracle.tfce_max_batch(off, idx, T[c].astype(np.float32), 2.0, 0.5, sign=s)[0]
                got = T_csv[c - 1][2 * p + si]
                assert abs(got - ref) <= 1e-3 * abs(ref) + 1e-3, (c, p, s, got, ref)
