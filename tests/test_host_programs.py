"""Host logic of the programmed GLM outputs and the tm-models drivers (no GPU):
output rows and per-design weights, the cosinor design and output program,
and the exchange-block rules of the two randomise families."""
import argparse

import numpy as np
import pytest

from oracle import oracle
from tfce_mediation_gb300 import pyfunc, randomise
from tfce_mediation_gb300.glm import (OUT_ACRO, OUT_AMP, OUT_F, OUT_NEG_T, OUT_T, DesignBatch, output_columns,
                                      output_program)


def test_output_program_rows_and_offsets():
    rows, stride = output_program([("f", 1, 3), ("amp", 1), ("acro", 3), ("t", 4), ("-t", 4), ("f", 2, 1)])
    np.testing.assert_array_equal(rows, [[OUT_F, 1, 3, 0], [OUT_AMP, 1, 2, 9], [OUT_ACRO, 3, 2, 12],
                                         [OUT_T, 4, 1, 0], [OUT_NEG_T, 4, 1, 0], [OUT_F, 2, 1, 15]])
    assert stride == 16
    assert output_columns([("amp", 1), ("t", 5)]) == {1, 2, 5}
    with pytest.raises(ValueError):
        output_program([("z", 1)])
    with pytest.raises(ValueError):
        output_program([("f", 1, 0)])


def test_program_weights_match_inverse_blocks():
    rng = np.random.default_rng(3)
    n, G = 40, 5
    X = np.column_stack([np.ones(n), rng.standard_normal((n, 4))])
    perms = np.stack([rng.permutation(n) for _ in range(G)])
    db = DesignBatch(X[perms])
    outs = [("f", 1, 4), ("amp", 1), ("acro", 3), ("t", 2), ("amp", 4)]
    W = db.program_weights(outs)
    rows, stride = output_program(outs)
    assert W.shape == (G, stride) and W.dtype == np.float32
    for g in range(G):
        Xg = X[perms[g]]
        inv = np.linalg.inv(Xg.T @ Xg)
        np.testing.assert_allclose(W[g, :16], np.linalg.inv(inv[1:5, 1:5]).ravel(), rtol=1e-6)
        np.testing.assert_allclose(W[g, 16:19], [inv[1, 1], inv[1, 2], inv[2, 2]], rtol=1e-6)
        np.testing.assert_allclose(W[g, 19:22], [inv[3, 3], inv[3, 4], inv[4, 4]], rtol=1e-6)
        assert np.all(W[g, 22:25] == 0.0)  # ("amp", 4) lies outside the 5 columns: NaN on the device
    np.testing.assert_array_equal(db.group_blocks([(1, 4)]), W[:, :16])
    out = np.full((G, stride), 7.0, np.float32)
    db.program_weights(outs, out=out)
    np.testing.assert_array_equal(out[:, :22], W[:, :22])


def test_cosinor_design_and_outputs():
    rng = np.random.default_rng(4)
    n = 30
    tv = rng.uniform(0, 48, n)
    ex = [rng.standard_normal((n, 2)), rng.standard_normal(n)]
    cov = rng.standard_normal((n, 1))
    X = pyfunc.cosinor_design(tv, [24.0, 8.0], ex, cov)
    np.testing.assert_array_equal(X, oracle.cosinor_design(tv, [24.0, 8.0], ex, cov))
    assert X.shape == (n, 1 + 4 + 3 + 1)
    outs = randomise.cosinor_outputs(2, 3, 1)
    assert outs[0] == ("f", 1, 8)
    assert outs[1:5] == [("amp", 1), ("acro", 1), ("amp", 3), ("acro", 3)]
    assert outs[5:] == [("t", 5), ("-t", 5), ("t", 6), ("-t", 6), ("t", 7), ("-t", 7)]
    assert 0 not in output_columns(outs)  # the centred residual form applies


@pytest.mark.parametrize("sizes", [(4, 4, 4), (3, 5, 4)])
def test_exchange_block_rules(tmp_path, sizes):
    """Vertex/voxel loops shuffle the blocks' order always; the tm-models loops
    (rand_blocks + check_blocks) only when the blocks are equal in size; both
    permute within every block."""
    labels = np.concatenate([np.full(s, "b%d" % i) for i, s in enumerate(sizes)])
    f = tmp_path / "blocks.csv"
    np.savetxt(f, labels, fmt="%s")
    n = labels.shape[0]
    X = np.arange(n, dtype=np.float64)[:, None]
    opts = argparse.Namespace(exchangeblock=[str(f)], specifyvars=None)
    equal = len(set(sizes)) == 1
    for tm in (False, True):
        D = randomise._designs_for(X, n, 0, 6, opts, 9, equal_blocks_only=tm)[:, :, 0].astype(int)
        for p in range(6):
            rng = np.random.RandomState(9 + p)
            uniq = np.unique(labels)
            order = rng.permutation(list(uniq)) if (not tm or equal) else uniq
            idx = np.arange(n)
            want = np.concatenate([rng.permutation(idx[labels == b]) for b in order])
            np.testing.assert_array_equal(D[p], want)
            if tm and not equal:
                # block order kept: every position stays inside its own block
                np.testing.assert_array_equal(labels[D[p]], labels)


def test_saved_none(tmp_path):
    np.save(tmp_path / "a.npy", np.array(None, dtype=object), allow_pickle=True)
    np.save(tmp_path / "b.npy", np.zeros((3, 1)))
    assert randomise._saved_none(np.load(tmp_path / "a.npy", allow_pickle=True))
    assert not randomise._saved_none(np.load(tmp_path / "b.npy"))
    assert randomise._saved_none(None)


def _rm_pipeline_fp64(model, Y, ras, cums):
    """The RM-ANCOVA device pipeline restated in FP64 numpy: the effect sums of
    squares from the packed pseudoinverse rows (Wald form), SS between/within
    subjects from the grouped data rows, the F maps."""
    P = len(ras)
    ess = {}
    for si, (rows, W) in enumerate(model.slot_operands(ras, cums)):
        b = np.einsum("pin,nv->piv", rows, Y)
        prog, _ = output_program(model.slot_outputs[si])
        for q, (kind, j, w, o) in enumerate(prog):
            nm = [k for k, v in model.ess_at.items() if v == (si, q)][0]
            Wb = W[:, o:o + w * w].reshape(P, w, w)
            ess[nm] = np.einsum("piv,pij,pjv->pv", b[:, j:j + w], Wb, b[:, j:j + w])
    g = model.grouped_rows(cums)
    out = np.zeros((P, len(model.f_maps), Y.shape[1]))
    for p in range(P):
        yg = Y[g[p]]
        bs = np.zeros(Y.shape[1])
        ws = np.zeros(Y.shape[1])
        mu = Y.mean(0)
        for k in range(model.n_groups):
            blk = yg[model.goff[k]:model.goff[k + 1]]
            m = blk.mean(0)
            ws += ((blk - m) ** 2).sum(0)
            bs += len(blk) * (m - mu) ** 2
        eb = bs - sum(ess[x][p] for x in model.between)
        ew = ws - sum(ess[x][p] for x in model.within)
        for f, (nm, df, err) in enumerate(model.f_maps):
            out[p, f] = (ess[nm][p] / df) / ((ew / model.df_w) if err else (eb / model.df_b))
    return out


@pytest.mark.parametrize("kind", ["obs", "perm"])
def test_rm_anova_decomposition_fp64_wider(golden, kind):
    """Three-level factor, two covariates, four intervals: the Wald-form
    decomposition equals the FP64 restatement."""
    from tfce_mediation_gb300 import rm_anova as R
    d = golden["rm3_data"]
    s, n, V = d.shape
    model = R.RMModel(n, s, golden["rm3_f1"], golden["rm3_subj"], dmy_covariates=golden["rm3_cov"])
    assert all(sum(model.blocks[i][2] for i in sl) <= R.SLOT_ROWS for sl in model.slots)
    Y = d.reshape(s * n, V).astype(np.float64)
    if kind == "obs":
        ras, cums, kw = [None], np.arange(s * n)[None], {}
    else:
        ras, cums = [golden["rm3_ra"]], golden["rm3_shuffle"][None]
        kw = dict(rand_array=ras[0], shuffle=cums[0])
    got = _rm_pipeline_fp64(model, Y, ras, cums)[0]
    ref64 = oracle.rm_ancova_one(d.astype(np.float64), golden["rm3_f1"], golden["rm3_subj"],
                                 dmy_covariates=golden["rm3_cov"], **kw)
    np.testing.assert_allclose(got, np.asarray(ref64), rtol=1e-9, atol=1e-12)


@pytest.mark.parametrize("two", [False, True])
@pytest.mark.parametrize("tag", ["nocov", "cov"])
@pytest.mark.parametrize("kind", ["obs", "perm"])
def test_rm_anova_decomposition_fp64(golden, two, tag, kind):
    """Wald-form effect sums of squares + subject split reproduce the
    reference's RM-ANCOVA F maps (golden vectors) in FP64: the algebra the
    tensor-core GLM and rm_anova_combine run."""
    from tfce_mediation_gb300 import rm_anova as R
    pre = "rm2" if two else "rm1"
    d = golden[f"{pre}_data"]
    s, n, V = d.shape
    cov = golden[f"{pre}_cov"] if tag == "cov" else None
    if two:
        model = R.RMModel(n, s, golden["rm2_fa"], golden["rm2_subj"], dmy_factor2=golden["rm2_fb"],
                          dmy_covariates=cov)
    else:
        model = R.RMModel(n, s, golden["rm1_f1"], golden["rm1_subj"], dmy_covariates=cov)
    Y = d.reshape(s * n, V).astype(np.float64)
    if kind == "obs":
        ras, cums = [None], np.arange(s * n)[None]
    else:
        ras, cums = [golden[f"{pre}_ra_{tag}"]], golden[f"{pre}_shuffle_{tag}"][None]
    got = _rm_pipeline_fp64(model, Y, ras, cums)[0]
    # exact algebra: the oracle with every sum of squares in FP64
    kw = {} if kind == "obs" else dict(rand_array=ras[0], shuffle=cums[0])
    if two:
        ref64 = oracle.rm_ancova_two(d.astype(np.float64), golden["rm2_fa"], golden["rm2_fb"], golden["rm2_subj"],
                                     dmy_covariates=cov, **kw)
    else:
        ref64 = oracle.rm_ancova_one(d.astype(np.float64), golden["rm1_f1"], golden["rm1_subj"], dmy_covariates=cov,
                                     **kw)
    np.testing.assert_allclose(got, np.asarray(ref64), rtol=1e-9, atol=1e-12)
    # the reference itself forms SS_Total as a float32 sum, which enters the
    # differences of sums of squares: ~1e-5 of max(1, F)
    ref = golden[f"{pre}_{kind}_{tag}"]
    assert np.max(np.abs(got - ref) / np.maximum(1.0, np.abs(ref))) <= 5e-5


def test_rm_model_packing():
    from tfce_mediation_gb300 import rm_anova as R
    rng = np.random.default_rng(1)
    n, s = 30, 3
    fa = R.dummy_code(rng.integers(0, 2, n))
    fb = R.dummy_code(rng.integers(0, 3, n))
    subj = R.dummy_code(np.arange(n), demean=False)
    m = R.RMModel(n, s, fa, subj, dmy_factor2=fb, dmy_covariates=rng.standard_normal((n, 1)))
    assert all(sum(m.blocks[i][2] for i in sl) <= R.SLOT_ROWS for sl in m.slots)
    assert sorted(i for sl in m.slots for i in sl) == list(range(len(m.blocks)))
    assert set(m.ess_at) == {"cells", "ab", "a", "b", "s", "scov", "sab", "sa", "sb"}
    assert m.df_b == n - 1 - 1 - 2 - 2 - 1 and m.df_w == m.df_b * 2
    np.testing.assert_array_equal(m.goff, np.arange(n + 1) * s)
    with pytest.raises(ValueError):
        R.RMModel(n, s, fa, rng.standard_normal((n, 2)))  # not a subject coding
    empty = R.dummy_code(np.r_[np.zeros(n // 2), np.ones(n - n // 2)])
    with pytest.raises(ValueError, match="rank deficient"):
        R.RMModel(n, s, empty, subj, dmy_factor2=empty.copy())  # f1 x f2 cells (0,1), (1,0) empty


def test_rm_permutations_replay_the_reference_loop():
    """rand_array then an in-place shuffle of the one data array per
    iteration (tm_models_randomise.py:522-530 with pyfunc.py:2139): the
    cumulative row orders equal what successive shuffles leave in the array."""
    n, s = 6, 3
    N = n * s
    data = np.arange(N * 2, dtype=np.float64).reshape(N, 2)
    ras, cums = randomise.rm_permutations(n, N, 3, 8, 40)
    arr = data.copy()
    for i, it in enumerate(range(3, 8)):
        rng = np.random.RandomState(40 + it)
        ra = rng.permutation(list(range(n)))
        rng.shuffle(arr)
        np.testing.assert_array_equal(ras[i], ra)
        np.testing.assert_array_equal(arr, data[cums[i]])


def test_gd_gather_list_keeps_the_scatter_order(golden):
    """The per-vertex gather list, accumulated in float32 in list order with
    the oracle's weights, equals the reference's scatter bit for bit."""
    from tfce_mediation_gb300.gd_fwhm import gather_list
    pairs, dist = golden["gd_pairs"], golden["gd_dist"]
    data = golden["gd_data0"]
    sg = float(golden["gd_sigma0"])
    V = data.shape[0]
    off, src, pidx = gather_list(pairs, V)
    assert off[-1] == 2 * len(pairs)
    w = np.array([oracle.gd_weight(d, sg) for d in dist], np.float32)
    w0 = oracle.gd_weight(0.0, sg)
    out = np.zeros(V, np.float32)
    for v in range(V):
        s = sw = np.float32(0.0)
        for k in range(off[v], off[v + 1]):
            s = np.float32(s + np.float32(w[pidx[k]] * data[src[k]]))
            sw = np.float32(sw + w[pidx[k]])
        out[v] = np.float32(s + np.float32(w0 * data[v])) / np.float32(sw + w0)
    np.testing.assert_array_equal(out, golden["gd_out0"])
    with pytest.raises(ValueError):
        gather_list([[0, V]], V)


def test_tm_models_randomise_cli_dispatch(monkeypatch):
    """The tm_models_randomise flags select the same branch as the reference."""
    calls = []
    for name in ("tm_models_glm_run", "tm_models_mediation_run", "tm_models_rmancova_run", "tm_models_cosinor_run",
                 "tm_models_cosinor_mediation_run"):
        monkeypatch.setattr(randomise, name, lambda opts, _n=name: calls.append((_n, opts.surface)))
    p = randomise.tm_models_randomise_parser()
    cases = [(["-r", "0", "9", "-s", "area", "-glm"], "tm_models_glm_run", ["area"]),
             (["-r", "0", "9", "-v", "-med"], "tm_models_mediation_run", None),
             (["-r", "0", "9", "-v", "-ofa"], "tm_models_rmancova_run", None),
             (["-r", "0", "9", "-s", "thickness", "-tfa"], "tm_models_rmancova_run", ["thickness"]),
             (["-r", "0", "9", "-v", "-cos"], "tm_models_cosinor_run", None),
             (["-r", "0", "9", "-v", "-mcos"], "tm_models_cosinor_mediation_run", None)]
    for argv, want, surf in cases:
        calls.clear()
        randomise.tm_models_randomise_run(p.parse_args(argv))
        assert calls == [(want, surf)], argv
    with pytest.raises(ValueError):
        randomise.tm_models_randomise_run(p.parse_args(["-r", "0", "9", "-t", "-glm"]))
    with pytest.raises(SystemExit):
        p.parse_args(["-r", "0", "9", "-v", "-glm", "-cos"])  # one statistic at a time


def test_tm_models_surface_space(tmp_path):
    """Surface tm-models inputs: both masked hemispheres as two segments of one
    CSR (the masked subgraphs), density weights of the masked vertices, the
    zero-fill floor and the vertex CSV format; a volume: one voxel CSR."""
    from tfce_mediation_gb300 import adjacency as A
    from tfce_mediation_gb300 import synth
    v, f = synth.icosphere(2)
    off, idx = A.mesh_csr(f, v.shape[0])
    adj = np.empty(v.shape[0], dtype=object)
    for i in range(v.shape[0]):
        adj[i] = np.asarray(idx[off[i]:off[i + 1]], np.int64)
    rng = np.random.default_rng(2)
    m_lh = rng.random(v.shape[0]) > 0.2
    m_rh = rng.random(v.shape[0]) > 0.3
    vd_rh = rng.random(v.shape[0]).astype(np.float32)
    d = tmp_path / "tmtemp_GLM_area"
    d.mkdir()
    np.save(d / "mask_lh.npy", m_lh)
    np.save(d / "mask_rh.npy", m_rh)
    np.save(d / "adjac_lh.npy", adj, allow_pickle=True)
    np.save(d / "adjac_rh.npy", adj, allow_pickle=True)
    np.save(d / "vdensity_lh.npy", np.array(1))
    np.save(d / "vdensity_rh.npy", vd_rh)
    o, i, kw, fmt, suffix = randomise._tm_models_space(str(d), "area")
    o1, i1 = A.induced_csr(adj, m_lh)
    o2, i2 = A.induced_csr(adj, m_rh)
    oc, ic, seg = A.concat_csr([(o1, i1), (o2, i2)])
    np.testing.assert_array_equal(o, oc)
    np.testing.assert_array_equal(i, ic)
    np.testing.assert_array_equal(kw["segments"], [0, m_lh.sum(), m_lh.sum() + m_rh.sum()])
    np.testing.assert_array_equal(kw["vdensity"], np.concatenate([np.ones(m_lh.sum(), np.float32), vd_rh[m_rh]]))
    assert kw["floor_zero"] and (fmt, suffix) == ("%.4f", "maxVertex")
    dv = tmp_path / "tmtemp_GLM_volume"
    dv.mkdir()
    np.save(dv / "adjac.npy", adj, allow_pickle=True)
    o, i, kw, fmt, suffix = randomise._tm_models_space(str(dv), None)
    np.testing.assert_array_equal(o, off)
    assert kw == {"segments": None} and (fmt, suffix) == ("%1.4f", "maxVoxel")


@pytest.mark.parametrize("s,la,lb,c", [(2, 2, 0, 0), (2, 3, 0, 1), (3, 2, 2, 1), (2, 2, 3, 0), (5, 2, 0, 2)])
def test_rm_anova_decomposition_shapes(s, la, lb, c):
    """Random studies over interval counts, factor levels and covariates: the
    Wald-form decomposition equals the FP64 restatement (permuted call)."""
    from tfce_mediation_gb300 import rm_anova as R
    rng = np.random.default_rng(s * 100 + la * 10 + lb + c)
    n, V = 36, 7
    ga = rng.permutation(np.arange(n) % la)
    gb = rng.permutation(np.arange(n) % lb) if lb else None
    fa = R.dummy_code(ga)
    fb = None if gb is None else R.dummy_code(gb)
    cov = rng.standard_normal((n, c)) if c else None
    subj = R.dummy_code(np.arange(n), demean=False)
    d = rng.standard_normal((s, n, V)) + rng.standard_normal(n)[None, :, None]
    model = R.RMModel(n, s, fa, subj, dmy_factor2=fb, dmy_covariates=cov)
    ra, sh = rng.permutation(n), rng.permutation(n * s)
    got = _rm_pipeline_fp64(model, d.reshape(s * n, V), [ra], sh[None])[0]
    if fb is None:
        ref = oracle.rm_ancova_one(d, fa, subj, dmy_covariates=cov, rand_array=ra, shuffle=sh)
    else:
        ref = oracle.rm_ancova_two(d, fa, fb, subj, dmy_covariates=cov, rand_array=ra, shuffle=sh)
    np.testing.assert_allclose(got, np.asarray(ref), rtol=1e-8, atol=1e-12)


@pytest.mark.parametrize("sizes", [(5, 5, 5), (4, 6, 5)])
def test_rm_permutations_exchange_blocks(sizes):
    """rand_blocks semantics inside the RM-ANCOVA loop: blocks shuffled only
    when of equal size, rows permuted within every block, then the long-row
    shuffle drawn from the same stream."""
    labels = np.concatenate([np.full(z, "b%d" % i) for i, z in enumerate(sizes)])
    n = labels.shape[0]
    s = 2
    ras, cums = randomise.rm_permutations(n, n * s, 0, 4, 3, block_list=labels)
    equal = len(set(sizes)) == 1
    c = np.arange(n * s)
    for i in range(4):
        rng = np.random.RandomState(3 + i)
        uniq = np.unique(labels)
        order = rng.permutation(list(uniq)) if equal else uniq
        idx = np.arange(n)
        want = np.concatenate([rng.permutation(idx[labels == b]) for b in order])
        c = c[rng.permutation(n * s)]
        np.testing.assert_array_equal(ras[i], want)
        np.testing.assert_array_equal(cums[i], c)


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_cosinor_closed_forms_random(seed):
    """The epilogue's trigonometry-free amplitude / acrophase t equal the
    reference's arctan / sin / cos error propagation on random fits (both
    coefficient signs, two periods)."""
    rng = np.random.default_rng(seed)
    n, V = 50, 40
    tv = rng.uniform(0, 48, n)
    y = rng.standard_normal((n, V)) + rng.choice([-1.0, 1.0], V) * np.cos(2 * np.pi * (tv[:, None] - 7) / 24)
    perm = rng.permutation(n)
    X = oracle.cosinor_design(tv, [24.0, 12.0])[perm]
    inv = np.linalg.inv(X.T @ X)
    b = inv @ X.T @ y
    sigma = np.sqrt(np.sum((y - X @ b) ** 2, 0) / (n - X.shape[1]))
    res = oracle.glm_cosinor(y.astype(np.float32), tv, rand_array=perm, period=[24.0, 12.0], calc_MESOR=False)
    for i in range(2):
        c_, s_ = 1 + 2 * i, 2 + 2 * i
        a2 = b[c_] ** 2 + b[s_] ** 2
        cr = 2 * inv[c_, s_] * np.abs(b[c_] * b[s_])
        t_amp = a2 / (sigma * np.sqrt(inv[c_, c_] * b[c_] ** 2 - cr + inv[s_, s_] * b[s_] ** 2))
        t_acro = a2 / (sigma * np.sqrt(inv[c_, c_] * b[s_] ** 2 + cr + inv[s_, s_] * b[c_] ** 2))
        np.testing.assert_allclose(t_amp, res[9][i], rtol=1e-6)
        np.testing.assert_allclose(t_acro, res[10][i], rtol=1e-6)


def test_design_batch_operators():
    """DesignBatch's host operators: inv(X'X) zero padded for designs of fewer
    columns, pinv = inv(X'X) X' (formed on first use for same-k batches),
    diag and dof, and the quadratic form's inv(Xc'Xc) = inv(X'X)[1:, 1:]."""
    import numpy as np
    from tfce_mediation_gb300.glm import DesignBatch
    rng = np.random.default_rng(4)
    n = 40
    X = np.column_stack([np.ones(n), rng.standard_normal((n, 3))])
    same = DesignBatch(np.stack([X[rng.permutation(n)] for _ in range(5)]))
    assert same._pinv64 is None  # not formed until asked for
    for g in range(5):
        Xg = same.X64[g]
        inv = np.linalg.inv(Xg.T @ Xg)
        np.testing.assert_allclose(same.inverse()[g], inv, rtol=1e-12, atol=1e-14)
        np.testing.assert_allclose(same.pinv64[g], inv @ Xg.T, rtol=1e-10, atol=1e-13)
        np.testing.assert_allclose(same.invdiag64[g], np.diag(inv), rtol=1e-12)
        Xc = Xg[:, 1:] - Xg[:, 1:].mean(axis=0)
        np.testing.assert_allclose(same.inverse()[g][1:, 1:], np.linalg.inv(Xc.T @ Xc), rtol=1e-10, atol=1e-14)
    assert same.dof.tolist() == [n - 4] * 5
    mixed = DesignBatch([X[:, :2], X, X[:, :3]], kmax=4)
    assert mixed.kmax == 4 and mixed.dof.tolist() == [n - 2, n - 4, n - 3]
    assert np.all(mixed.inverse()[0, 2:, :] == 0) and np.all(mixed.inverse()[0, :, 2:] == 0)
    assert np.all(mixed.X64[2, :, 3] == 0) and np.all(mixed.pinv64[0, 2:] == 0)
    np.testing.assert_allclose(mixed.inverse()[2, :3, :3], np.linalg.inv(X[:, :3].T @ X[:, :3]), rtol=1e-12)
