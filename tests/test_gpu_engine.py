"""End-to-end permutation inference on config 1 (icosphere L5, n=100, k=3)
against the oracle pipeline on the same host-seeded permutation streams.

The GPU computes t in FP32 arithmetic (precision 'fp32', ~1e-6 relative to
FP64) or as a split-BF16 tensor-core GEMM with FP32 accumulation ('bf16x3',
~3e-5), the oracle in float64, so the sweeps see maps that differ slightly; a
vertex that sits on a threshold can then change one increment.  Stated
tolerances:
  * per-permutation max-TFCE: relative error <= 1e-3 for every value, median
    <= 1e-5 ('fp32') / 1e-4 ('bf16x3');
  * 1-p(FWER) maps: max |delta p| <= 0.005 (the target of the path).
"""
import numpy as np
import pytest

from oracle import oracle
from tfce_mediation_gb300 import engine as E
from tfce_mediation_gb300 import fwer

pytestmark = pytest.mark.gpu

SEED = 7


def oracle_maxima(st, perms, contrasts=(1, 2)):
    X = st.design()
    out = np.zeros((perms.shape[0], len(contrasts), 2), np.float32)
    for p in range(perms.shape[0]):
        t = oracle.tval_fp64(X[perms[p]], st.Y)
        for ci, c in enumerate(contrasts):
            img = t[c].astype(np.float32)
            for si, s in enumerate((1.0, -1.0)):
                out[p, ci, si] = oracle.tfce_max_batch(st.offsets, st.indices, img, 2.0, 1.0, sign=s)[0]
    return out


MEDIAN_BAR = {"fp32": 1e-5, "bf16x3": 1e-4}


@pytest.fixture(scope="module")
def ref100(config1):
    perms = E.permutations(config1.n, SEED, 0, 100)
    return perms, oracle_maxima(config1, perms)


@pytest.fixture(scope="module", params=["bf16x3", "bf16x3-residual", "fp32"])
def run100(config1, ref100, request):
    """bf16x3: the tensor-core GLM in its quadratic form (the engines'
    default here); bf16x3-residual: with the residual epilogue."""
    st = config1
    eng = E.PermutationEngine(st.Y, st.pred_x, (st.offsets, st.indices), st.segments, 2.0, 1.0, batch=32,
                              precision=request.param.split("-")[0])
    if request.param.endswith("residual"):
        eng._tc.quadratic_form = False
    assert eng._graph_qf() == (request.param == "bf16x3")
    perms, ref = ref100
    gpu = E.reduce_vertex(eng.run(perms=perms))
    return st, eng, perms, gpu, ref


def test_null_maxima_match_oracle(run100):
    st, eng, perms, gpu, ref = run100
    rel = np.abs(gpu - ref) / np.abs(ref)
    print(eng.precision, "median", np.median(rel), "max", rel.max())
    assert np.median(rel) <= MEDIAN_BAR[eng.precision], np.median(rel)
    assert rel.max() <= 1e-3, rel.max()


def test_batching_is_invisible(run100):
    st, eng, perms, gpu, ref = run100
    again = E.reduce_vertex(eng.run(perms=perms[:37]))
    np.testing.assert_array_equal(again, gpu[:37])


def test_fwer_map_matches_oracle(run100):
    st, eng, perms, gpu, ref = run100
    tmaps, tfce_maps, mx = eng.observed()
    X = st.design()
    t_ref = oracle.tval_fp64(X, st.Y)
    for ci in range(2):
        null_g = E.null_distribution(gpu, ci)
        null_o = E.null_distribution(ref, ci)
        img = t_ref[ci + 1].astype(np.float32)
        e = oracle.tfce(st.offsets, st.indices, img, 2.0, 1.0)
        obs_o = e * (img.max() / np.float32(100))
        p_g = fwer.fwep(tfce_maps[ci, 0], null_g)
        p_o = oracle.fwep_vertex(obs_o, null_o)
        assert np.abs(p_g - p_o).max() <= 0.005
    # the planted effect (regressor 1) is found
    assert fwer.fwep(tfce_maps[0, 0], E.null_distribution(gpu, 0)).max() >= 0.95


def test_observed_maps_match_oracle(run100):
    st, eng, perms, gpu, ref = run100
    tmaps, tfce_maps, mx = eng.observed()
    t_ref = oracle.tval_fp64(st.design(), st.Y)
    err = np.abs(tmaps - t_ref[1:3]) / np.maximum(1.0, np.abs(t_ref[1:3]))
    assert err.max() <= 1e-4
    # feeding the GPU's own t maps to the oracle sweep reproduces the GPU TFCE bit for bit
    for ci in range(2):
        for si, s in enumerate((1.0, -1.0)):
            img = (s * tmaps[ci]).astype(np.float32)
            e = oracle.tfce(st.offsets, st.indices, img, 2.0, 1.0, hh_exact=True)
            np.testing.assert_array_equal(tfce_maps[ci, si], e * (img.max() / np.float32(100)))


@pytest.mark.parametrize("precision", ["bf16x3", "fp32"])
def test_graph_runner_matches_uncaptured(config1, precision):
    st = config1
    eng = E.PermutationEngine(st.Y, st.pred_x, (st.offsets, st.indices), st.segments, 2.0, 1.0, batch=16,
                              precision=precision)
    perms = E.permutations(st.n, 13, 0, 16 * 5 + 7)  # 5 full captured batches + a partial one
    a = eng.run(perms=perms)
    b = eng.run_graph(perms=perms)
    np.testing.assert_array_equal(a, b)
    c = eng.run_graph(perms=perms)  # replays again
    np.testing.assert_array_equal(a, c)


def test_run_stream_with_new_data_per_step(config1):
    """run_stream: new host data at chosen steps takes effect exactly from
    that step (stream order), short batches are padded inside the graph."""
    import torch
    st = config1
    Y2 = (st.Y[::-1].copy() + 0.1).astype(np.float32)
    kw = dict(segments=st.segments, H=2.0, E=1.0, batch=8)
    eng = E.PermutationEngine(st.Y, st.pred_x, (st.offsets, st.indices), **kw)
    e1 = E.PermutationEngine(st.Y, st.pred_x, (st.offsets, st.indices), **kw)
    e2 = E.PermutationEngine(Y2, st.pred_x, (st.offsets, st.indices), **kw)
    perms = E.permutations(st.n, 31, 0, 29)
    P1 = torch.from_numpy(st.Y).pin_memory()
    P2 = torch.from_numpy(Y2).pin_memory()
    steps = [(None, perms[0:8]), (P2, perms[8:16]), (None, perms[16:24]), (P1, perms[24:29])]
    got = eng.run_stream(steps)
    assert [g.shape[0] for g in got] == [8, 8, 8, 5]
    np.testing.assert_allclose(got[0], e1.run(perms=perms[0:8]), rtol=1e-6)
    np.testing.assert_allclose(got[1], e2.run(perms=perms[8:16]), rtol=1e-6)
    np.testing.assert_allclose(got[2], e2.run(perms=perms[16:24]), rtol=1e-6)
    np.testing.assert_allclose(got[3], e1.run(perms=perms[24:29]), rtol=1e-6)


def test_sweep_shapes_agree(config1):
    """The two CTA shapes of the per-component sweep (3 x 512 threads per SM,
    40 registers; 2 x 512, 64 registers) give the same maxima."""
    import torch
    st = config1
    eng = E.PermutationEngine(st.Y, st.pred_x, (st.offsets, st.indices), st.segments, 2.0, 1.0, batch=32,
                              floor_zero=True)
    perms = E.permutations(st.n, 3, 0, 32)
    res = []
    for shape in (3, 2):
        eng.adj.set_sweep_shape(shape)
        res.append(eng.run(perms=perms))
    np.testing.assert_allclose(res[0], res[1], rtol=1e-6)
    with pytest.raises(Exception):
        eng.adj.set_sweep_shape(4)
