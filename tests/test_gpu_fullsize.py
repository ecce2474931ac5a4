"""The headline workload at its full size (2 x icosphere L7 = 327,684 vertices,
n = 350, k = 5): a few permutations against the oracle, the exact-mode
observed map bit for bit, and size-independent properties of the batched
path (batch splitting, graph replay, determinism, segment independence, the
two GLM precisions).

Bars as in test_gpu_engine: per-permutation max-TFCE relative error <= 1e-3,
median <= 1e-4 (t from the split-BF16 GLM); t |dt| <= 2e-4 max(1, |t|).
Property checks compare launches at 1e-6 relative: in per-component
accumulation the order of positions inside a threshold bucket follows warp
scheduling, which can move the double sums of the potentials by a last bit."""
import numpy as np
import pytest

from oracle import oracle
from tfce_mediation_gb300 import adjacency as A
from tfce_mediation_gb300 import engine as E
from tfce_mediation_gb300 import synth
from tfce_mediation_gb300.glm import WHAT_T, DesignBatch, glm_stat, glm_tstat_tc

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def study():
    return synth.config2()


@pytest.fixture(scope="module")
def engine(study):
    st = study
    return E.PermutationEngine(st.Y, st.pred_x, (st.offsets, st.indices), st.segments, 2.0, 1.0, batch=8,
                               floor_zero=True)


def _seg(st, h):
    v0, v1 = int(st.segments[h]), int(st.segments[h + 1])
    off = st.offsets[v0:v1 + 1] - st.offsets[v0]
    idx = st.indices[st.offsets[v0]:st.offsets[v1]] - v0
    return off, idx, v0, v1


def test_fullsize_maxima_vs_oracle(study, engine):
    st = study
    perms = E.permutations(st.n, 2026, 0, 2)
    got = engine.run(perms=perms)  # (P, C, 2, S)
    X = st.design()
    ref = np.zeros_like(got)
    for p in range(perms.shape[0]):
        t = oracle.tval_fp64(X[perms[p]], st.Y)
        for ci, c in enumerate(engine.contrasts):
            img = t[c].astype(np.float32)
            for si, s in enumerate((1.0, -1.0)):
                for h in range(2):
                    off, idx, v0, v1 = _seg(st, h)
                    ref[p, ci, si, h] = oracle.tfce_max_batch(off, idx, img[v0:v1], 2.0, 1.0, sign=s,
                                                              floor_zero=True)[0]
    rel = np.abs(got - ref) / np.abs(ref)
    print("config-2 maxima: median", np.median(rel), "max", rel.max())
    assert np.median(rel) <= 1e-4
    assert rel.max() <= 1e-3


def test_fullsize_observed_map_bitexact(study, engine):
    """Exact-mode sweep of the observed t map (the drop-in CreateAdjSet.run
    arithmetic) equals the oracle's correctly rounded sweep bit for bit."""
    st = study
    tmaps, tfce_maps, _ = engine.observed()
    for h in range(2):
        off, idx, v0, v1 = _seg(st, h)
        img = tmaps[0][v0:v1].astype(np.float32)
        e = oracle.tfce(off, idx, img, 2.0, 1.0, hh_exact=True)
        np.testing.assert_array_equal(tfce_maps[0, 0, v0:v1], e * (img.max() / np.float32(100)))


def test_fullsize_tensor_core_t(study):
    st = study
    perms = E.permutations(st.n, 7, 0, 24)
    db = DesignBatch(st.design()[perms])
    t_tc = glm_tstat_tc(st.Y, db, [1, 2, 3, 4]).cpu().numpy()
    t_32 = glm_stat(st.Y, db, WHAT_T, coef=[1, 2, 3, 4]).cpu().numpy()
    err = np.max(np.abs(t_tc - t_32) / np.maximum(1.0, np.abs(t_32)))
    print("config-2 tensor-core vs FP32 t:", err)
    assert err <= 2e-4


def test_fullsize_batching_graph_determinism(study, engine):
    st = study
    perms = E.permutations(st.n, 99, 0, 12)
    a = engine.run(perms=perms)                   # batches of 8 + 4
    b = np.concatenate([engine.run(perms=perms[:5]), engine.run(perms=perms[5:])])
    np.testing.assert_allclose(a, b, rtol=1e-6)
    c = engine.run_graph(perms=perms)
    np.testing.assert_allclose(a, c, rtol=1e-6)
    np.testing.assert_allclose(a, engine.run(perms=perms), rtol=1e-6)


def test_fullsize_segments_are_independent(study, engine):
    """Per-hemisphere maxima of the two-segment launch equal one-segment
    handles of each hemisphere on the same t maps."""
    import torch
    st = study
    perms = E.permutations(st.n, 5, 0, 4)
    tm = engine.tmaps(DesignBatch(engine.X[perms]))  # (P, C, V) on the device
    both = engine.sweep_max(tm, 4 * engine.C).cpu().numpy().reshape(4, engine.C, 2, 2)
    for h in range(2):
        off, idx, v0, v1 = _seg(st, h)
        adj = A.AdjacencySet((off, idx), 2.0, 1.0)
        adj.set_accumulation("component")
        sub = tm[:, :, v0:v1].contiguous()
        mx = torch.empty((4 * engine.C, 2, 1), device="cuda")
        adj.sweep_batch(sub.data_ptr(), v1 - v0, 4 * engine.C, 2, None, 1, mx.data_ptr(), None, 0,
                        torch.cuda.current_stream().cuda_stream)
        adj.status()
        np.testing.assert_allclose(both[..., h], mx.cpu().numpy().reshape(4, engine.C, 2), rtol=1e-6)
