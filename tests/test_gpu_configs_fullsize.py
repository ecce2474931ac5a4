"""Parity at the specified sizes of the synthetic configurations:

* the headline study (two icosphere-L7 hemispheres, 327,684 vertices,
  n = 350, k = 5): the 1-p(FWER) maps of every contrast and sign from a
  1,000-permutation GPU null against the FP64 oracle's null of the same
  permutations (tests/golden/config2_null.npz, made by make_config2_null.py),
  max |delta p| <= 0.005;
* the voxel study (91 x 109 x 91 grid, ~230k-voxel ellipsoid, 26-neighbour
  lists, n = 200, k = 4, H = 2, E = 0.5): per-permutation maxima;
* the mediation study (the headline mesh, n = 350, medtype 'M', Aroian z):
  per-permutation maxima.

Bars: null maxima relative error median <= 1e-4, max <= 1e-3 (split-BF16 GLM
against FP64 t; for the 8,000 maxima of the 1,000-permutation null the
99.9th percentile <= 5e-3 and the worst <= 5%: a t value within the GLM's
error of a threshold can merge two clusters one step earlier); the CSV's
'%.4f' rounding is applied to both nulls as the reference's files hold them
(calculate_fweP_vertex.py:37-69 reads them back).
"""
import os

import numpy as np
import pytest

from oracle import oracle
from tfce_mediation_gb300 import engine as E
from tfce_mediation_gb300 import fwer, synth

pytestmark = pytest.mark.gpu

NULL = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "config2_null.npz")


def _assert_maxima(got, ref, q999=1e-3, worst=1e-3):
    got, ref = np.asarray(got, np.float64), np.asarray(ref, np.float64)
    rel = np.abs(got - ref) / np.maximum(np.abs(ref), 1e-12)
    print("maxima: median", np.median(rel), "99.9%", np.quantile(rel, 0.999), "max", rel.max())
    assert np.median(rel) <= 1e-4, np.median(rel)
    assert np.quantile(rel, 0.999) <= q999, np.quantile(rel, 0.999)
    assert rel.max() <= worst, rel.max()


def _seg(st, h):
    v0, v1 = int(st.segments[h]), int(st.segments[h + 1])
    off = st.offsets[v0:v1 + 1] - st.offsets[v0]
    idx = st.indices[st.offsets[v0]:st.offsets[v1]] - v0
    return off, idx, v0, v1


@pytest.mark.parametrize("quadratic_form", [True, False])
def test_config2_fwer_maps_vs_fp64_oracle(quadratic_form):
    """The headline study, with the GLM in its quadratic form and with the
    residual epilogue (the two forms the autotuner chooses from)."""
    fx = np.load(NULL)
    null_ref = fx["null"]  # (N, 4 contrasts, 2 signs)
    N = null_ref.shape[0]
    assert N >= 1000
    st = synth.config2(seed=int(fx["study_seed"]))
    eng = E.PermutationEngine(st.Y, st.pred_x, (st.offsets, st.indices), st.segments, 2.0, 1.0, batch=256,
                              floor_zero=True)
    eng._tc.quadratic_form = quadratic_form
    assert eng._graph_qf() == quadratic_form
    perms = E.permutations(st.n, int(fx["seed"]), 0, N)
    got = eng.run_graph(perms=perms)  # (N, C, 2, S)
    null_gpu = np.vectorize(lambda v: float("%.4f" % v))(got.max(axis=-1))
    # 8,000 maxima: a t value within the GLM's ~3e-5 of a threshold can join
    # two large clusters one step earlier or later, which moves that map's
    # maximum by a few percent -- a handful of maxima, so the tail bound is
    # on the 99.9th percentile and the worst case is bounded loosely; the
    # 1-p maps below carry the bar that matters
    _assert_maxima(null_gpu, null_ref, q999=5e-3, worst=0.05)
    tv, maps, _ = eng.observed()
    X = st.design()
    t64 = oracle.tval_fp64(X, st.Y)
    worst = 0.0
    for ci, c in enumerate((1, 2, 3, 4)):
        # the CSV of a contrast holds + and - maxima of every permutation
        nr, ng = null_ref[:, ci, :].reshape(-1), null_gpu[:, ci, :].reshape(-1)
        for si, sgn in enumerate((1.0, -1.0)):
            for h in range(2):
                off, idx, v0, v1 = _seg(st, h)
                img = (t64[c, v0:v1] * sgn).astype(np.float32)
                ref_tfce = oracle.tfce(off, idx, img, 2.0, 1.0) * (img.max() / np.float32(100))
                p_ref = oracle.fwep_vertex(ref_tfce, nr)
                p_gpu = fwer.fwep(maps[ci, si, v0:v1], ng)
                d = np.abs(p_gpu - p_ref).max()
                worst = max(worst, d)
                assert d <= 0.005, (c, sgn, h, d)
    print("config-2 1-p(FWER): max |delta p| over 16 maps =", worst)


def test_config3_voxel_fullsize_vs_oracle():
    st = synth.config3()
    assert st.V > 220_000
    eng = E.PermutationEngine(st.Y, st.pred_x, (st.offsets, st.indices), None, 2.0, 0.5, batch=8)
    perms = E.permutations(st.n, 3, 0, 3)
    got = eng.run(perms=perms)[..., 0]  # (P, C, 2)
    X = st.design()
    ref = np.zeros_like(got)
    for p in range(perms.shape[0]):
        t = oracle.tval_fp64(X[perms[p]], st.Y)
        for ci, c in enumerate((1, 2, 3)):
            for si, s in enumerate((1.0, -1.0)):
                ref[p, ci, si] = oracle.tfce_max_batch(st.offsets, st.indices, t[c].astype(np.float32), 2.0, 0.5,
                                                       sign=s)[0]
    _assert_maxima(got, ref)


def test_config4a_mediation_fullsize_vs_oracle():
    st = synth.config4_mediation()
    x, dy = st.pred_x[:, 0], st.depend_y
    eng = E.MediationEngine(st.Y, x, dy, "M", (st.offsets, st.indices), st.segments, 2.0, 1.0, floor_zero=True,
                            batch=8)
    perms = E.permutations(st.n, 4, 0, 3)
    got = eng.run(perms=perms)[:, 0, 0, :]  # (P, S)
    ref = np.zeros_like(got)
    Y64 = st.Y.astype(np.float64)
    for p in range(perms.shape[0]):
        with np.errstate(all="ignore"):
            z = oracle.calc_sobelz("M", x[perms[p]], dy, Y64, st.n).astype(np.float32)
        for h in range(2):
            off, idx, v0, v1 = _seg(st, h)
            ref[p, h] = oracle.tfce_max_batch(off, idx, z[v0:v1], 2.0, 1.0, floor_zero=True)[0]
    _assert_maxima(got, ref)
