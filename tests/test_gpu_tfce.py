"""TFCE sweep on the GPU against the reference (golden vectors) and the oracle.

Bars:
  * component labels (as partitions) and extents at every threshold:
    bit-exact against the oracle's restatement of the reference sweep;
  * TFCE values: bit-exact against the oracle evaluated with the correctly
    rounded threshold weight HH = T^H (hh_exact=True: T*T for H = 2, the
    double power rounded once otherwise), which is the kernel's arithmetic;
  * TFCE values against the reference's own outputs: relative error <= 1e-6.
    The reference takes HH from the host libm's powf, which is not always
    correctly rounded (glibc: up to 0.82 ulp), so at a few thresholds its HH
    is one float ulp away and the sums can differ in their last bits.
"""
import numpy as np
import pytest

from oracle import oracle
from tfce_mediation_gb300 import adjacency as A
from tfce_mediation_gb300.tfce import CreateAdjSet

pytestmark = pytest.mark.gpu


def _partition_equal(a, b):
    """Labels equal up to renaming (and the same inactive set)."""
    if not np.array_equal(a < 0, b < 0):
        return False
    m = a >= 0
    pairs = np.unique(np.stack([a[m], b[m]]), axis=1)
    return pairs.shape[1] == np.unique(a[m]).size == np.unique(b[m]).size


REF_RTOL = 1e-6


def test_run_vs_reference_and_oracle(golden):
    off, idx, maps = golden["sweep_off"], golden["sweep_idx"], golden["sweep_maps"]
    adj = A.from_csr(off, idx)
    for pi, (H, E) in enumerate(golden["sweep_params"]):
        op = CreateAdjSet(H, E, adj)
        for mi in range(maps.shape[0]):
            e = np.zeros(maps.shape[1], np.float32)
            op.run(maps[mi].copy(), e)
            ref = golden["sweep_enhn"][pi, mi]
            rel = np.abs(e - ref) / np.maximum(np.abs(ref), 1e-30)
            assert rel.max() <= REF_RTOL, (H, E, mi, rel.max())
            exact = oracle.tfce(off, idx, maps[mi], float(H), float(E), hh_exact=True)
            if float(E) in (1.0, 0.5, 2.0):
                np.testing.assert_array_equal(e, exact, err_msg=f"H={H} E={E} map {mi}")
            else:  # pow(size, E) in double: CUDA and the host libm may differ by 1 ulp
                np.testing.assert_allclose(e, exact, rtol=2.5e-7, err_msg=f"H={H} E={E} map {mi}")


def test_run_accumulates(golden):
    op = CreateAdjSet(2.0, 1.0, (golden["sweep_off"], golden["sweep_idx"]))
    e = golden["sweep_accum_in"].copy()
    op.run(golden["sweep_maps"][2].copy(), e)
    np.testing.assert_array_equal(e, golden["sweep_accum_out"])


def test_run_argument_checks(golden):
    op = CreateAdjSet(2.0, 1.0, (golden["sweep_off"], golden["sweep_idx"]))
    V = op.n_vertices
    with pytest.raises(ValueError):
        op.run(np.zeros(V, np.float64), np.zeros(V, np.float32))
    with pytest.raises(ValueError):
        op.run(np.zeros((2, V), np.float32), np.zeros(V, np.float32))
    with pytest.raises(ValueError):
        op.run(np.zeros(2 * V, np.float32)[::2], np.zeros(V, np.float32))
    with pytest.raises(ValueError):
        op.run(np.zeros(V - 1, np.float32), np.zeros(V - 1, np.float32))
    with pytest.raises(TypeError):
        op.run([0.0] * V, np.zeros(V, np.float32))


def _config1_maps(st, n_perm=6, seed=11):
    X = st.design()
    maps = []
    for p in range(n_perm):
        perm = np.random.RandomState(seed + p).permutation(st.n)
        t = oracle.tval_fp64(X[perm], st.Y)
        maps.append(t[1].astype(np.float32))
        maps.append(t[2].astype(np.float32))
    return np.stack(maps)


def test_labels_and_extents_bitexact(config1):
    st = config1
    op = CreateAdjSet(2.0, 1.0, (st.offsets, st.indices))
    t = oracle.tval_fp64(st.design(), st.Y)
    maps = [t[1].astype(np.float32), (-t[1]).astype(np.float32), t[2].astype(np.float32)]
    maps += list(_config1_maps(st, n_perm=3, seed=11))
    for img in maps:
        e_o, lab_o, ext_o = oracle.tfce_labels(st.offsets, st.indices, img, 2.0, 1.0, hh_exact=True)
        e_g, lab_g, ext_g = op.adjacency.run_labels(img)
        assert lab_g.shape == lab_o.shape
        for s in range(lab_o.shape[0]):
            assert _partition_equal(lab_o[s], lab_g[s]), f"step {s}"
            np.testing.assert_array_equal(ext_o[s], ext_g[s])
        np.testing.assert_array_equal(e_g, e_o)


def test_batch_maxima_bitexact(config1):
    import torch
    st = config1
    maps = _config1_maps(st)
    adj = A.AdjacencySet((st.offsets, st.indices), 2.0, 1.0)
    d = torch.from_numpy(maps).cuda()
    out = torch.empty((maps.shape[0], 2, 1), device="cuda")
    adj.sweep_batch(d.data_ptr(), st.V, maps.shape[0], 2, None, 0, out.data_ptr())
    adj.status()
    got = out.cpu().numpy()
    for sgn, s in enumerate((1.0, -1.0)):
        ref = oracle.tfce_max_batch(st.offsets, st.indices, maps, 2.0, 1.0, sign=s, hh_exact=True)
        np.testing.assert_array_equal(got[:, sgn, 0], ref)
        ref_powf = oracle.tfce_max_batch(st.offsets, st.indices, maps, 2.0, 1.0, sign=s)
        np.testing.assert_allclose(got[:, sgn, 0], ref_powf, rtol=REF_RTOL)


def test_batch_scaled_maps_and_vdensity(config1):
    import torch
    st = config1
    maps = _config1_maps(st, n_perm=2)
    vd = A.vertex_density((st.offsets, st.indices))
    adj = A.AdjacencySet((st.offsets, st.indices), 2.0, 1.0)
    d = torch.from_numpy(maps).cuda()
    vdd = torch.from_numpy(vd).cuda()
    mx = torch.empty((maps.shape[0], 2, 1), device="cuda")
    om = torch.empty((maps.shape[0], 2, st.V), device="cuda")
    adj.sweep_batch(d.data_ptr(), st.V, maps.shape[0], 2, vdd.data_ptr(), 0, mx.data_ptr(),
                    om.data_ptr(), 1)
    adj.status()
    for m in range(maps.shape[0]):
        for sgn, s in enumerate((1.0, -1.0)):
            img = (s * maps[m]).astype(np.float32)
            e = oracle.tfce(st.offsets, st.indices, img, 2.0, 1.0, hh_exact=True)
            ref = (e * (img.max() / np.float32(100))) * vd
            np.testing.assert_array_equal(om[m, sgn].cpu().numpy(), ref)
            assert mx[m, sgn, 0].item() == ref.max()


def test_two_segments_and_floor_zero(golden):
    """lh/rh as two segments of one launch (masked rh scattered into zeros)."""
    import torch
    off, idx = golden["sweep_off"], golden["sweep_idx"]
    maps = golden["sweep_maps"]
    Vh = off.shape[0] - 1
    O, I, seg = A.concat_csr([(off, idx), (off, idx)])
    adj = A.AdjacencySet((O, I), [2.0, 2.0], [1.0, 0.5], seg)
    stat = np.concatenate([maps[0], maps[1]])[None].astype(np.float32)
    stat[0, Vh: Vh + 50] = 0.0
    out = torch.empty((1, 2, 2), device="cuda")
    adj.sweep_batch(torch.from_numpy(stat).cuda().data_ptr(), 2 * Vh, 1, 2, None, 1, out.data_ptr())
    adj.status()
    got = out.cpu().numpy()[0]
    for sgn, s in enumerate((1.0, -1.0)):
        for h, E in ((0, 1.0), (1, 0.5)):
            img = s * stat[0, h * Vh:(h + 1) * Vh]
            ref = oracle.tfce_max_batch(off, idx, img, 2.0, E, floor_zero=True, hh_exact=True)[0]
            assert got[sgn, h] == ref


def test_asymmetric_lists_follow_insertion_rule():
    """mmr voxel lists (self entries, voxel 0's one-way list) against the oracle."""
    mask = np.zeros((9, 8, 7), bool)
    mask[1:8, 1:7, 1:6] = True
    mask[0, 0, 0] = True
    off, idx = A.voxel_csr(mask, 26, "mmr")
    adj = A.AdjacencySet((off, idx), 2.0, 1.0)
    assert not adj.symmetric
    rng = np.random.default_rng(3)
    for _ in range(5):
        img = rng.standard_normal(off.shape[0] - 1).astype(np.float32) + 0.5
        e_g = np.zeros_like(img)
        adj.run(img, e_g)
        e_o = oracle.tfce(off, idx, img, 2.0, 1.0, hh_exact=True)
        np.testing.assert_array_equal(e_g, e_o)


def test_degenerate_maps(golden):
    off, idx = golden["sweep_off"], golden["sweep_idx"]
    op = CreateAdjSet(2.0, 1.0, (off, idx))
    V = op.n_vertices
    for img in (np.zeros(V, np.float32), -np.ones(V, np.float32),
                np.full(V, np.nan, np.float32)):
        e = np.ones(V, np.float32)
        op.run(img, e)
        np.testing.assert_array_equal(e, np.ones(V, np.float32))
    img = golden["sweep_maps"][0].copy()
    img[::7] = np.nan
    e = np.zeros(V, np.float32)
    op.run(img, e)
    np.testing.assert_array_equal(e, oracle.tfce(off, idx, img, 2.0, 1.0, hh_exact=True))
    single = CreateAdjSet(2.0, 1.0, [[]])
    e = np.zeros(1, np.float32)
    single.run(np.array([3.0], np.float32), e)
    np.testing.assert_array_equal(e, oracle.tfce(np.array([0, 0]), np.zeros(0, np.int32),
                                                 np.array([3.0], np.float32), 2.0, 1.0, hh_exact=True))


COMPONENT_RTOL = 1e-5
# Per-component sums resolve a vertex as a difference of component potentials
# (doubles of the order of the map's largest value); vertices that enter only
# at the last thresholds (T ~ 0) have values near 1e-10 where that
# cancellation dominates.  Bar: |delta| <= 1e-5 |ref| + 1e-12 max|ref|.
COMPONENT_ATOL_OF_MAX = 1e-12


def _batch(adj, maps, signs=2, vd=None, floor_zero=0, maps_out=False):
    import torch
    d = torch.from_numpy(np.ascontiguousarray(maps)).cuda()
    V = maps.shape[1]
    mx = torch.empty((maps.shape[0], signs, adj.n_seg), device="cuda")
    om = torch.empty((maps.shape[0], signs, V), device="cuda") if maps_out else None
    vdd = None if vd is None else torch.from_numpy(vd).cuda()
    adj.sweep_batch(d.data_ptr(), V, maps.shape[0], signs, None if vdd is None else vdd.data_ptr(),
                    floor_zero, mx.data_ptr(), None if om is None else om.data_ptr(), 1 if maps_out else 0)
    adj.status()
    return mx.cpu().numpy(), (None if om is None else om.cpu().numpy())


def test_component_accumulation_matches_exact(config1):
    """Per-component accumulation: same components, exact sum of the same
    float increments -> within 1e-5 (relative) of the reference arithmetic."""
    st = config1
    maps = _config1_maps(st, n_perm=4, seed=21)
    vd = A.vertex_density((st.offsets, st.indices))
    adj = A.AdjacencySet((st.offsets, st.indices), 2.0, 1.0)
    mx_e, om_e = _batch(adj, maps, vd=vd, maps_out=True)
    adj.set_accumulation("component")
    mx_c, om_c = _batch(adj, maps, vd=vd, maps_out=True)
    np.testing.assert_allclose(mx_c, mx_e, rtol=COMPONENT_RTOL)
    np.testing.assert_array_equal(om_c == 0, om_e == 0)
    for m in range(om_e.shape[0]):
        for s in range(om_e.shape[1]):
            ref, got = om_e[m, s], om_c[m, s]
            tol = COMPONENT_RTOL * np.abs(ref) + COMPONENT_ATOL_OF_MAX * np.abs(ref).max()
            assert np.all(np.abs(got - ref) <= tol), (m, s, np.max(np.abs(got - ref) - tol))
    nz = om_e != 0
    rel = np.abs(om_c[nz] - om_e[nz]) / np.abs(om_e[nz])
    assert np.median(rel) <= 1e-6


def test_component_accumulation_segments_and_asymmetric(golden):
    off, idx = golden["sweep_off"], golden["sweep_idx"]
    maps = golden["sweep_maps"]
    O, I, seg = A.concat_csr([(off, idx), (off, idx)])
    adj = A.AdjacencySet((O, I), [2.0, 1.5], [1.0, 0.5], seg)
    stat = np.stack([np.concatenate([maps[0], maps[1]]), np.concatenate([maps[4], maps[5]])])
    mx_e, _ = _batch(adj, stat, floor_zero=1)
    adj.set_accumulation("component")
    mx_c, _ = _batch(adj, stat, floor_zero=1)
    np.testing.assert_allclose(mx_c, mx_e, rtol=COMPONENT_RTOL)
    mask = np.zeros((9, 8, 7), bool)
    mask[1:8, 1:7, 1:6] = True
    mask[0, 0, 0] = True
    o2, i2 = A.voxel_csr(mask, 26, "mmr")
    adj2 = A.AdjacencySet((o2, i2), 2.0, 0.5)
    rng = np.random.default_rng(9)
    m2 = (rng.standard_normal((4, o2.shape[0] - 1)) + 0.4).astype(np.float32)
    e_e, _ = _batch(adj2, m2)
    adj2.set_accumulation("component")
    e_c, _ = _batch(adj2, m2)
    np.testing.assert_allclose(e_c, e_e, rtol=COMPONENT_RTOL)


def test_maxima_only_bit_exact_with_groups_and_asymmetric_lists(golden):
    """The maxima-only form equals the exact mode bit for bit with threshold
    groups (one table per group and sign), per-segment H/E, asymmetric lists,
    a segment whose map has no positive values (an empty +x table),
    floor_zero on and off, and both CTA shapes of the per-component kernels."""
    off, idx = golden["sweep_off"], golden["sweep_idx"]
    maps = golden["sweep_maps"]
    O, I, seg = A.concat_csr([(off, idx), (off, idx), (off, idx)])
    adj = A.AdjacencySet((O, I), [2.0, 1.5, 2.0], [1.0, 0.5, 0.67], seg)
    n = off.shape[0] - 1
    neg_only = -np.abs(maps[2])
    stat = np.stack([np.concatenate([maps[0], maps[1], neg_only]),
                     np.concatenate([maps[4], neg_only, maps[5]]),
                     np.concatenate([maps[3], maps[3], maps[3]])]).astype(np.float32)
    assert stat.shape[1] == 3 * n
    for groups in (None, [0, 0, 1], [0, 1, 0]):
        adj.set_threshold_groups(groups)
        for fz in (0, 1):
            adj.set_accumulation("exact")
            mx_e, _ = _batch(adj, stat, floor_zero=fz)
            adj.set_accumulation("component")
            for shape in (3, 2):  # resident CTAs per SM of the per-component kernels
                adj.set_sweep_shape(shape)
                mx_c, _ = _batch(adj, stat, floor_zero=fz)
                np.testing.assert_array_equal(mx_c, mx_e, err_msg=f"groups={groups} floor_zero={fz} shape={shape}")
    adj.set_threshold_groups(None)
    adj.set_sweep_shape(3)
    # one sign only: the single-sign maxima-only items agree too
    adj.set_accumulation("exact")
    one_e, _ = _batch(adj, stat, signs=1, floor_zero=1)
    adj.set_accumulation("component")
    one_c, _ = _batch(adj, stat, signs=1, floor_zero=1)
    np.testing.assert_array_equal(one_c, one_e)


def test_large_segment_without_activity_bitmap():
    """A segment above the shared-memory activity bitmap's capacity (393,216
    vertices) sweeps without it: exact mode bit-identical to the oracle,
    per-component mode within its bar."""
    import torch
    rng = np.random.default_rng(71)
    mask = np.ones((80, 80, 66), bool)  # 422,400 voxels
    off, idx = A.voxel_csr(mask, 6, "pyfunc")
    V = int(mask.sum())
    maps = rng.standard_normal((2, V)).astype(np.float32)
    vol = maps.reshape(2, 80, 80, 66)
    for _ in range(2):  # light smoothing so clusters form
        vol = (vol + np.roll(vol, 1, 1) + np.roll(vol, -1, 1) + np.roll(vol, 1, 2) + np.roll(vol, -1, 2)) / 5.0
    maps = np.ascontiguousarray(vol.reshape(2, V) * 3.0, np.float32)
    adj = A.AdjacencySet((off, idx), 2.0, 0.5)
    d = torch.from_numpy(maps).cuda()
    out = torch.empty((2, 2, 1), device="cuda")
    adj.sweep_batch(d.data_ptr(), V, 2, 2, None, 0, out.data_ptr())
    adj.status()
    got = out.cpu().numpy()
    for sgn, s in enumerate((1.0, -1.0)):
        ref = oracle.tfce_max_batch(off, idx, maps, 2.0, 0.5, sign=s, hh_exact=True)
        np.testing.assert_array_equal(got[:, sgn, 0], ref)
    adj.set_accumulation("component")
    adj.sweep_batch(d.data_ptr(), V, 2, 2, None, 0, out.data_ptr())
    adj.status()
    np.testing.assert_allclose(out.cpu().numpy(), got, rtol=COMPONENT_RTOL)


@pytest.mark.parametrize("E", [1.0, 0.5])
def test_maxima_only_form_is_bit_exact(E):
    """Maxima-only launches keep each component's largest float sum (rounding
    is monotone, so that is the largest per-vertex float accumulation of its
    members): the maxima equal the exact mode's and the oracle's (correctly
    rounded HH) bit for bit, on smooth maps of both signs and two segments;
    the potential form (double sums, one rounding) is within the float
    summation error."""
    import torch
    from oracle import oracle
    from tfce_mediation_gb300 import adjacency as A
    from tfce_mediation_gb300 import synth
    v, f = synth.icosphere(5)
    o1, i1 = A.mesh_csr(f, v.shape[0])
    off, idx, seg = A.concat_csr([(o1, i1), (o1, i1)])
    V = off.shape[0] - 1
    S = synth.smoothing_matrix(off, idx)
    rng = np.random.default_rng(17)
    m = rng.standard_normal((V, 24)).astype(np.float32)
    for _ in range(5):
        m = (S @ m).astype(np.float32)
    maps = np.ascontiguousarray((3.5 * m.T / m.std()).astype(np.float32))
    adj = A.AdjacencySet((off, idx), 2.0, E, seg)
    d = torch.from_numpy(maps).cuda()
    res = {}
    for mode in ("exact", "component", "component-chain"):
        adj.set_accumulation(mode)
        out = torch.empty((24, 2, 2), device="cuda")
        adj.sweep_batch(d.data_ptr(), V, 24, 2, None, 1, out.data_ptr())
        adj.status()
        res[mode] = out.cpu().numpy()
    np.testing.assert_array_equal(res["component"], res["exact"])
    np.testing.assert_allclose(res["component"], res["component-chain"], rtol=COMPONENT_RTOL, atol=0)
    Vh = V // 2
    for i in range(0, 24, 5):
        for si, s in enumerate((1.0, -1.0)):
            for h in range(2):
                ref = oracle.tfce_max_batch(o1, i1, maps[i, h * Vh:(h + 1) * Vh], 2.0, E, sign=s,
                                            floor_zero=True, hh_exact=True)[0]
                assert res["component"][i, si, h] == ref, (i, s, h, res["component"][i, si, h], ref)
