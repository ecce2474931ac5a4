"""tcgen05 split-BF16 GLM against the FP64 oracle: the residual epilogue
(glm_tstat_tc) and the quadratic form (glm_tstat_tc_qf: t of coefficients
>= 1 of intercept designs from c = Xc'(y - centre), RSS = yy - c'inv(Xc'Xc)c).

Bar: |t_tc - t_fp64| <= 2e-4 * max(1, |t|).  Split BF16 represents each
operand to ~2^-17 relative and drops the lo.lo product, so the betas carry
~1e-5 relative error; the residual pass reads the FP32 data, and the
quadratic form's RSS carries the cross products' split error scaled by
R^2 / (1 - R^2) of the fit."""
import numpy as np
import pytest

from oracle import oracle
from tfce_mediation_gb300.glm import WHAT_T, DesignBatch, TensorCoreOperands, glm_stat, glm_tstat_tc

pytestmark = pytest.mark.gpu

TOL = 2e-4


def _err(a, ref):
    return float(np.max(np.abs(np.asarray(a, np.float64) - ref) / np.maximum(1.0, np.abs(ref))))


def _split(x):
    import torch
    xt = torch.from_numpy(np.ascontiguousarray(x, np.float32))
    hi = xt.to(torch.bfloat16)
    lo = (xt - hi.float()).to(torch.bfloat16)
    return hi.view(torch.int16).numpy(), lo.view(torch.int16).numpy()


def test_tile_layout_matches_definition():
    """Device tiles of a [rows][cols] matrix against the documented byte layout."""
    import torch
    from tfce_mediation_gb300 import _lib
    from tfce_mediation_gb300.device import ptr
    lib = _lib.load()
    rng = np.random.default_rng(5)
    rows, cols, rb, n_pad = 300, 37, 128, 48
    A = rng.standard_normal((rows, cols)).astype(np.float32)
    shift = rng.standard_normal(rows).astype(np.float32)
    nbytes = lib.glm_tile_bytes(rows, rb, n_pad)
    for transpose, with_shift in ((0, False), (1, False), (1, True)):
        src = torch.from_numpy(A.T.copy() if transpose else A).cuda()
        sh = torch.from_numpy(shift).cuda() if with_shift else None
        ld = rows if transpose else cols
        dst = torch.zeros(nbytes, dtype=torch.uint8, device="cuda")
        shifted = torch.zeros_like(src)
        _lib.check(lib.glm_tile_split(ptr(src), ld, transpose, rows, cols, ptr(sh), rb, n_pad, ptr(dst),
                                      ptr(shifted), None))
        exp_shift = (A - shift[:, None]) if with_shift else A
        np.testing.assert_array_equal(shifted.cpu().numpy(), exp_shift.T if transpose else exp_shift)
        got = dst.cpu().view(torch.int16).numpy()
        Ap = np.zeros(((rows + rb - 1) // rb * rb, n_pad), np.float32)
        Ap[:rows, :cols] = (A - shift[:, None]) if with_shift else A
        hi, lo = _split(Ap)
        KS = n_pad // 16
        exp = np.zeros_like(got)
        for R in range(Ap.shape[0]):
            for c in range(n_pad):
                base = ((R // rb * KS + c // 16) * 2) * rb * 16 + ((c % 16) // 8) * rb * 8 + (R % rb) * 8 + c % 8
                exp[base] = hi[R, c]
                exp[base + rb * 16] = lo[R, c]
        np.testing.assert_array_equal(got, exp)


@pytest.mark.parametrize("form", ["quadratic", "residual"])
@pytest.mark.parametrize("n,V,G", [(100, 10242, 40), (350, 4000, 33), (57, 777, 16), (350, 20000, 64)])
def test_tc_vs_fp64(n, V, G, form):
    rng = np.random.default_rng(n + V)
    Y = rng.standard_normal((n, V)).astype(np.float32)
    Y[:, : V // 3] += 0.4 * rng.standard_normal(n)[:, None].astype(np.float32)
    Y += 3.0  # an offset: the residual pass must not lose it
    X = np.column_stack([np.ones(n), rng.integers(0, 2, n), rng.standard_normal((n, 3))])
    perms = np.stack([rng.permutation(n) for _ in range(G)])
    db = DesignBatch(X[perms])
    coef = [1, 2, 3, 4]
    t_tc = glm_tstat_tc(Y, db, coef, quadratic_form=form == "quadratic").cpu().numpy()
    t_32 = glm_stat(Y, db, WHAT_T, coef=coef).cpu().numpy()
    e_tc, e_32 = 0.0, 0.0
    for g in range(G):
        ref = oracle.tval_fp64(X[perms[g]], Y)[coef]
        e_tc = max(e_tc, _err(t_tc[g], ref))
        e_32 = max(e_32, _err(t_32[g], ref))
    print(f"n={n} V={V} G={G} {form}: tc {e_tc:.2e}  fp32 {e_32:.2e}")
    assert e_tc <= TOL, e_tc


@pytest.mark.parametrize("ks", [(2, 3, 5, 8, 4), (6, 7, 6), (1, 1, 2)])
def test_tc_mixed_k_designs(ks):
    rng = np.random.default_rng(sum(ks))
    n, V = 120, 3000
    Y = rng.standard_normal((n, V)).astype(np.float32)
    mats = [np.column_stack([np.ones(n), rng.standard_normal((n, k - 1))]) if k > 1 else np.ones((n, 1))
            for k in ks]
    coef = [0] if min(ks) == 1 else [0, 1]
    t_tc = glm_tstat_tc(Y, DesignBatch(mats), coef).cpu().numpy()
    for g, Xg in enumerate(mats):
        ref = oracle.tval_fp64(Xg, Y)[coef]
        assert _err(t_tc[g], ref) <= TOL, (g, _err(t_tc[g], ref))


def test_tc_many_blocks_kmax7():
    """kmax 7: 16 designs per tile, 70 designs = 5 design blocks."""
    rng = np.random.default_rng(11)
    n, V, G = 200, 5000, 70
    Y = rng.standard_normal((n, V)).astype(np.float32)
    X = np.column_stack([np.ones(n), rng.standard_normal((n, 6))])
    perms = np.stack([rng.permutation(n) for _ in range(G)])
    ops = TensorCoreOperands(__import__("torch").from_numpy(Y).cuda())
    t_tc = glm_tstat_tc(Y, DesignBatch(X[perms]), [1, 6], ops=ops).cpu().numpy()
    for g in range(0, G, 7):
        ref = oracle.tval_fp64(X[perms[g]], Y)[[1, 6]]
        assert _err(t_tc[g], ref) <= TOL
    assert int(ops.err.item()) == 0


@pytest.mark.parametrize("offset", [0.0, 25.0, 1000.0])
def test_tc_offset_data(offset):
    """Data far from zero (mean/SD up to 1000): the per-vertex centring keeps
    the split error on the data's spread."""
    rng = np.random.default_rng(21)
    n, V, G = 150, 3000, 20
    Y = (offset + rng.standard_normal((n, V))).astype(np.float32)
    X = np.column_stack([np.ones(n), rng.standard_normal((n, 2))])
    perms = np.stack([rng.permutation(n) for _ in range(G)])
    t_tc = glm_tstat_tc(Y, DesignBatch(X[perms]), [1, 2]).cpu().numpy()
    for g in range(G):
        ref = oracle.tval_fp64(X[perms[g]], Y.astype(np.float64))[[1, 2]]
        assert _err(t_tc[g], ref) <= TOL, (offset, g, _err(t_tc[g], ref))


def test_tc_no_intercept_design():
    """Designs without a constant column: beta = beta_c + mean * pinv(X).1 is
    still exact."""
    rng = np.random.default_rng(8)
    n, V = 90, 2000
    Y = (5.0 + rng.standard_normal((n, V))).astype(np.float32)
    mats = [rng.standard_normal((n, 3)) + 1.0 for _ in range(5)]
    t_tc = glm_tstat_tc(Y, DesignBatch(mats), [0, 1, 2]).cpu().numpy()
    for g, Xg in enumerate(mats):
        assert _err(t_tc[g], oracle.tval_fp64(Xg, Y)[[0, 1, 2]]) <= TOL



@pytest.mark.parametrize("kmax", [3, 5])
def test_design_block_16_equals_32(kmax):
    """The tensor-core GLM with 16-design tiles (N = 128 MMA columns) gives the
    t maps of the 32-design tiles (N = 256): the same products and sums per
    design; both within the bar of the FP64 oracle."""
    import torch
    rng = np.random.default_rng(9)
    n, V, G = 120, 700, 40
    Y = rng.standard_normal((n, V)).astype(np.float32)
    X = np.concatenate([np.ones((G, n, 1)), rng.standard_normal((G, n, kmax - 1))], axis=2)
    coef = list(range(1, kmax))
    res = []
    for block in (32, 16):
        ops = TensorCoreOperands(torch.from_numpy(Y).cuda())
        ops.design_block = block
        assert ops.block(kmax) == block
        res.append(glm_tstat_tc(Y, DesignBatch(X), coef, ops=ops, quadratic_form=False).cpu().numpy())
    np.testing.assert_allclose(res[0], res[1], rtol=1e-6, atol=1e-6)
    ref = np.stack([oracle.tval_fp64(X[g], Y)[coef] for g in range(G)])
    assert _err(res[1], ref) <= TOL


@pytest.mark.parametrize("kmax", [2, 3, 4, 5, 6, 7, 8])
def test_quadratic_form_every_kmax(kmax):
    """Every column count: 4 rows per design (64-design tiles) up to kmax 5,
    8 rows (32-design tiles) above; 70 designs leave a partial design tile
    and 1,000 vertices a partial vertex tile."""
    import torch
    rng = np.random.default_rng(40 + kmax)
    n, V, G = 97, 1000, 70
    Y = (2.0 + rng.standard_normal((n, V))).astype(np.float32)
    X = np.column_stack([np.ones(n), rng.standard_normal((n, kmax - 1))])
    perms = np.stack([rng.permutation(n) for _ in range(G)])
    db = DesignBatch(X[perms])
    coef = list(range(1, kmax))
    ops = TensorCoreOperands(torch.from_numpy(Y).cuda())
    assert ops.qf_ok(db, coef)
    t_qf = glm_tstat_tc(Y, db, coef, ops=ops).cpu().numpy()
    assert int(ops.err.item()) == 0
    ref = np.stack([oracle.tval_fp64(X[perms[g]], Y)[coef] for g in range(G)])
    assert _err(t_qf, ref) <= TOL, _err(t_qf, ref)


@pytest.mark.parametrize("r2", [0.5, 0.9, 0.97])
def test_quadratic_form_strong_fits(r2):
    """Vertices whose data the design explains to R^2 = 0.5 .. 0.97 (the
    unpermuted design, t up to ~100): the quadratic form's RSS = yy - c'b
    loses relative precision as R^2 / (1 - R^2); within the bar up to 0.97."""
    rng = np.random.default_rng(int(r2 * 100))
    n, V, G = 350, 2048, 8
    X = np.column_stack([np.ones(n), rng.integers(0, 2, n), rng.standard_normal((n, 3))])
    fit = X[:, 1:] @ rng.standard_normal((4, V))
    fit /= fit.std(axis=0, keepdims=True)
    noise = rng.standard_normal((n, V))
    noise /= noise.std(axis=0, keepdims=True)
    Y = (10.0 + np.sqrt(r2) * fit + np.sqrt(1.0 - r2) * noise).astype(np.float32)
    designs = np.stack([X] + [X[rng.permutation(n)] for _ in range(G - 1)])
    coef = [1, 2, 3, 4]
    t_qf = glm_tstat_tc(Y, DesignBatch(designs), coef, quadratic_form=True).cpu().numpy()
    e = max(_err(t_qf[g], oracle.tval_fp64(designs[g], Y)[coef]) for g in range(G))
    print(f"R^2 {r2}: quadratic form {e:.2e}")
    assert e <= TOL, e


def test_quadratic_form_mixed_k_designs():
    """The mediation engine's batches: designs [1, x] and [1, x, m] padded to
    kmax 3; the shorter design's missing column has zero cross products and
    inverse rows."""
    rng = np.random.default_rng(77)
    n, V = 150, 1500
    Y = rng.standard_normal((n, V)).astype(np.float32)
    x, m = rng.standard_normal(n), rng.standard_normal(n)
    mats = []
    for g in range(24):
        p = rng.permutation(n)
        mats.append(np.column_stack([np.ones(n), x[p]]) if g % 2 == 0 else np.column_stack([np.ones(n), x[p], m]))
    db = DesignBatch(mats, kmax=3)
    t_qf = glm_tstat_tc(Y, db, [1], quadratic_form=True).cpu().numpy()
    t_res = glm_tstat_tc(Y, db, [1], quadratic_form=False).cpu().numpy()
    for g, Xg in enumerate(mats):
        ref = oracle.tval_fp64(Xg, Y)[[1]]
        assert _err(t_qf[g], ref) <= TOL, (g, _err(t_qf[g], ref))
    assert _err(t_qf, t_res.astype(np.float64)) <= TOL


def test_quadratic_form_coefficient_outside_design_is_nan():
    """A requested coefficient outside [1, kmax) gives a NaN row through the
    C ABI (the documented behaviour), the other rows unaffected."""
    import torch
    from tfce_mediation_gb300.device import dev
    rng = np.random.default_rng(3)
    n, V, G, k = 80, 600, 10, 4
    Y = rng.standard_normal((n, V)).astype(np.float32)
    X = np.column_stack([np.ones(n), rng.standard_normal((n, k - 1))])
    db = DesignBatch(np.stack([X[rng.permutation(n)] for _ in range(G)]))
    ops = TensorCoreOperands(torch.from_numpy(Y).cuda())
    XR, GI = ops.host_operands_qf(db)
    xt = ops.tile_designs_qf(dev(XR), G, k)
    out = torch.empty((G, 2, V), device="cuda")
    ops.tstat_qf(xt, dev(GI), dev(db.invdiag64.astype(np.float32)), dev(db.dof.astype(np.float32)), G, k,
                 dev(np.array([2, 7], np.int32)), 2, out, V)
    got = out.cpu().numpy()
    assert np.isnan(got[:, 1]).all()
    ref = np.stack([oracle.tval_fp64(db.X64[g], Y)[2] for g in range(G)])
    assert _err(got[:, 0], ref) <= TOL
