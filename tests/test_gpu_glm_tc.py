"""tcgen05 split-BF16 GLM against the FP32 CUDA-core GLM and the FP64 oracle.

Bar: |t_tc - t_fp64| <= 2e-4 * max(1, |t|) (split BF16 drops the lo.lo term,
~2^-16 relative per product, and the residual pass reads y = hi + lo)."""
import numpy as np
import pytest

from oracle import oracle
from tfce_mediation_gb300.glm import WHAT_T, DesignBatch, glm_stat, glm_tstat_tc

pytestmark = pytest.mark.gpu

TOL = 2e-4


def _err(a, ref):
    return float(np.max(np.abs(np.asarray(a, np.float64) - ref) / np.maximum(1.0, np.abs(ref))))


@pytest.mark.parametrize("n,V,G", [(100, 10242, 40), (350, 4000, 33), (57, 777, 16)])
def test_tc_vs_fp32_and_fp64(n, V, G):
    rng = np.random.default_rng(n + V)
    Y = rng.standard_normal((n, V)).astype(np.float32)
    Y[:, : V // 3] += 0.4 * rng.standard_normal(n)[:, None].astype(np.float32)
    X = np.column_stack([np.ones(n), rng.integers(0, 2, n), rng.standard_normal((n, 3))])
    perms = np.stack([rng.permutation(n) for _ in range(G)])
    db = DesignBatch(X[perms])
    coef = [1, 2, 3, 4]
    t_tc = glm_tstat_tc(Y, db, coef).cpu().numpy()
    t_32 = glm_stat(Y, db, WHAT_T, coef=coef).cpu().numpy()
    e_tc, e_32 = 0.0, 0.0
    for g in range(G):
        ref = oracle.tval_fp64(X[perms[g]], Y)[coef]
        e_tc = max(e_tc, _err(t_tc[g], ref))
        e_32 = max(e_32, _err(t_32[g], ref))
    print(f"n={n} V={V} G={G}: tc {e_tc:.2e}  fp32 {e_32:.2e}")
    assert e_tc <= TOL, e_tc


def test_tc_mixed_k_designs():
    rng = np.random.default_rng(9)
    n, V = 120, 3000
    Y = rng.standard_normal((n, V)).astype(np.float32)
    mats = [np.column_stack([np.ones(n), rng.standard_normal((n, k - 1))]) for k in (2, 3, 5, 8, 4)]
    t_tc = glm_tstat_tc(Y, DesignBatch(mats), [1]).cpu().numpy()
    for g, Xg in enumerate(mats):
        assert _err(t_tc[g, 0], oracle.tval_fp64(Xg, Y)[1]) <= TOL
