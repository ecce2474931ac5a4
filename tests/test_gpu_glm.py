"""GLM kernels on the GPU against the reference's own values (golden vectors)
and the FP64 oracle.

Tolerance (FP32 path): |t_gpu - t_ref| <= 1e-4 * max(1, |t_ref|), i.e. the
relative tolerance of the FP32 path with an absolute floor for t near 0
(the kernel accumulates n-term dot products in float32).  FP64 path
(tval_int, calc_beta_se, glm_stat_f64): t within 1e-6 relative of the
reference's (the SE is rounded to float32 in both; only the order of the
double sums differs, which can move that rounding by one float ulp), and
most values exactly equal in float32.
"""
import numpy as np
import pytest

from oracle import oracle
from tfce_mediation_gb300 import cynumstats as cy
from tfce_mediation_gb300.glm import DesignBatch, WHAT_T, glm_stat

pytestmark = pytest.mark.gpu

T_TOL = 1e-4


def assert_t_close(got, ref, tol=T_TOL):
    ref = np.asarray(ref, np.float64)
    err = np.abs(np.asarray(got, np.float64) - ref) / np.maximum(1.0, np.abs(ref))
    assert np.nanmax(err) <= tol, f"max scaled error {np.nanmax(err):.3e}"


def test_tval_int(golden):
    y, x = golden["glm_y"], golden["glm_x"]
    n, V = y.shape
    X = np.column_stack([np.ones(n), x])
    t = cy.tval_int(X, np.linalg.inv(X.T @ X), y, n, X.shape[1], V)
    assert t.shape == golden["glm_tval_int"].shape and t.dtype == np.float64
    ref = golden["glm_tval_int"]
    np.testing.assert_allclose(t, ref, rtol=1e-6, atol=1e-12)
    # cast to float32 as callers do before sweeping: almost every value is the reference's
    assert np.mean(t.astype(np.float32) == ref.astype(np.float32)) >= 0.99


def test_calc_beta_se_and_lstsqr(golden):
    y, x = golden["glm_y"], golden["glm_x"]
    n, V = y.shape
    b, se = cy.calc_beta_se(x[:, 0], y, n, V)
    np.testing.assert_allclose(b, golden["glm_cbs_beta"], rtol=1e-10, atol=1e-12)
    assert se.dtype == np.float32
    np.testing.assert_allclose(se, golden["glm_cbs_se"], rtol=2e-7)
    X = np.column_stack([np.ones(n), x])
    np.testing.assert_allclose(cy.cy_lin_lstsqr_mat(X, y), golden["glm_lstsqr"], rtol=1e-4, atol=1e-5)
    a, rss = cy.cy_lin_lstsqr_mat_residual(X, y)
    np.testing.assert_allclose(a, golden["glm_lsr_a"], rtol=1e-4, atol=1e-5)
    np.testing.assert_allclose(rss, golden["glm_lsr_rss"], rtol=1e-4)


def test_resid_covars_and_calcF(golden):
    y, x = golden["glm_y"], golden["glm_x"]
    n, V = y.shape
    X = np.column_stack([np.ones(n), x])
    np.testing.assert_allclose(cy.resid_covars(X[:, :2], y.T), golden["glm_resid_covars"],
                               rtol=1e-4, atol=1e-5)
    np.testing.assert_allclose(cy.calcF(X, y, n, X.shape[1]), golden["glm_calcF"], rtol=1e-4, atol=1e-5)


def test_se_of_slope(golden):
    y, x = golden["glm_y"], golden["glm_x"]
    n, V = y.shape
    X = np.column_stack([np.ones(n), x])
    se = cy.se_of_slope(V, np.linalg.inv(X.T @ X), golden["glm_sig2"], X.shape[1])
    np.testing.assert_array_equal(se, golden["glm_se_of_slope"])


def test_permuted_batch_vs_fp64_oracle(config1):
    st = config1
    X = st.design()
    perms = np.stack([np.random.RandomState(100 + p).permutation(st.n) for p in range(24)])
    t = glm_stat(st.Y, DesignBatch(X[perms]), WHAT_T, coef=[1, 2]).cpu().numpy()
    for p in range(perms.shape[0]):
        ref = oracle.tval_fp64(X[perms[p]], st.Y)
        assert_t_close(t[p], ref[1:3])


def test_mixed_k_designs(config1):
    """Designs of different k in one launch (the mediation a/b paths)."""
    st = config1
    x = st.pred_x[:, 0]
    Xa = np.column_stack([np.ones(st.n), x])
    Xb = np.column_stack([np.ones(st.n), st.pred_x[:, 1], x])
    t = glm_stat(st.Y, DesignBatch([Xa, Xb]), WHAT_T, coef=[1]).cpu().numpy()
    assert_t_close(t[0, 0], oracle.tval_fp64(Xa, st.Y)[1])
    assert_t_close(t[1, 0], oracle.tval_fp64(Xb, st.Y)[1])


@pytest.mark.parametrize("medtype", ["I", "M", "Y"])
@pytest.mark.parametrize("alg", ["aroian", "sobel", "goodman"])
def test_sobelz(golden, medtype, alg):
    from tfce_mediation_gb300 import pyfunc
    n = golden["sobel_x"].shape[0]
    V = golden["sobel_y"].shape[1]
    z = pyfunc.calc_sobelz(medtype, golden["sobel_x"], golden["sobel_dy"], golden["sobel_y"], n, V, alg=alg)
    ref = golden[f"sobel_{medtype}_{alg}"]
    fin = np.isfinite(ref)
    np.testing.assert_array_equal(np.isfinite(z), fin)
    np.testing.assert_allclose(z[fin], ref[fin], rtol=2e-4, atol=1e-5)
