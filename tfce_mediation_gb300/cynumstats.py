"""Drop-in for ``tfce_mediation.cynumstats`` (tfce_mediation/cynumstats.pyx).

Same names, arguments and return shapes; the n x V work runs on the GPU.
``tval_int`` and ``calc_beta_se`` use the FP64 kernel (``glm_stat_f64``)
with the reference's precision: betas and sigma^2 in float64, SE rounded to
float32 (cynumstats.pyx:47-52), t = beta / SE.  The other helpers use the
float32 kernel (``glm_stat``).  Results come back as host float64 arrays like
the reference's, except ``se`` outputs, which the reference itself returns as
float32.
"""
from __future__ import annotations

import numpy as np

from .gd_fwhm import calc_gd_fwhm  # noqa: F401  (cynumstats.pyx:76-107, on the GPU)
from .glm import WHAT_BETA, WHAT_RESID, WHAT_RSS, WHAT_SE, WHAT_T, DesignBatch, glm_fstat, glm_stat, glm_stat_f64


def _as_2d(y):
    y = np.asarray(y)
    return (y[:, None], True) if y.ndim == 1 else (y, False)


def _host(t, squeeze_last=False):
    a = t.detach().to("cpu").numpy().astype(np.float64)
    return a[..., 0] if squeeze_last else a


def cy_lin_lstsqr_mat(X, y):
    """inv(X'X) X' y (cynumstats.pyx:28-29): (k, V) betas."""
    X = np.asarray(X, np.float64)
    y2, sq = _as_2d(y)
    out = glm_stat(y2.astype(np.float32), DesignBatch([X]), WHAT_BETA)[0]
    return _host(out, sq)


def tval_int(X, invXX, y, n, k, numvoxel):
    """t of every coefficient (cynumstats.pyx:59-64): (k, V).  Betas use
    inv(X'X) recomputed from X (as cy_lin_lstsqr_mat does); the SE factor uses
    the diagonal of the invXX passed in."""
    X = np.asarray(X, np.float64)
    y2, sq = _as_2d(y)
    db = DesignBatch([X], invXX=np.asarray(invXX, np.float64)[None])
    if db.dof[0] != n - k:
        db.dof[0] = n - k
    out = glm_stat_f64(y2.astype(np.float32), db, WHAT_T)[0]
    return _host(out, sq)


def calc_beta_se(x, y, n, num_voxel):
    """Design [1, x]; returns (beta of column 1, se (k, V) float32)
    (cynumstats.pyx:66-74)."""
    X = np.column_stack([np.ones(n), x])
    y2, sq = _as_2d(y)
    Yf = y2.astype(np.float32)
    db = DesignBatch([X])
    beta = glm_stat_f64(Yf, db, WHAT_BETA, coef=[1])[0, 0]
    se = glm_stat_f64(Yf, db, WHAT_SE)[0]
    b = beta.to("cpu").numpy().astype(np.float64)
    s = se.to("cpu").numpy().astype(np.float32)
    return (b[0], s[:, 0]) if sq else (b, s)


def se_of_slope(num_voxel, invXX, sigma2, k):
    """sqrt(diag(sigma2_j * invXX)) as float32 (cynumstats.pyx:47-52); an
    elementwise host helper (the fused kernel computes SE itself)."""
    d = np.diag(np.asarray(invXX, np.float64))
    return np.sqrt(np.asarray(sigma2, np.float64)[None, :] * d[:, None]).astype(np.float32)


def resid_covars(x_covars, data):
    """Residuals of data (V x n) on x_covars (n x c) (cynumstats.pyx:54-57): (n, V)."""
    Y = np.ascontiguousarray(np.asarray(data).T, np.float32)
    out = glm_stat(Y, DesignBatch([np.asarray(x_covars, np.float64)]), WHAT_RESID)[0]
    return _host(out)


def calcF(X, y, n, k):
    """Model F per column (cynumstats.pyx:31-36); like the reference, TSS is
    taken around np.mean(y), the grand mean of the whole matrix."""
    X = np.asarray(X, np.float64)
    y2, sq = _as_2d(y)
    db = DesignBatch([X])
    db.dof[0] = n - k
    out = glm_fstat(y2.astype(np.float32), db, centre=float(np.mean(y2)))[0]
    a = out.to("cpu").numpy().astype(np.float64)
    return a[0] if sq else a


def cy_lin_lstsqr_mat_residual(exog_vars, endog_arr):
    """(betas, RSS) (cynumstats.pyx:109-112)."""
    X = np.asarray(exog_vars, np.float64)
    y2, sq = _as_2d(endog_arr)
    Yf = y2.astype(np.float32)
    db = DesignBatch([X])
    a = _host(glm_stat(Yf, db, WHAT_BETA)[0], sq)
    r = glm_stat(Yf, db, WHAT_RSS)[0].to("cpu").numpy().astype(np.float64)
    return a, (r[0] if sq else r)


def cython_lstsqr(x, y):
    """Simple-regression intercept and slope (cynumstats.pyx:38-45); a scalar
    host helper the pipeline never calls."""
    x = np.asarray(x, np.float64)
    y = np.asarray(y, np.float64)
    x_avg, y_avg = x.mean(), y.mean()
    slope = np.sum((x - x_avg) * (y - y_avg)) / np.sum((x - x_avg) ** 2)
    return (y_avg - slope * x_avg, slope)

