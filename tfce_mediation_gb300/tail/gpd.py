"""Generalised-Pareto tail of a max-TFCE null, features of a small null
sample, and p-values.

p-values keep the convention of tfce_mediation/tmanalysis/calculate_fweP_vertex.py:37-69
below the tail threshold u (1-p = max(idx-1, 0)/N with idx = #{null < x});
above u the tail is P(M > x) = p_u (1 + xi (x - u) / sigma)^(-1/xi) with
p_u = 1 - QUANT (u is the QUANT quantile of the null sample).
"""
from __future__ import annotations

import numpy as np

QUANT = 0.90
FEATURE_QUANTILES = (0.05, 0.1, 0.25, 0.5, 0.75, 0.9, 0.95, 0.975, 0.99)
N_FEATURES = len(FEATURE_QUANTILES) + 1 + 3 + 3 + 5


def fit_gpd(exceedances):
    """(xi, sigma) maximum-likelihood fit of a GPD to positive exceedances
    (scipy.stats.genpareto, location fixed at 0); falls back to the method of
    moments when the optimiser fails."""
    y = np.asarray(exceedances, np.float64)
    y = y[y > 0]
    if y.size < 5:
        return 0.0, float(max(np.mean(y), 1e-12)) if y.size else 1e-12
    try:
        from scipy.stats import genpareto
        xi, _, sigma = genpareto.fit(y, floc=0)
        if np.isfinite(xi) and np.isfinite(sigma) and sigma > 0:
            return float(np.clip(xi, -0.9, 2.0)), float(sigma)
    except Exception:
        pass
    m, v = np.mean(y), np.var(y)
    xi = 0.5 * (1 - m * m / max(v, 1e-300))
    return float(np.clip(xi, -0.9, 2.0)), float(max(0.5 * m * (m * m / max(v, 1e-300) + 1), 1e-12))


def tail_params(null, quant=QUANT):
    """(u, xi, sigma) of a null sample: u its quant quantile, GPD on the excess."""
    s = np.asarray(null, np.float64)
    u = float(np.quantile(s, quant))
    xi, sigma = fit_gpd(s[s > u] - u)
    return u, xi, sigma


def features(null, n_vertices, smoothness, E, n, k):
    """Summary of a small null sample (a few hundred permutation maxima) plus
    the study's size and smoothness (mean correlation between neighbouring
    vertices across subjects, see data.neighbour_correlation); scale-free
    (log of maxima / median)."""
    s = np.maximum(np.asarray(null, np.float64), 1e-12)
    m = float(np.median(s))
    z = np.log(s / m)
    q = np.quantile(z, FEATURE_QUANTILES)
    sd = float(np.std(z)) + 1e-12
    skew = float(np.mean(((z - z.mean()) / sd) ** 3))
    u, xi, sigma = tail_params(s)
    meta = [np.log(n_vertices) / 12.0, float(smoothness), float(E), np.log(n) / 6.0, k / 6.0]
    f = np.concatenate([q, [z.max()], [z.mean(), sd, skew],
                        [np.clip(xi, -0.9, 2.0), np.log(sigma / m), np.log(u / m)], meta])
    return f.astype(np.float32), m


def targets(full_null, m):
    """Regression target of a setting: the tail of its full null relative to
    the small sample's median m: (xi, log(sigma/m), log(u/m))."""
    u, xi, sigma = tail_params(full_null)
    return np.asarray([xi, np.log(sigma / m), np.log(u / m)], np.float32)


def decode(pred, m):
    """(u, xi, sigma) from a network output row and the sample median."""
    xi = float(np.clip(pred[0], -0.9, 2.0))
    return float(m * np.exp(pred[2])), xi, float(m * np.exp(pred[1]))


def apply_tail(out, v, u, xi, sigma, quant=QUANT):
    """Overwrite out[i] with the GPD tail's 1-p where v[i] > u."""
    tail = v > u
    if np.any(tail):
        y = (v[tail] - u) / sigma
        if abs(xi) < 1e-9:
            sf = np.exp(-y)
        else:
            base = np.maximum(1.0 + xi * y, 0.0)
            sf = np.where(base > 0, base ** (-1.0 / xi), 0.0)
        out[tail] = 1.0 - (1.0 - quant) * sf
    return out


def one_minus_p(values, null, u=None, xi=None, sigma=None, quant=QUANT, presorted=False):
    """1-p(FWER) of TFCE values given a null sample and (optionally) a tail.
    Without a tail this is exactly the reference's calculate_fweP formula."""
    srt = np.asarray(null, np.float64) if presorted else np.sort(np.asarray(null, np.float64))
    N = srt.shape[0]
    v = np.asarray(values, np.float64)
    idx = np.searchsorted(srt, v, side="left")
    out = np.maximum(idx - 1, 0) / N
    if u is not None:
        apply_tail(out, v, u, xi, sigma, quant)
    out[v <= 0] = 0.0
    return out
