"""Learned-tail FWER maps with margin-triggered fallback.

learned_fwer() runs a small number of permutations, predicts the GPD tail of
the max-TFCE null from them (the trained MLP, BF16 inference), maps every
TFCE value to 1-p(FWER), and sends every vertex whose p-value lies within
`margin` of alpha back for more permutations (the empirical p of the
extended null replaces the surrogate there).  method="gpd" uses the classical
maximum-likelihood GPD fit of the same small sample instead of the network,
method="empirical" no tail model at all -- the comparisons that show what the
network gains.
"""
from __future__ import annotations

import os
import time

import numpy as np

from . import gpd
from .mlp import MLP

DEFAULT_WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights.npz")


class TailSurrogate:
    def __init__(self, path=DEFAULT_WEIGHTS):
        self.model, extra = MLP.load(path)
        self.fm, self.fs = extra["feat_mean"], extra["feat_std"]
        self.tm, self.ts = extra["targ_mean"], extra["targ_std"]

    def tail(self, null_small, n_vertices, smoothness, E, n, k):
        f, m = gpd.features(null_small, n_vertices, smoothness, E, n, k)
        pred = self.model.predict_bf16(((f - self.fm) / self.fs)[None])[0] * self.ts + self.tm
        return gpd.decode(pred, m)


def _null(eng, start, count, seed, contrast):
    mx = eng.run_graph(start=start, stop=start + count, seed=seed) if count >= eng.batch else \
        eng.run(start=start, stop=start + count, seed=seed)
    return mx[:, contrast, :, :].max(axis=-1).reshape(-1).astype(np.float64)


def learned_fwer(eng, tfce_values, contrast, smoothness, E, alpha=0.05, margin=0.01, n_small=300,
                 n_fallback=1700, seed=0, method="mlp", surrogate=None):
    """1-p(FWER) of `tfce_values` (observed TFCE image, host) for one contrast
    of a PermutationEngine; returns (map, info)."""
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    null = _null(eng, 0, n_small, seed, contrast)
    tail = None
    if method == "mlp":
        sur = surrogate or TailSurrogate()
        tail = sur.tail(null, eng.V, smoothness, E, eng.n, eng.k)
    elif method == "gpd":
        tail = gpd.tail_params(null)
    omp = gpd.one_minus_p(tfce_values, null, *(tail or (None, None, None)))
    p = 1.0 - omp
    near = (np.abs(p - alpha) <= margin) & (np.asarray(tfce_values) > 0)
    used = n_small
    if near.any() and n_fallback > 0:
        null_all = np.concatenate([null, _null(eng, n_small, n_fallback, seed, contrast)])
        omp[near] = gpd.one_minus_p(np.asarray(tfce_values)[near], null_all)
        used += n_fallback
    torch.cuda.synchronize()
    return omp, {"perms": used, "seconds": time.perf_counter() - t0, "near_alpha": int(near.sum()),
                 "tail": None if tail is None else [float(x) for x in tail]}
