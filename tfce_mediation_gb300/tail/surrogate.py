"""Learned-tail FWER maps with margin-triggered fallback.

learned_fwer() runs a small number of permutations, predicts the GPD tail of
the max-TFCE null from them (the trained MLP, BF16 inference), maps every
TFCE value to 1-p(FWER), and sends every vertex whose p-value lies within
`margin` of alpha -- by the surrogate's p or by the small sample's own
empirical p -- back for more permutations (the empirical p of the extended
null replaces the surrogate there).  method="gpd" uses the classical
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


def _maxima(eng, start, count, seed):
    """(count, C, signs) per-permutation maxima (max over segments): whole
    batches through the captured graphs, the remainder as one short batch
    (no padding to a full batch)."""
    P = eng.batch
    full = count // P * P
    parts = []
    if full:
        parts.append(eng.run_graph(start=start, stop=start + full, seed=seed))
    if count > full:
        parts.append(eng.run(start=start + full, stop=start + count, seed=seed))
    return np.concatenate(parts).max(axis=-1)


def _image_maps(img, srt, tail, alpha, margin):
    """1-p of one image from a sorted null (model tail where given) and the
    vertices to send back: the model's p or the sample's own empirical p
    within `margin` of alpha.  Taking the union keeps a surrogate whose tail
    is biased from moving a vertex across alpha unchecked: the empirical p of
    the same sample flags it too."""
    v = np.asarray(img, np.float64)
    pos = v > 0
    vp = v[pos]
    emp = np.maximum(np.searchsorted(srt, vp, side="left") - 1, 0) / srt.shape[0]
    model = emp if tail is None else gpd.apply_tail(emp.copy(), vp, *tail)
    omp = np.zeros(v.shape[0])
    omp[pos] = model
    near = np.zeros(v.shape[0], bool)
    near[pos] = (np.abs((1.0 - model) - alpha) <= margin) | (np.abs((1.0 - emp) - alpha) <= margin)
    return omp, near


def learned_fwer(eng, tfce_values, contrast, smoothness, E, alpha=0.05, margin=0.02, n_small=300,
                 n_fallback=1200, seed=0, method="mlp", surrogate=None):
    """1-p(FWER) of `tfce_values` (observed TFCE image, host) for one contrast
    of a PermutationEngine; returns (map, info)."""
    maps, info = learned_fwer_maps(eng, {contrast: tfce_values}, smoothness, E, alpha, margin, n_small,
                                   n_fallback, seed, method, surrogate)
    return maps[contrast], info


def learned_fwer_maps(eng, images, smoothness, E, alpha=0.05, margin=0.02, n_small=300, n_fallback=1200,
                      seed=0, method="mlp", surrogate=None):
    """1-p(FWER) maps of several observed TFCE images at once.  images:
    {contrast index: image or list of images (e.g. the + and - images)}; the
    null of a contrast holds both signs' maxima of every permutation, as the
    reference's CSV does.  One small permutation run serves every contrast;
    one fallback run serves every vertex near alpha.  Returns ({contrast:
    map or list of maps}, info)."""
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    small = _maxima(eng, 0, n_small, seed)  # (n_small, C, signs)
    sur = surrogate or (TailSurrogate() if method == "mlp" else None)
    out, near_any, tails = {}, {}, {}
    for c, imgs in images.items():
        null = small[:, c, :].reshape(-1).astype(np.float64)
        tail = None
        if method == "mlp":
            tail = sur.tail(null, eng.V, smoothness, E, eng.n, eng.k)
        elif method == "gpd":
            tail = gpd.tail_params(null)
        tails[c] = None if tail is None else [float(x) for x in tail]
        lst = imgs if isinstance(imgs, (list, tuple)) else [imgs]
        srt = np.sort(null)
        maps, nears = [], []
        for img in lst:
            omp, nr = _image_maps(img, srt, tail, alpha, margin)
            maps.append(omp)
            nears.append(nr)
        out[c] = maps
        near_any[c] = nears
    n_near = int(sum(int(n.sum()) for v in near_any.values() for n in v))
    used = n_small
    if n_near and n_fallback > 0:
        more = _maxima(eng, n_small, n_fallback, seed)
        for c, imgs in images.items():
            srt = np.sort(np.concatenate([small[:, c, :].reshape(-1), more[:, c, :].reshape(-1)]).astype(np.float64))
            lst = imgs if isinstance(imgs, (list, tuple)) else [imgs]
            for i, img in enumerate(lst):
                nr = near_any[c][i]
                if nr.any():
                    out[c][i][nr] = gpd.one_minus_p(np.asarray(img)[nr], srt, presorted=True)
        used += n_fallback
    torch.cuda.synchronize()
    res = {c: (m if isinstance(images[c], (list, tuple)) else m[0]) for c, m in out.items()}
    return res, {"perms": used, "seconds": time.perf_counter() - t0, "near_alpha": n_near, "tail": tails,
                 "fallback_vertices": near_any}
