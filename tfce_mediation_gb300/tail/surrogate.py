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

from .. import fwer
from ..device import dev
from . import gpd
from .mlp import MLP

DEFAULT_WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights.npz")


class TailSurrogate:
    def __init__(self, path=DEFAULT_WEIGHTS):
        self.model, extra = MLP.load(path)
        self.fm, self.fs = extra["feat_mean"], extra["feat_std"]
        self.tm, self.ts = extra["targ_mean"], extra["targ_std"]

    def tail(self, null_small, n_vertices, smoothness, E, n, k):
        return self.tails([gpd.features(null_small, n_vertices, smoothness, E, n, k)])[0]

    def tails(self, feats):
        """(u, xi, sigma) of several null samples in one BF16 inference:
        feats = [(features, median), ...] from gpd.features (host work that
        can run while permutations are still on the device)."""
        F = np.stack([(f - self.fm) / self.fs for f, _ in feats])
        pred = self.model.predict_bf16(F) * self.ts + self.tm
        return [gpd.decode(pred[i], m) for i, (_, m) in enumerate(feats)]


def _image_maps(img, srt, tail, alpha, margin):
    """1-p of one image from a null sorted on the device (fwer.sorted_null;
    model tail where given) and the vertices to send back: the model's p or
    the sample's own empirical p within `margin` of alpha.  Taking the union
    keeps a surrogate whose tail is biased from moving a vertex across alpha
    unchecked: the empirical p of the same sample flags it too.  Computed on
    the device: the empirical p is the calculate_fweP lookup (fwer_lookup),
    the tail and the flags elementwise."""
    import torch
    v = dev(np.ascontiguousarray(img, np.float32)).double()
    emp = fwer.lookup_presorted(srt, v)
    model = emp
    if tail is not None:
        u, xi, sigma = tail
        y = (v - u) / sigma
        if abs(xi) < 1e-9:
            sf = torch.exp(-y)
        else:
            base = torch.clamp(1.0 + xi * y, min=0.0)
            sf = torch.where(base > 0, base.pow(-1.0 / xi), torch.zeros_like(base))
        model = torch.where(v > u, 1.0 - (1.0 - gpd.QUANT) * sf, emp)
    near = (v > 0) & (((1.0 - model) - alpha).abs().le(margin) | ((1.0 - emp) - alpha).abs().le(margin))
    return model.cpu().numpy(), near.cpu().numpy()


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
    reference's CSV does.  One permutation run serves every contrast: its
    first n_small permutations give the model tails, and all of them (at
    least n_small + n_fallback, rounded up to whole batches of the engine)
    the empirical p of every vertex near alpha.  Returns ({contrast: map or list
    of maps}, info)."""
    import torch
    from ..engine import permutations
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    # the fallback permutations run with the small sample, as one pipelined
    # run: a whole-study map nearly always has vertices near alpha, and one
    # run (one pipeline fill) costs less than two.  The fallback is rounded
    # up to whole batches of the engine: a short last batch costs a full one
    # on the device, so its permutations are used rather than padded away.
    P = eng.batch
    n_fallback = max(n_fallback, 0)
    if n_fallback:
        n_fallback = -(-(n_small + n_fallback) // P) * P - n_small
    total = n_small + n_fallback
    perms = permutations(eng.n, seed, 0, total)
    need = -(-n_small // P)  # batches holding the small sample
    got, fit = {}, {}

    def small_sample():
        return np.concatenate([got[i] for i in range(need)])[:n_small].max(axis=-1)  # (n_small, C, signs)

    def host_fits():
        # the tail fits of the small sample: host work
        small = small_sample()
        for c in images:
            null = small[:, c, :].reshape(-1).astype(np.float64)
            if method == "mlp":
                fit[c] = gpd.features(null, eng.V, smoothness, E, eng.n, eng.k)
            elif method == "gpd":
                fit[c] = gpd.tail_params(null)
            else:
                fit[c] = None

    def on_batch(i, maxima):
        # once the small sample is back, its fits run while the fallback
        # permutations are still on the device
        got[i] = maxima
        if not fit and all(j in got for j in range(need)):
            host_fits()

    res = eng.run_stream(((None, perms[b:b + P]) for b in range(0, total, P)), on_batch=on_batch)
    both = np.concatenate(res).max(axis=-1)  # (total, C, signs)
    small, more = both[:n_small], both[n_small:]
    if not fit:
        host_fits()
    sur = surrogate or (TailSurrogate() if method == "mlp" else None)
    cs = list(images)
    if method == "mlp":
        tl = dict(zip(cs, sur.tails([fit[c] for c in cs])))
    else:
        tl = {c: fit[c] for c in cs}
    out, near_any, tails = {}, {}, {}
    for c, imgs in images.items():
        tail = tl[c]
        tails[c] = None if tail is None else [float(x) for x in tail]
        lst = imgs if isinstance(imgs, (list, tuple)) else [imgs]
        srt = fwer.sorted_null(small[:, c, :].reshape(-1))
        maps, nears = [], []
        for img in lst:
            omp, nr = _image_maps(img, srt, tail, alpha, margin)
            maps.append(omp)
            nears.append(nr)
        out[c] = maps
        near_any[c] = nears
    n_near = int(sum(int(n.sum()) for v in near_any.values() for n in v))
    used = n_small + n_fallback
    if n_near and n_fallback > 0:
        for c, imgs in images.items():
            srt = np.sort(np.concatenate([small[:, c, :].reshape(-1), more[:, c, :].reshape(-1)]).astype(np.float64))
            lst = imgs if isinstance(imgs, (list, tuple)) else [imgs]
            for i, img in enumerate(lst):
                nr = near_any[c][i]
                if nr.any():
                    out[c][i][nr] = gpd.one_minus_p(np.asarray(img)[nr], srt, presorted=True)
    torch.cuda.synchronize()
    res = {c: (m if isinstance(images[c], (list, tuple)) else m[0]) for c, m in out.items()}
    return res, {"perms": used, "seconds": time.perf_counter() - t0, "near_alpha": n_near, "tail": tails,
                 "fallback_vertices": near_any}
