"""Geodesic FWHM smoothing on the GPU: calc_gd_fwhm
(tfce_mediation/cynumstats.pyx:76-107) and the per-subject loop of
tools/tm_gd_fwhm_smoothing.py, batched over images.

The pair list (i, j, distance) is fixed per template: its per-vertex gather
list (pair order kept) and the Gaussian weights are formed once, then every
batch of images is one launch (one thread per vertex and image, the
reference's accumulation order and float32 roundings)."""
from __future__ import annotations

import numpy as np

from . import _lib
from .device import dev, ptr, require_cuda, stream_handle


def gather_list(indices, n_vertices):
    """Per-vertex gather list of a pair list: pair x = (i, j) gives entry
    (i, x) under vertex j and (j, x) under vertex i; each vertex's entries in
    the order the reference's scatter visits them.  Returns (off int64[V+1],
    src int32, pidx int32)."""
    ind = np.asarray(indices, np.int64).reshape(-1, 2)
    M = ind.shape[0]
    if M and (ind.min() < 0 or ind.max() >= n_vertices):
        raise ValueError("pair index outside [0, n_vertices)")
    target = np.stack([ind[:, 1], ind[:, 0]], axis=1).reshape(-1)  # (x, 0) -> j, (x, 1) -> i
    source = np.stack([ind[:, 0], ind[:, 1]], axis=1).reshape(-1)
    pair = np.repeat(np.arange(M, dtype=np.int64), 2)
    order = np.argsort(target, kind="stable")
    off = np.zeros(n_vertices + 1, np.int64)
    np.cumsum(np.bincount(target, minlength=n_vertices), out=off[1:])
    return off, source[order].astype(np.int32), pair[order].astype(np.int32)


class GeodesicSmoother:
    """Smooth images over one template's pair list: smooth(images) with images
    (B, V) or (V,) float32 -> the same shape (device compute)."""

    def __init__(self, indices, dist, sigma, n_vertices):
        t = require_cuda()
        self.t = t
        self.lib = _lib.load()
        self.V = int(n_vertices)
        off, src, pidx = gather_list(indices, self.V)
        dist = np.ascontiguousarray(dist, np.float32).reshape(-1)
        self.M = dist.shape[0]
        if self.M != len(pidx) // 2:
            raise ValueError("one distance per pair")
        self.off, self.src, self.pidx = dev(off), dev(src), dev(pidx)
        self.w = t.empty(self.M + 1, device="cuda", dtype=t.float32)
        dist_d = dev(dist) if self.M else None  # referenced until the launch is queued
        _lib.check(self.lib.gd_fwhm_weights(ptr(dist_d), self.M, float(np.float32(sigma)), ptr(self.w),
                                            stream_handle()))
        self.err = t.zeros(1, device="cuda", dtype=t.int32)

    def smooth(self, images):
        t = self.t
        x = np.asarray(images, np.float32) if not isinstance(images, t.Tensor) else images
        one = x.ndim == 1
        xd = dev(x.reshape(1, -1) if one else x, t.float32)
        B = xd.shape[0]
        if xd.shape[1] != self.V:
            raise ValueError(f"images have {xd.shape[1]} vertices, the template {self.V}")
        out = t.empty_like(xd)
        for b0 in range(0, B, 65535):
            nb = min(65535, B - b0)
            _lib.check(self.lib.gd_fwhm_smooth(ptr(self.off), ptr(self.src), ptr(self.pidx), ptr(self.w), self.M,
                                               ptr(xd[b0:]), self.V, nb, self.V, ptr(out[b0:]), self.V, ptr(self.err),
                                               stream_handle()))
        if int(self.err.item()):
            self.err.zero_()
            raise RuntimeError("gd_fwhm_smooth: a gather entry was out of range")
        res = out.cpu().numpy()
        return res[0] if one else res


def calc_gd_fwhm(indices, dist, data, sigma):
    """cynumstats.calc_gd_fwhm (cynumstats.pyx:83-107): smoothed float32 copy of
    data (V,), on the GPU."""
    data = np.asarray(data, np.float32)
    return GeodesicSmoother(indices, dist, sigma, data.shape[0]).smooth(data)
