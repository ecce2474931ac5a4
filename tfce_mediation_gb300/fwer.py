"""1-p(FWER) from permutation maxima on the device (fwer_sort / fwer_lookup).

* ``fwep`` -- tfce_mediation/tmanalysis/calculate_fweP_vertex.py:37-69 and
  calculate_fweP_voxel.py:23-49: 1-p = max(idx-1, 0)/N where idx counts the
  null maxima below the TFCE value, only where TFCE > 0.
* ``nearest`` -- tfce_mediation/tm_func.py:566-573: p_array of the nearer rank.
* ``apply_mfwer`` -- tfce_mediation/tm_func.py:403-491: per-surface
  log-standardisation of the maxima and images, optional log-mask-size weighted
  surface choice, nearest-rank lookup of every vertex on the device.
"""
from __future__ import annotations

import numpy as np

from . import _lib
from .device import dev, ptr, require_cuda, stream_handle


def sorted_null(null):
    """Device copy of the null maxima, sorted ascending (float64)."""
    t = require_cuda()
    d = dev(np.asarray(null, np.float64), t.float64).clone()
    _lib.check(_lib.load().fwer_sort(ptr(d), d.numel(), stream_handle()))
    return d


def _lookup(srt, image, mode):
    t = require_cuda()
    img = dev(np.asarray(image, np.float64) if not isinstance(image, t.Tensor) else image, t.float64)
    out = t.empty_like(img)
    _lib.check(_lib.load().fwer_lookup(ptr(srt), srt.numel(), ptr(img), img.numel(), mode, ptr(out),
                                       stream_handle()))
    return out


def fwep(tfce_image, null):
    """1-p(FWER) image (host float64) for a TFCE image and its null maxima."""
    return _lookup(sorted_null(null), tfce_image, 0).cpu().numpy()


def fwep_presorted(srt, tfce_image):
    """fwep against a null already sorted on the device (sorted_null), so
    that several images share one sort; host float64."""
    return _lookup(srt, tfce_image, 0).cpu().numpy()


def lookup_presorted(srt, tfce_image):
    """fwep_presorted left on the device (float64 tensor)."""
    return _lookup(srt, tfce_image, 0)


def nearest(values, null):
    return _lookup(sorted_null(null), values, 1).cpu().numpy()


def accuracy(num_perm):
    """The +/- margin the reference prints (calculate_fweP_vertex.py:75)."""
    return 2 * (np.sqrt(0.05 * 0.95 / num_perm))


def apply_mfwer(pos_images, neg_images, perm_max, position_array, weight=None, mediation=False):
    """tm_func.apply_mfwer with the permutation CSV contents passed in memory:
    perm_max[(surface, contrast)] -> 1-D maxima.  Returns (pos_1mp, neg_1mp)."""
    pos_images = np.asarray(pos_images, np.float64)
    num_contrasts = pos_images.shape[1]
    num_surf = len(position_array) - 1
    num_perm = min(len(v) for v in perm_max.values())
    if weight == "logmasksize":
        x = np.diff(np.asarray(position_array, np.float64))
        weights = (np.log(x) / np.log(x).sum()) / np.mean(np.log(x) / np.log(x).sum())
    V = pos_images.shape[0]
    pos_out = np.zeros((V, num_contrasts))
    neg_out = None if mediation else np.zeros((V, num_contrasts))
    with np.errstate(divide="ignore", invalid="ignore"):
        for c in range(num_contrasts):
            temp_max = np.zeros((num_perm, num_surf))
            w_temp_max = np.zeros((num_perm, num_surf))
            pos_lt = np.zeros(V)
            neg_lt = np.zeros(V)
            for s in range(num_surf):
                lp = np.log(np.asarray(perm_max[(s, c)], np.float64)[:num_perm])
                lp[np.isinf(lp)] = 0
                a, b = position_array[s], position_array[s + 1]
                mu, sd = lp.mean(), lp.std()
                for src, dst in ((pos_images, pos_lt),) + (() if mediation else ((neg_images, neg_lt),)):
                    seg = np.asarray(src, np.float64)[a:b, c]
                    lv = np.log(seg)
                    vm = lv > 0
                    dst[a:b][vm] = (((lv[vm] - mu) / sd) + 10)
                z = (lp - mu) / sd
                if weight == "logmasksize":
                    w_temp_max[:, s] = z * weights[s] + 10
                temp_max[:, s] = z + 10
            if weight is not None:
                w_temp_max[np.isnan(w_temp_max)] = 0
                mi = np.argmax(w_temp_max, axis=1)
                mv = temp_max[np.arange(num_perm), mi].astype(np.float32)
            else:
                mv = temp_max.max(axis=1)
            srt = sorted_null(mv.astype(np.float64))
            pos_out[:, c] = _lookup(srt, pos_lt, 1).cpu().numpy()
            if not mediation:
                neg_out[:, c] = _lookup(srt, neg_lt, 1).cpu().numpy()
    return pos_out, neg_out
