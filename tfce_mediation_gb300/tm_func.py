"""Drop-in for the multimodal multisurface (mmr) bodies of ``tfce_mediation.tm_func``.

Same names, arguments, outputs and CSV files as tfce_mediation/tm_func.py.
Every call is one GLM launch (t of all contrasts, or the path-a / path-b t of
the indirect effect) and one sweep launch over every (contrast, sign, surface)
of the study on the GPU; surfaces are segments of one device adjacency cut
from the caller's merged adjacency (the masked vertices of each surface, in
position_array order), and the threshold tables follow the reference's sweep
of the merged image:

* calculate_tfce              (tm_func.py:54-123)   one threshold table per
  map from the max over all surfaces (the merged adjacency's global dT),
  each surface scaled by its own max / 100
* low_ram_calculate_tfce      (tm_func.py:144-185)  one surface
* calculate_mediation_tfce    (tm_func.py:207-249)
* low_ram_calculate_mediation_tfce (tm_func.py:269-305)
* calc_mixed_tfce             (tm_func.py:327-378)  one threshold group and one
  (H, E) per TFCE setting, all settings in the same launch
* apply_mfwer                 (tm_func.py:403-491)  study-wide FWER
* create_full_mask, merge_adjacency_array, lowest_length,
  create_position_array, find_nearest (tm_func.py:502-573)

Permutation seeding follows the reference: ``perm_number + perm_seed`` when a
seed is given, the time-based seed otherwise.  The batched permutation loop
over many permutations per launch is ``randomise.mmr_run``.
"""
from __future__ import annotations

import math
import os
from time import time

import numpy as np

from .adjacency import AdjacencySet, concat_csr, induced_csr
from .adjacency import merge_adjacency_array  # noqa: F401
from .device import dev, ptr, require_cuda, stream_handle
from .fwer import apply_mfwer as _apply_mfwer_gpu
from .glm import WHAT_T, DesignBatch, glm_stat_f64
from .pyfunc import sobel_z_device


def _append(path, line):
    with open(path, "a") as fh:
        fh.write(line + "\n")


def _seed(perm_number, perm_seed=None):
    if perm_seed is not None:
        np.random.seed(perm_number + perm_seed)
    else:
        np.random.seed(perm_number + int(float(str(time())[-6:]) * 100))


_DATA = {}


def _data_dev(y):
    """The data on the device, kept between the calls of a permutation loop
    (the same array is passed to every call)."""
    y = np.asarray(y)
    key = (id(y), y.__array_interface__["data"][0], y.shape, y.dtype.str)
    if _DATA.get("key") != key:
        _DATA.clear()
        _DATA["dev"] = dev(np.ascontiguousarray(y, np.float32))
        _DATA["key"] = key
    return _DATA["dev"]


def _surface_lengths(masking_array):
    """Length of every surface in the merged (zero-filled) image: the whole
    surface for [V,1,1] masks, the in-mask voxels for volumes
    (create_full_mask, tm_func.py:502-510)."""
    return [int(np.asarray(m).shape[0]) if np.asarray(m).shape[2] == 1 else int(np.asarray(m).sum())
            for m in masking_array]


def _surface_parts(adjset, masking_array, fullmask):
    """Per-surface CSRs (local indices) of the masked vertices, cut from the
    merged adjacency of a CreateAdjSet; surfaces are disconnected in a merged
    adjacency, so each cut keeps every entry."""
    off, idx = adjset.csr
    full = np.asarray(fullmask) == 1
    lens = _surface_lengths(masking_array)
    if sum(lens) != full.shape[0] or off.shape[0] - 1 != full.shape[0]:
        raise ValueError(f"merged adjacency has {off.shape[0] - 1} vertices, the masks {sum(lens)}, "
                         f"fullmask {full.shape[0]}")
    parts, base = [], 0
    for n_s in lens:
        o = off[base:base + n_s + 1] - off[base]
        x = idx[off[base]:off[base + n_s]].astype(np.int64) - base
        parts.append(induced_csr((o, x), full[base:base + n_s]))
        base += n_s
    return parts


class _Study:
    """One device adjacency of a multisurface study: the surfaces as
    segments, per-segment H/E and threshold groups, reference arithmetic."""

    def __init__(self, parts, H, E, groups):
        off, idx, seg = concat_csr(parts)
        self.adj = AdjacencySet((off, idx), H, E, seg)
        self.adj.set_accumulation("exact")
        self.adj.set_threshold_groups(groups)
        self.seg = seg
        self.V = int(seg[-1])
        self.n_seg = seg.shape[0] - 1

    def sweep(self, maps, n_maps, signs, vdensity=1, floor_zero=False, want_maps=False):
        """Per-surface maxima (n_maps, signs, n_seg) and, with want_maps, the
        scaled maps (n_maps, signs, V), host float32."""
        t = require_cuda()
        vd = None
        if not (np.isscalar(vdensity) and float(vdensity) == 1.0):
            vd = dev(np.ascontiguousarray(np.broadcast_to(np.asarray(vdensity, np.float32), (self.V,))))
        out_max = t.empty((n_maps, signs, self.n_seg), device="cuda", dtype=t.float32)
        out_maps = t.empty((n_maps, signs, self.V), device="cuda", dtype=t.float32) if want_maps else None
        self.adj.sweep_batch(ptr(maps), self.V, n_maps, signs, ptr(vd), int(bool(floor_zero)), ptr(out_max),
                             ptr(out_maps), 1 if want_maps else 0, stream_handle())
        self.adj.status()
        return out_max.cpu().numpy(), (out_maps.cpu().numpy() if want_maps else None)


def _study_for(ops, groups_of_ops, masking_array, fullmask_of):
    """The _Study of a list of CreateAdjSets (one per threshold group),
    cached on the first operator."""
    masks = list(masking_array)
    key = (tuple(id(o) for o in ops), tuple(int(g) for g in groups_of_ops),
           tuple(_surface_lengths(masks)), tuple(int(np.asarray(m).sum()) for m in masks))
    cache = getattr(ops[0], "_tfgb_studies", None)
    if cache is None:
        cache = {}
        try:
            ops[0]._tfgb_studies = cache
        except AttributeError:
            pass
    if key in cache:
        return cache[key]
    groups_of_ops = np.asarray(groups_of_ops)
    parts = [None] * len(masks)
    H = np.zeros(len(masks), np.float32)
    E = np.zeros(len(masks), np.float32)
    grp = np.zeros(len(masks), np.int32)
    for gi, op in enumerate(ops):
        surf = np.flatnonzero(groups_of_ops == gi)
        sub = [masks[s] for s in surf]
        for s, part in zip(surf, _surface_parts(op.adjacency, sub, fullmask_of(sub))):
            parts[s] = part
            H[s], E[s], grp[s] = op.H, op.E, gi
    study = _Study(parts, H, E, grp)
    cache[key] = study
    return study


def _tmaps(merge_y, X, coefs):
    """t maps (1, C, V) float32 on the device, computed in FP64 with the
    reference's precision (tval_int) and cast to float32 as the reference
    casts them before sweeping (tm_func.py:64)."""
    return glm_stat_f64(_data_dev(merge_y), DesignBatch([X]), WHAT_T, coef=coefs).float().contiguous()


def _perm_design(X, perm_number, randomise, perm_seed=None, clock=True):
    if not randomise:
        return X
    if clock:
        np.random.seed(perm_number + int(float(str(time())[-6:]) * 100))
    else:
        _seed(perm_number, perm_seed)
    return X[np.random.permutation(list(range(X.shape[0])))]


def _write_surface_maxima(mx, labels, path_of):
    for tc in range(mx.shape[0]):
        for sc, label in enumerate(labels):
            _append(path_of(label, tc), "%f" % mx[tc, 0, sc])
            _append(path_of(label, tc), "%f" % mx[tc, 1, sc])


def calculate_tfce(merge_y, masking_array, pred_x, calcTFCE, vdensity, position_array, fullmask,
                   perm_number=None, randomise=False, verbose=False, no_intercept=True,
                   set_surf_count=None, print_interation=False):
    """tm_func.py:54-123: t of every contrast, each swept as + and - over all
    surfaces in one launch with the merged image's threshold table."""
    n = np.asarray(merge_y).shape[0]
    X = _perm_design(np.column_stack([np.ones(n), pred_x]), perm_number, randomise)
    k = X.shape[1]
    coefs = list(range(1 if no_intercept else 0, k))
    study = _study_for([calcTFCE], np.zeros(len(masking_array), np.int32), masking_array, create_full_mask)
    if np.asarray(position_array)[-1] != study.V:
        raise ValueError("position_array does not match the masks")
    tm = _tmaps(merge_y, X, coefs)
    C = len(coefs)
    mx, maps = study.sweep(tm, C, 2, vdensity, want_maps=not randomise)
    labels = ([int(np.ravel(set_surf_count[sc])[0]) for sc in range(len(masking_array))]
              if set_surf_count is not None else list(range(len(masking_array))))
    if randomise:
        _write_surface_maxima(mx, labels, lambda lab, tc: "perm_maxTFCE_surf%d_tcon%d.csv" % (lab, tc + 1))
        if print_interation:
            print("Interation number: %d" % perm_number)
        return None
    tvals = tm[0].cpu().numpy()
    for tc in range(C):
        for sc, label in enumerate(labels):
            print("Maximum (untransformed) postive tfce value for surface %s, tcon %d: %f" % (label, tc + 1, mx[tc, 0, sc]))
            print("Maximum (untransformed) negative tfce value for surface %s, tcon %d: %f" % (label, tc + 1, mx[tc, 1, sc]))
        if verbose:
            print("T-contrast: %d" % tc)
            print("Max tfce from all surfaces = %f" % maps[tc, 0].max())
            print("Max negative tfce from all surfaces = %f" % maps[tc, 1].max())
    return (np.ascontiguousarray(tvals, np.float32), np.ascontiguousarray(maps[:, 0], np.float32),
            np.ascontiguousarray(maps[:, 1], np.float32))


def low_ram_calculate_tfce(data, mask, pred_x, calcTFCE, vdensity, set_surf_count=0, perm_number=None,
                           randomise=False, no_intercept=True, output_dir=None, perm_seed=None):
    """tm_func.py:144-185: one surface; the scale is the max over the
    zero-filled surface (masked-out vertices count as 0)."""
    n = np.asarray(data).shape[0]
    X = _perm_design(np.column_stack([np.ones(n), pred_x]), perm_number, randomise, perm_seed, clock=False)
    k = X.shape[1]
    coefs = list(range(1 if no_intercept else 0, k))
    m = np.asarray(mask).ravel() == 1
    masks = [m[:, None, None]]
    study = _study_for([calcTFCE], [0], masks, lambda ms: np.asarray(ms[0])[:, 0, 0].astype(np.float64))
    tm = _tmaps(data, X, coefs)
    C = len(coefs)
    mx, maps = study.sweep(tm, C, 2, vdensity, floor_zero=not m.all(), want_maps=not randomise)
    if randomise:
        name = lambda lab, tc: "perm_maxTFCE_surf%d_tcon%d.csv" % (lab, tc + 1)  # noqa: E731
        path_of = (lambda lab, tc: os.path.join(output_dir, name(lab, tc))) if output_dir is not None else name
        _write_surface_maxima(mx, [int(set_surf_count)], path_of)
        return None
    return (np.ascontiguousarray(tm[0].cpu().numpy(), np.float32), np.ascontiguousarray(maps[:, 0], np.float32),
            np.ascontiguousarray(maps[:, 1], np.float32))


def _mediation_perm(medtype, pred_x, depend_y, n):
    idx = np.random.permutation(list(range(n)))
    if medtype in ("M", "I"):
        return pred_x[idx], depend_y
    return pred_x[idx], depend_y[idx]


def calculate_mediation_tfce(medtype, merge_y, masking_array, pred_x, depend_y, calcTFCE, vdensity,
                             position_array, fullmask, perm_number=None, randomise=False, verbose=False,
                             no_intercept=True, print_interation=False):
    """tm_func.py:207-249: the indirect-effect z map, swept (one sign) over all
    surfaces in one launch with the merged image's threshold table."""
    n = np.asarray(merge_y).shape[0]
    if randomise:
        np.random.seed(perm_number + int(float(str(time())[-6:]) * 100))
        pred_x, depend_y = _mediation_perm(medtype, pred_x, depend_y, n)
    study = _study_for([calcTFCE], np.zeros(len(masking_array), np.int32), masking_array, create_full_mask)
    z = sobel_z_device(medtype, pred_x, depend_y, _data_dev(merge_y), n)
    mx, maps = study.sweep(z, 1, 1, vdensity, want_maps=not randomise)
    for sc in range(len(masking_array)):
        if randomise:
            _append("perm_maxTFCE_surf%d_%s_zstat.csv" % (sc, medtype), "%f" % mx[0, 0, sc])
        else:
            print("Max Sobel Z tfce value for surface %s:\t %1.5f" % (sc, mx[0, 0, sc]))
    if verbose and maps is not None:
        print("Max Zstat tfce from all surfaces = %f" % maps[0, 0].max())
    if randomise:
        print("Interation number: %d" % perm_number)
        return None
    return (np.ascontiguousarray(z[0].cpu().numpy(), np.float32), np.ascontiguousarray(maps[0, 0], np.float32))


def low_ram_calculate_mediation_tfce(medtype, data, mask, pred_x, depend_y, calcTFCE, vdensity, set_surf_count=0,
                                     perm_number=None, randomise=False, no_intercept=True, output_dir=None,
                                     perm_seed=None):
    """tm_func.py:269-305."""
    n = np.asarray(data).shape[0]
    if randomise:
        _seed(perm_number, perm_seed)
        pred_x, depend_y = _mediation_perm(medtype, pred_x, depend_y, n)
    m = np.asarray(mask).ravel() == 1
    study = _study_for([calcTFCE], [0], [m[:, None, None]], lambda ms: np.asarray(ms[0])[:, 0, 0].astype(np.float64))
    z = sobel_z_device(medtype, pred_x, depend_y, _data_dev(data), n)
    mx, maps = study.sweep(z, 1, 1, vdensity, floor_zero=not m.all(), want_maps=not randomise)
    if randomise:
        name = "perm_maxTFCE_surf%d_%s_zstat.csv" % (set_surf_count, medtype)
        permfile = os.path.join(output_dir, name) if output_dir is not None else name
        _append(permfile, "%f" % mx[0, 0, 0])
        return None
    return np.ascontiguousarray(z[0].cpu().numpy(), np.float32), np.ascontiguousarray(maps[0, 0], np.float32)


def calc_mixed_tfce(assigntfcesettings, merge_y, masking_array, position_array, vdensity, pred_x, calcTFCE,
                    perm_number=None, randomise=False, medtype=None, depend_y=None):
    """tm_func.py:327-378: the surfaces of each TFCE setting i swept with
    calcTFCE[i]'s H and E and their own merged threshold table, every
    setting in one launch.  One permutation serves all settings (the
    reference re-seeds from the clock for each setting)."""
    assign = np.asarray(assigntfcesettings)
    settings = np.unique(assign)
    ops = [calcTFCE[int(i)] for i in settings]
    group_of = np.searchsorted(settings, assign)
    study = _study_for(ops, group_of, masking_array, create_full_mask)
    n = np.asarray(merge_y).shape[0]
    X = _perm_design(np.column_stack([np.ones(n), pred_x]), perm_number, randomise)
    coefs = list(range(1, X.shape[1]))
    if np.asarray(position_array)[-1] != study.V:
        raise ValueError("position_array does not match the masks")
    tm = _tmaps(merge_y, X, coefs)
    C = len(coefs)
    mx, maps = study.sweep(tm, C, 2, vdensity, want_maps=not randomise)
    if randomise:
        _write_surface_maxima(mx, list(range(len(assign))),
                              lambda lab, tc: "perm_maxTFCE_surf%d_tcon%d.csv" % (lab, tc + 1))
        print("Interation number: %d" % perm_number)
        return None
    # the reference binds tvals, tfce_tvals and neg_tfce_tvals to one array,
    # which ends up holding the negative maps
    out = np.asarray(maps[:, 1], np.float64)
    return out, out, out


def apply_mfwer(image_array, num_contrasts, surface_range, num_perm, num_surf, tminame, position_array, pos_range,
                neg_range=None, method="scale", weight=None, mediation=False, medtype=None):
    """tm_func.py:403-491: reads output_<tminame>/perm_maxTFCE_surf*_*.csv as
    the reference does; the per-vertex lookups run on the device."""
    perm = {}
    for contrast in range(num_contrasts):
        for surface in surface_range:
            if not mediation:
                f = "output_%s/perm_maxTFCE_surf%d_tcon%d.csv" % (tminame, surface, contrast + 1)
            else:
                f = "output_%s/perm_maxTFCE_surf%d_%s_zstat.csv" % (tminame, surface, str(medtype))
            perm[(surface, contrast)] = np.genfromtxt(f)[:num_perm]
    img = image_array[0]
    pos = img[:, [pos_range[c] for c in range(num_contrasts)]]
    neg = None if mediation else img[:, [neg_range[c] for c in range(num_contrasts)]]
    p, q = _apply_mfwer_gpu(pos, neg, perm, position_array, weight=weight, mediation=mediation)
    return p if mediation else (p, q)


def create_full_mask(masking_array):
    """tm_func.py:502-510."""
    fullmask = []
    for m in masking_array:
        if m.shape[2] == 1:
            fullmask = np.hstack((fullmask, m[:, 0, 0]))
        else:
            fullmask = np.hstack((fullmask, m[m == True]))  # noqa: E712
    return fullmask


def lowest_length(num_contrasts, surface_range, tmifilename, medtype=None):
    """tm_func.py:544-552."""
    lengths = []
    for contrast in range(num_contrasts):
        for surface in surface_range:
            if medtype is not None:
                f = "output_%s/perm_maxTFCE_surf%d_%s_zstat.csv" % (tmifilename, surface, medtype)
            else:
                f = "output_%s/perm_maxTFCE_surf%d_tcon%d.csv" % (tmifilename, surface, contrast + 1)
            lengths.append(np.array(np.genfromtxt(f).shape[0]))
    return np.array(lengths).min()


def create_position_array(masking_array):
    """tm_func.py:556-562."""
    pointer = 0
    position_array = [0]
    for m in masking_array:
        pointer += len(m[m == True])  # noqa: E712
        position_array.append(pointer)
    return position_array


def find_nearest(array, value, p_array):
    """tm_func.py:566-573."""
    idx = np.searchsorted(array, value, side="left")
    if idx == len(p_array):
        return p_array[idx - 1]
    elif math.fabs(value - array[idx - 1]) < math.fabs(value - array[idx]):
        return p_array[idx - 1]
    else:
        return p_array[idx]
