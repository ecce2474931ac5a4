"""Drop-in for the multimodal multisurface (mmr) bodies of ``tfce_mediation.tm_func``.

Same names, arguments, outputs and CSV files as tfce_mediation/tm_func.py;
regressions, indirect-effect maps and TFCE sweeps run on the GPU:

* calculate_tfce              (tm_func.py:54-123)   one sweep over the merged
  adjacency of all surfaces (global dT), each surface scaled by its own max
* low_ram_calculate_tfce      (tm_func.py:144-185)  one surface
* calculate_mediation_tfce    (tm_func.py:207-249)
* low_ram_calculate_mediation_tfce (tm_func.py:269-305)
* calc_mixed_tfce             (tm_func.py:327-378)  per-group H/E settings
* apply_mfwer                 (tm_func.py:403-491)  study-wide FWER
* create_full_mask, merge_adjacency_array, lowest_length,
  create_position_array, find_nearest (tm_func.py:502-573)

Permutation seeding follows the reference: ``perm_number + perm_seed`` when a
seed is given, the time-based seed otherwise.
"""
from __future__ import annotations

import math
import os
from time import time

import numpy as np

from . import cynumstats
from .adjacency import merge_adjacency_array  # noqa: F401
from .fwer import apply_mfwer as _apply_mfwer_gpu
from .pyfunc import calc_sobelz


def _append(path, line):
    with open(path, "a") as fh:
        fh.write(line + "\n")


def _seed(perm_number, perm_seed=None):
    if perm_seed is not None:
        np.random.seed(perm_number + perm_seed)
    else:
        np.random.seed(perm_number + int(float(str(time())[-6:]) * 100))


def _tvals(X, y):
    k = X.shape[1]
    invXX = np.linalg.inv(np.dot(X.T, X))
    return cynumstats.tval_int(X, invXX, y, y.shape[0], k, y.shape[1])


def _sweep(calcTFCE, img):
    out = np.zeros_like(img)
    calcTFCE.run(np.ascontiguousarray(img, np.float32), out)
    return out


def calculate_tfce(merge_y, masking_array, pred_x, calcTFCE, vdensity, position_array, fullmask,
                   perm_number=None, randomise=False, verbose=False, no_intercept=True,
                   set_surf_count=None, print_interation=False):
    """tm_func.py:54-123."""
    X = np.column_stack([np.ones(merge_y.shape[0]), pred_x])
    if randomise:
        np.random.seed(perm_number + int(float(str(time())[-6:]) * 100))
        X = X[np.random.permutation(list(range(merge_y.shape[0])))]
    tvals = _tvals(X, merge_y)
    if no_intercept:
        tvals = tvals[1:, :]
    tvals = tvals.astype(np.float32, order="C")
    tfce_tvals = np.zeros_like(tvals).astype(np.float32, order="C")
    neg_tfce_tvals = np.zeros_like(tvals).astype(np.float32, order="C")
    for tc in range(tvals.shape[0]):
        tval_temp = np.zeros_like(fullmask).astype(np.float32, order="C")
        tval_temp[fullmask == 1] = tvals[0] if tvals.shape[0] == 1 else tvals[tc]
        tfce_temp = _sweep(calcTFCE, tval_temp)
        neg_tfce_temp = _sweep(calcTFCE, tval_temp * -1)
        tval_temp = tval_temp[fullmask == 1]
        tfce_temp = tfce_temp[fullmask == 1]
        neg_tfce_temp = neg_tfce_temp[fullmask == 1]
        for sc in range(len(masking_array)):
            start, end = position_array[sc], position_array[sc + 1]
            vd = vdensity if isinstance(vdensity, int) else vdensity[start:end]
            tfce_tvals[tc, start:end] = tfce_temp[start:end] * (tval_temp[start:end].max() / 100) * vd
            neg_tfce_tvals[tc, start:end] = (neg_tfce_temp[start:end] * ((tval_temp * -1)[start:end].max() / 100)
                                             * vd)
            label = int(set_surf_count[sc]) if set_surf_count is not None else sc
            if randomise:
                _append("perm_maxTFCE_surf%d_tcon%d.csv" % (label, tc + 1),
                        "%f" % np.nanmax(tfce_tvals[tc, start:end]))
                _append("perm_maxTFCE_surf%d_tcon%d.csv" % (label, tc + 1),
                        "%f" % np.nanmax(neg_tfce_tvals[tc, start:end]))
            else:
                print("Maximum (untransformed) postive tfce value for surface %s, tcon %d: %f"
                      % (label, tc + 1, np.nanmax(tfce_tvals[tc, start:end])))
                print("Maximum (untransformed) negative tfce value for surface %s, tcon %d: %f"
                      % (label, tc + 1, np.nanmax(neg_tfce_tvals[tc, start:end])))
        if verbose:
            print("T-contrast: %d" % tc)
            print("Max tfce from all surfaces = %f" % tfce_tvals[tc].max())
            print("Max negative tfce from all surfaces = %f" % neg_tfce_tvals[tc].max())
    if randomise:
        if print_interation:
            print("Interation number: %d" % perm_number)
        return None
    return (tvals.astype(np.float32, order="C"), tfce_tvals.astype(np.float32, order="C"),
            neg_tfce_tvals.astype(np.float32, order="C"))


def low_ram_calculate_tfce(data, mask, pred_x, calcTFCE, vdensity, set_surf_count=0, perm_number=None,
                           randomise=False, no_intercept=True, output_dir=None, perm_seed=None):
    """tm_func.py:144-185."""
    X = np.column_stack([np.ones(data.shape[0]), pred_x])
    if randomise:
        _seed(perm_number, perm_seed)
        X = X[np.random.permutation(list(range(data.shape[0])))]
    tvals = _tvals(X, data)
    if no_intercept:
        tvals = tvals[1:, :]
    tvals = tvals.astype(np.float32, order="C")
    tfce_tvals = np.zeros_like(tvals).astype(np.float32, order="C")
    neg_tfce_tvals = np.zeros_like(tvals).astype(np.float32, order="C")
    for tc in range(tvals.shape[0]):
        tval_temp = np.zeros_like(mask).astype(np.float32, order="C")
        tval_temp[mask == 1] = tvals[0] if tvals.shape[0] == 1 else tvals[tc]
        tfce_temp = _sweep(calcTFCE, tval_temp)
        neg_tfce_temp = _sweep(calcTFCE, -tval_temp)
        tfce_tvals[tc, :] = tfce_temp[mask == 1] * (tval_temp.max() / 100) * vdensity
        neg_tfce_tvals[tc, :] = neg_tfce_temp[mask == 1] * ((tval_temp * -1).max() / 100) * vdensity
        if randomise:
            name = "perm_maxTFCE_surf%d_tcon%d.csv" % (int(set_surf_count), tc + 1)
            permfile = os.path.join(output_dir, name) if output_dir is not None else name
            _append(permfile, "%f" % np.nanmax(tfce_tvals[tc, :]))
            _append(permfile, "%f" % np.nanmax(neg_tfce_tvals[tc, :]))
    if not randomise:
        return (tvals.astype(np.float32, order="C"), tfce_tvals.astype(np.float32, order="C"),
                neg_tfce_tvals.astype(np.float32, order="C"))


def _mediation_perm(medtype, pred_x, depend_y, n):
    idx = np.random.permutation(list(range(n)))
    if medtype in ("M", "I"):
        return pred_x[idx], depend_y
    return pred_x[idx], depend_y[idx]


def calculate_mediation_tfce(medtype, merge_y, masking_array, pred_x, depend_y, calcTFCE, vdensity,
                             position_array, fullmask, perm_number=None, randomise=False, verbose=False,
                             no_intercept=True, print_interation=False):
    """tm_func.py:207-249."""
    if randomise:
        np.random.seed(perm_number + int(float(str(time())[-6:]) * 100))
        pred_x, depend_y = _mediation_perm(medtype, pred_x, depend_y, merge_y.shape[0])
    SobelZ = calc_sobelz(medtype, pred_x, depend_y, merge_y, merge_y.shape[0], merge_y.shape[1])
    SobelZ = SobelZ.astype(np.float32, order="C")
    tfce_SobelZ = np.zeros_like(SobelZ).astype(np.float32, order="C")
    zval_temp = np.zeros_like(fullmask).astype(np.float32, order="C")
    zval_temp[fullmask == 1] = SobelZ
    tfce_temp = _sweep(calcTFCE, zval_temp)
    zval_temp = zval_temp[fullmask == 1]
    tfce_temp = tfce_temp[fullmask == 1]
    for sc in range(len(masking_array)):
        start, end = position_array[sc], position_array[sc + 1]
        vd = vdensity if isinstance(vdensity, int) else vdensity[start:end]
        tfce_SobelZ[start:end] = tfce_temp[start:end] * (zval_temp[start:end].max() / 100) * vd
        if randomise:
            _append("perm_maxTFCE_surf%d_%s_zstat.csv" % (sc, medtype), "%f" % np.nanmax(tfce_SobelZ[start:end]))
        else:
            print("Max Sobel Z tfce value for surface %s:\t %1.5f" % (sc, np.nanmax(tfce_SobelZ[start:end])))
    if verbose:
        print("Max Zstat tfce from all surfaces = %f" % tfce_SobelZ.max())
    if randomise:
        print("Interation number: %d" % perm_number)
        return None
    return SobelZ.astype(np.float32, order="C"), tfce_SobelZ.astype(np.float32, order="C")


def low_ram_calculate_mediation_tfce(medtype, data, mask, pred_x, depend_y, calcTFCE, vdensity, set_surf_count=0,
                                     perm_number=None, randomise=False, no_intercept=True, output_dir=None,
                                     perm_seed=None):
    """tm_func.py:269-305."""
    if randomise:
        _seed(perm_number, perm_seed)
        pred_x, depend_y = _mediation_perm(medtype, pred_x, depend_y, data.shape[0])
    SobelZ = calc_sobelz(medtype, pred_x, depend_y, data, data.shape[0], data.shape[1])
    SobelZ = SobelZ.astype(np.float32, order="C")
    zval = np.zeros_like(mask).astype(np.float32, order="C")
    zval[mask == 1] = SobelZ
    tfce_zval = _sweep(calcTFCE, zval)
    zval = zval[mask == 1]
    tfce_zval = tfce_zval[mask == 1]
    tfce_zval = tfce_zval * (zval.max() / 100) * vdensity
    if randomise:
        name = "perm_maxTFCE_surf%d_%s_zstat.csv" % (set_surf_count, medtype)
        permfile = os.path.join(output_dir, name) if output_dir is not None else name
        _append(permfile, "%f" % np.nanmax(tfce_zval))
    else:
        return zval.astype(np.float32, order="C"), tfce_zval.astype(np.float32, order="C")


def calc_mixed_tfce(assigntfcesettings, merge_y, masking_array, position_array, vdensity, pred_x, calcTFCE,
                    perm_number=None, randomise=False, medtype=None, depend_y=None):
    """tm_func.py:327-378: surfaces grouped by TFCE setting, each group swept
    with its own operator."""
    tvals = tfce_tvals = neg_tfce_tvals = None
    for i in np.unique(assigntfcesettings):
        data_mask = np.zeros(merge_y.shape[1], dtype=bool)
        extract_range = np.argwhere(assigntfcesettings == i)
        for surface in extract_range:
            data_mask[position_array[int(surface)]:position_array[int(surface) + 1]] = True
        sub = merge_y[:, data_mask]
        try:
            temp_vdensity = vdensity[data_mask]
        except Exception:
            temp_vdensity = 1
        group = np.array(masking_array)[assigntfcesettings == i]
        if randomise:
            calculate_tfce(sub, group, pred_x, calcTFCE[i], temp_vdensity, create_position_array(group),
                           create_full_mask(group), set_surf_count=extract_range, perm_number=perm_number,
                           randomise=True, print_interation=(i == 0))
        else:
            tv, tp, tn = calculate_tfce(sub, group, pred_x, calcTFCE[i], temp_vdensity,
                                        create_position_array(group), create_full_mask(group),
                                        set_surf_count=extract_range)
            if tvals is None:
                # the reference binds the three names to one array here
                tvals = tfce_tvals = neg_tfce_tvals = np.zeros((tv.shape[0], merge_y.shape[1]))
            tvals[:, data_mask] = tv
            tfce_tvals[:, data_mask] = tp
            neg_tfce_tvals[:, data_mask] = tn
    if not randomise:
        return tvals, tfce_tvals, neg_tfce_tvals


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
