"""Observed-statistic outputs of the STEP_1 drivers, batched on the GPU:
the t (or sqrt F) images and their TFCE images with the reference's file
names, formats and max_TFCE_contrast_values.csv lines.

* vertex_observed_run -- the output half of
  tfce_mediation/tmanalysis/STEP_1_vertex_tfce_multiple_regression.py:353-403:
  from the python_temp_<surface>/ hand-off that script writes (merge_y, masks,
  affines, adjacency, TFCE settings, density weights), t of every contrast in
  one GLM launch, the + and - TFCE of every contrast and hemisphere in one
  sweep launch, then output_<surface>/{neg,}tstat_con<j>_<surface>_<lh|rh>{,_TFCE}.mgh
  in the reference's order (write_vertStat_img, pyfunc.py:80-92).
* voxel_observed_run -- STEP_1_voxel_tfce_multiple_regression.py:209-228:
  from python_temp/ (raw_nonzero_corr, pred_x, adjac, optstfce, ancova,
  data_mask, affine_mask), output/{neg,}tstat_con<j>{,_TFCE}.nii.gz, or
  fstat{,_TFCE}.nii.gz for the F-test (write_voxelStat_img, pyfunc.py:94-103).

The statistic maps use the FP64 GLM with the reference's precision
(glm_stat_f64) and the reference's sweep arithmetic (bit-identical sweeps of the same map).  Each
TFCE image is scaled by the max of its own statistic / 100 (and the vertex
density weights), as the reference's writers do.
"""
from __future__ import annotations

import os

import numpy as np

from .adjacency import AdjacencySet, to_csr
from .device import dev, ptr, require_cuda, stream_handle
from .glm import WHAT_T, DesignBatch, glm_fstat, glm_stat_f64
from .pyfunc import vert_stat_images, voxel_stat_images
from .randomise import _hemispheres, _load, _vd


def _sweep_maps(adj, maps_dev, n_maps, signs, vd=None):
    t = require_cuda()
    adj.set_accumulation("exact")
    out = t.empty((n_maps, signs, adj.n_vertices), device="cuda", dtype=t.float32)
    mx = t.empty((n_maps, signs, adj.n_seg), device="cuda", dtype=t.float32)
    adj.sweep_batch(ptr(maps_dev), adj.n_vertices, n_maps, signs, ptr(vd), 0, ptr(mx), ptr(out), 1,
                    stream_handle())
    adj.status()
    return out.cpu().numpy()


def vertex_observed_run(surface, outdir=None):
    """Write the observed images of a vertex-wise regression; returns the t
    maps (C, V_masked) and the scaled TFCE maps (C, 2, V_masked)."""
    d = "python_temp_%s" % surface
    merge_y = np.ascontiguousarray(_load(f"{d}/merge_y.npy"), np.float32)
    n = int(_load(f"{d}/num_subjects.npy"))
    pred_x = _load(f"{d}/pred_x.npy")
    mask_lh, mask_rh = _load(f"{d}/bin_mask_lh.npy"), _load(f"{d}/bin_mask_rh.npy")
    aff_lh, aff_rh = _load(f"{d}/affine_mask_lh.npy"), _load(f"{d}/affine_mask_rh.npy")
    adj_lh, adj_rh = _load(f"{d}/adjac_lh.npy"), _load(f"{d}/adjac_rh.npy")
    optstfce = _load(f"{d}/optstfce.npy")
    vd_lh, vd_rh = _load(f"{d}/vdensity_lh.npy"), _load(f"{d}/vdensity_rh.npy")
    off, idx, seg = _hemispheres(adj_lh, adj_rh, mask_lh, mask_rh)
    weighted = not (np.ndim(vd_lh) == 0 and float(vd_lh) == 1 and np.ndim(vd_rh) == 0 and float(vd_rh) == 1)
    vd = dev(np.concatenate([_vd(vd_lh, mask_lh), _vd(vd_rh, mask_rh)])) if weighted else None
    X = np.column_stack([np.ones(n), pred_x])
    k = X.shape[1]
    coefs = list(range(1, k))
    tm = glm_stat_f64(merge_y, DesignBatch([X]), WHAT_T, coef=coefs)[0].float().contiguous()  # (C, V)
    adj = AdjacencySet((off, idx), float(optstfce[0]), float(optstfce[1]), seg)
    maps = _sweep_maps(adj, tm, len(coefs), 2, vd)
    tv = tm.cpu().numpy().astype(np.float64)
    out = outdir or "output_%s" % surface
    os.makedirs(out, exist_ok=True)
    cwd = os.getcwd()
    os.chdir(out)
    try:
        hemis = (("lh", mask_lh, aff_lh), ("rh", mask_rh, aff_rh))
        outdata = {h: np.zeros((m.shape[0], 1, 1), np.float32) for h, m, _ in hemis}
        for j in range(len(coefs)):
            for si, (name, sgn) in enumerate((("tstat_con%d", 1.0), ("negtstat_con%d", -1.0))):
                for h, (hemi, mask, aff) in enumerate(hemis):
                    v0, v1 = seg[h], seg[h + 1]
                    full = np.zeros(mask.shape[0], np.float32)
                    full[np.asarray(mask, bool)] = maps[j, si, v0:v1]
                    vert_stat_images(name % (j + 1), tv[j, v0:v1] * sgn, full, outdata[hemi], aff, surface, hemi,
                                     np.asarray(mask, bool), mask.shape[0])
    finally:
        os.chdir(cwd)
    return tv, maps


def voxel_observed_run(temp="python_temp", outdir="output", imgext=".nii.gz"):
    """Write the observed images of a voxel-wise regression (or the F-test
    when the hand-off says ancova); returns the statistic maps and the scaled
    TFCE maps."""
    ny = np.ascontiguousarray(_load(f"{temp}/raw_nonzero_corr.npy").T, np.float32)
    pred_x = _load(f"{temp}/pred_x.npy")
    adjac = _load(f"{temp}/adjac.npy")
    optstfce = _load(f"{temp}/optstfce.npy")
    ancova = int(_load(f"{temp}/ancova.npy"))
    data_mask = np.asarray(_load(f"{temp}/data_mask.npy"))
    affine = _load(f"{temp}/affine_mask.npy")
    data_index = data_mask > 0.99
    out_path = data_mask.copy()
    n = ny.shape[0]
    X = np.column_stack([np.ones(n), pred_x])
    k = X.shape[1]
    adj = AdjacencySet(to_csr(adjac), float(optstfce[0]), float(optstfce[1]))
    os.makedirs(outdir, exist_ok=True)
    cwd = os.getcwd()
    if ancova == 1:
        t = require_cuda()
        F = glm_fstat(ny, DesignBatch([X]), centre=float(np.mean(ny)))[0]
        f = t.sqrt(t.clamp(F, min=0.0)).contiguous()
        maps = _sweep_maps(adj, f, 1, 1)
        fv = f.cpu().numpy().astype(np.float64)
        os.chdir(outdir)
        try:
            voxel_stat_images("fstat", fv, maps[0, 0], out_path, data_index, affine, imgext)
        finally:
            os.chdir(cwd)
        return fv[None], maps
    coefs = list(range(1, k))
    tm = glm_stat_f64(ny, DesignBatch([X]), WHAT_T, coef=coefs)[0].float().contiguous()
    tm[tm.isnan()] = 0.0
    maps = _sweep_maps(adj, tm, len(coefs), 2)
    tv = tm.cpu().numpy().astype(np.float64)
    os.chdir(outdir)
    try:
        for j in range(len(coefs)):
            voxel_stat_images("tstat_con%d" % (j + 1), tv[j], maps[j, 0], out_path, data_index, affine, imgext)
            voxel_stat_images("negtstat_con%d" % (j + 1), -tv[j], maps[j, 1], out_path, data_index, affine, imgext)
    finally:
        os.chdir(cwd)
    return tv, maps
