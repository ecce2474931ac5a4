"""Drop-in for the hot-path functions of ``tfce_mediation.pyfunc``.

Same names, arguments, outputs and file formats as tfce_mediation/pyfunc.py;
sweeps, regressions and indirect-effect maps run on the GPU:

* create_adjac_vertex / create_adjac_voxel       (pyfunc.py:37-76)
* write_vertStat_img / write_voxelStat_img       (pyfunc.py:80-103)
* write_perm_maxTFCE_vertex / _voxel             (pyfunc.py:107-126)
* calc_sobelz                                    (pyfunc.py:130-162)
* find_nearest                                   (pyfunc.py:254-261)
* calc_indirect, check_blocks, rand_blocks       (pyfunc.py:2678-2757)
* glm_typeI                                      (pyfunc.py:2282-2400)
* glm_cosinor (+ its design, cosinor_design)     (pyfunc.py:2406-2560)
* reg_rm_ancova_one_bs_factor / _two_bs_factor   (pyfunc.py:2067-2280, 1712-2060)
* dummy_code, column_product, stack_ones         (pyfunc.py:2564-2676)
"""
from __future__ import annotations

import math
import os

import numpy as np

from . import _lib
from .adjacency import create_adjac_vertex, create_adjac_voxel  # noqa: F401
from .device import dev, ptr, require_cuda, stream_handle
from .glm import WHAT_T, DesignBatch, glm_stat, glm_stat_f64
from .io import save_mgh, save_nifti
from .rm_anova import column_product, dummy_code, stack_ones  # noqa: F401  (pyfunc.py:2564-2676)

ALG = {"aroian": 0, "sobel": 1, "goodman": 2}


def _append(path, line):
    with open(path, "a") as fh:
        fh.write(line + "\n")


def _sweep_max_scaled(op, stat_full, density):
    """Max over one hemisphere of TFCE * (max/100) * density (pyfunc.py:116-117),
    computed by one device sweep."""
    t = require_cuda()
    adj = op.adjacency
    s = dev(np.ascontiguousarray(stat_full, np.float32))
    vd = None
    if not (np.isscalar(density) and float(density) == 1.0):
        vd = dev(np.ascontiguousarray(np.broadcast_to(np.asarray(density, np.float32), s.shape)))
    out = t.empty(1, device="cuda", dtype=t.float32)
    adj.sweep_batch(ptr(s), s.numel(), 1, 1, ptr(vd), 0, ptr(out))
    adj.status()
    return np.float32(out.item())


def write_perm_maxTFCE_vertex(statname, vertStat, num_vertex, bin_mask_lh, bin_mask_rh, calcTFCE_lh,
                              calcTFCE_rh, density_corr_lh=1, density_corr_rh=1):
    """Scatter into zero-filled hemispheres, sweep each, scale, append the max to
    perm_<statname>_TFCE_maxVertex.csv as %.4f (pyfunc.py:107-119)."""
    lh = np.zeros(bin_mask_lh.shape[0], np.float32)
    rh = np.zeros(bin_mask_rh.shape[0], np.float32)
    lh[bin_mask_lh] = vertStat[:num_vertex]
    rh[bin_mask_rh] = vertStat[num_vertex:]
    m = max(_sweep_max_scaled(calcTFCE_lh, lh, density_corr_lh),
            _sweep_max_scaled(calcTFCE_rh, rh, density_corr_rh))
    _append("perm_%s_TFCE_maxVertex.csv" % statname, "%.4f" % m)


def write_perm_maxTFCE_voxel(statname, voxelStat, TFCEfunc):
    """pyfunc.py:121-126: max(TFCE) * max(stat)/100, appended as %1.4f."""
    m = _sweep_max_scaled(TFCEfunc, np.asarray(voxelStat, np.float32), 1)
    _append("perm_%s_TFCE_maxVoxel.csv" % statname, "%1.4f" % m)


def _tfce_map(op, image):
    e = np.zeros(image.shape[0], np.float32)
    op.run(np.ascontiguousarray(image, np.float32), e)
    return e


def vert_stat_images(statname, vertStat, tfce_scaled, outdata_mask, affine_mask, surf, hemi, bin_mask,
                     all_vertex):
    """The file side of write_vertStat_img (pyfunc.py:80-92) for a TFCE image
    already scaled (full hemisphere, or None for TFCE=False): the TFCE image
    and its max line in max_TFCE_contrast_values.csv, then the statistic."""
    vertStat_out = np.zeros(all_vertex).astype(np.float32, order="C")
    vertStat_out[bin_mask] = vertStat
    if tfce_scaled is not None:
        outdata_mask[:, 0, 0] = tfce_scaled
        _append("max_TFCE_contrast_values.csv", "%s_%s_%s,%f" % (
            statname, surf, hemi, outdata_mask[np.isfinite(outdata_mask[:, 0, 0])].max()))
        save_mgh(outdata_mask, affine_mask, "%s_%s_%s_TFCE.mgh" % (statname, surf, hemi))
    outdata_mask[:, 0, 0] = vertStat_out
    save_mgh(outdata_mask, affine_mask, "%s_%s_%s.mgh" % (statname, surf, hemi))


def write_vertStat_img(statname, vertStat, outdata_mask, affine_mask, surf, hemi, bin_mask, TFCEfunc,
                       all_vertex, density_corr=1, TFCE=True):
    """pyfunc.py:80-92: TFCE image scaled by max(masked stat)/100 * density,
    max appended to max_TFCE_contrast_values.csv, both images saved as MGH."""
    scaled = None
    if TFCE:
        vertStat_out = np.zeros(all_vertex).astype(np.float32, order="C")
        vertStat_out[bin_mask] = vertStat
        vertStat_TFCE = _tfce_map(TFCEfunc, vertStat_out)
        scaled = vertStat_TFCE * (vertStat[np.isfinite(vertStat)].max() / 100) * density_corr
    vert_stat_images(statname, vertStat, scaled, outdata_mask, affine_mask, surf, hemi, bin_mask, all_vertex)


def voxel_stat_images(statname, voxelStat, tfce_scaled, out_path, data_index, affine, imgext=".nii.gz"):
    """The file side of write_voxelStat_img (pyfunc.py:94-103) for a TFCE map
    already scaled (over the mask's voxels, or None for TFCE=False)."""
    if tfce_scaled is not None:
        out_path[data_index] = tfce_scaled
        save_nifti(out_path, affine, "%s_TFCE%s" % (statname, imgext))
        _append("max_TFCE_contrast_values.csv", "%s,%f" % (statname, out_path.max()))
    out_path[data_index] = voxelStat
    save_nifti(out_path, affine, "%s%s" % (statname, imgext))


def write_voxelStat_img(statname, voxelStat, out_path, data_index, affine, TFCEfunc, imgext=".nii.gz",
                        TFCE=True):
    """pyfunc.py:94-103."""
    scaled = None
    if TFCE:
        voxelStat_out = voxelStat.astype(np.float32, order="C")
        voxelStat_TFCE = _tfce_map(TFCEfunc, voxelStat_out)
        scaled = voxelStat_TFCE * (voxelStat_out.max() / 100)
    voxel_stat_images(statname, voxelStat, scaled, out_path, data_index, affine, imgext)


# ---------------------------------------------------------------------------
# mediation
# ---------------------------------------------------------------------------
def mediation_designs(medtype, pred_x, depend_y, n, covariates=None):
    """Path-a and path-b designs of calc_sobelz (pyfunc.py:131-145); the tested
    coefficient is column 1 of each.  For medtype 'Y' path a is a scalar
    regression of depend_y on pred_x (scipy linregress), returned as ta.
    covariates: appended to both designs, as the tm-models mediation branch
    passes dmy_covariates to glm_typeI (tm_models_randomise.py:430-503); path a
    of 'Y' is then the FP64 OLS t of pred_x in [1, pred_x, covariates]."""
    x = np.asarray(pred_x, np.float64).reshape(n, -1)
    dy = np.asarray(depend_y, np.float64).reshape(n, -1)
    one = np.ones((n, 1))
    cov = [] if covariates is None else [np.asarray(covariates, np.float64).reshape(n, -1)]
    if medtype == "I":
        return np.hstack([one, x] + cov), np.hstack([one, x, dy] + cov), None
    if medtype == "M":
        return np.hstack([one, x] + cov), np.hstack([one, dy, x] + cov), None
    if medtype == "Y":
        if covariates is None:
            from scipy.stats import linregress
            lr = linregress(np.asarray(pred_x, np.float64).ravel(), np.asarray(depend_y, np.float64).ravel())
            return None, np.hstack([one, dy, x]), lr.slope / lr.stderr
        Xa = np.hstack([one, x] + cov)
        inv = np.linalg.inv(Xa.T @ Xa)
        y = dy[:, 0]
        a = inv @ Xa.T @ y
        sigma2 = np.sum((y - Xa @ a) ** 2) / (n - Xa.shape[1])
        return None, np.hstack([one, dy, x] + cov), a[1] / np.sqrt(sigma2 * inv[1, 1])
    raise ValueError("Invalid mediation type")


def sobel_from_t(ta, tb, alg="aroian", ta_scalar=None):
    """Indirect-effect z of path t maps (device tensors (P, V)) -> (P, V)."""
    t = require_cuda()
    P, V = tb.shape
    z = t.empty((P, V), device="cuda", dtype=t.float32)
    tas = None if ta_scalar is None else dev(np.asarray(ta_scalar, np.float32).reshape(P))
    _lib.check(_lib.load().sobel_combine(ptr(ta), V, ptr(tas), ptr(tb), V, P, V, ALG[alg], ptr(z), V,
                                         stream_handle()))
    return z


def sobel_z_device(medtype, pred_x, depend_y, Y, n, alg="aroian", precision="fp64", covariates=None):
    """Indirect-effect z of the data Y (n, V) as a device tensor (1, V): the
    path-a and path-b t maps in one GLM launch (FP64 with the reference's
    precision by default, or 'fp32'), then sobel_combine."""
    if alg not in ALG:
        raise ValueError("Unknown indirect test algorithm")
    Xa, Xb, ta_scalar = mediation_designs(medtype, pred_x, depend_y, n, covariates=covariates)

    def tmap(designs):
        if precision == "fp64":
            return glm_stat_f64(Y, DesignBatch(designs), WHAT_T, coef=[1])[:, 0].float().contiguous()
        return glm_stat(Y, DesignBatch(designs), WHAT_T, coef=[1])[:, 0]
    if ta_scalar is None:
        tab = tmap([Xa, Xb])
        return sobel_from_t(tab[0:1], tab[1:2], alg)
    tb = tmap([Xb])
    return sobel_from_t(None, tb, alg, ta_scalar=[ta_scalar])


def calc_sobelz(medtype, pred_x, depend_y, merge_y, n, num_vertex, alg="aroian"):
    """Sobel/Aroian/Goodman z per vertex (pyfunc.py:130-162), float64 host array."""
    if alg not in ALG:
        raise ValueError("Unknown indirect test algorithm")
    z = sobel_z_device(medtype, pred_x, depend_y, np.asarray(merge_y, np.float32), n, alg)
    return z[0].cpu().numpy().astype(np.float64)


def calc_indirect(ta, tb, alg="aroian"):
    """pyfunc.py:2678-2709 on the device."""
    if alg not in ALG:
        raise ValueError("Unknown indirect test algorithm")
    t = require_cuda()
    ta_d = dev(np.atleast_2d(np.asarray(ta, np.float32)), t.float32)
    tb_d = dev(np.atleast_2d(np.asarray(tb, np.float32)), t.float32)
    z = sobel_from_t(ta_d, tb_d, alg)
    out = z.cpu().numpy().astype(np.float64)
    return out[0] if np.ndim(ta) == 1 else out


# ---------------------------------------------------------------------------
# host helpers (no device work in the reference either)
# ---------------------------------------------------------------------------
def find_nearest(array, value, p_array):
    """pyfunc.py:254-261."""
    idx = np.searchsorted(array, value, side="left")
    if idx == len(p_array):
        return p_array[idx - 1]
    elif math.fabs(value - array[idx - 1]) < math.fabs(value - array[idx]):
        return p_array[idx - 1]
    else:
        return p_array[idx]


def check_blocks(block_list):
    """pyfunc.py:2711-2731."""
    unique_blocks = np.unique(block_list)
    sizes = [len(block_list[block_list == b]) for b in unique_blocks]
    eq = all(x == sizes[0] for x in sizes)
    if not eq:
        print("Warning: blocks are not equal. Swaping with only occur within blocks, but not among blocks.")
    return eq


def rand_blocks(block_list, is_equal_sizes):
    """pyfunc.py:2733-2757 (draws from the global legacy numpy RNG, as the reference)."""
    indexer = np.array(range(len(block_list)))
    randindex = []
    blocks = np.random.permutation(list(np.unique(block_list))) if is_equal_sizes is True \
        else np.unique(block_list)
    for block in blocks:
        randindex.append(np.random.permutation(indexer[block_list == block]))
    return np.concatenate(randindex)


def _typeI_design(n, exog, dmy_covariates):
    """[1, exog variables..., covariates] and the column widths of the exog
    variables (pyfunc.py:2305-2317)."""
    kvars, cols = [], [np.ones((n, 1))]
    for var in exog:
        var = np.asarray(var, np.float64)
        kvars.append(1 if var.ndim == 1 else var.shape[1])
        cols.append(var.reshape(n, -1))
    if dmy_covariates is not None:
        cols.append(np.asarray(dmy_covariates, np.float64).reshape(n, -1))
    return np.column_stack(cols), kvars


def glm_typeI(endog, exog, dmy_covariates=None, output_fvalues=True, output_tvalues=False, output_pvalues=False,
              verbose=True, rand_array=None, use_reduced_residuals=False, output_reduced_residuals=False,
              exog_names=None):
    """Generalised ANCOVA of the tm-models path, pyfunc.py:2282-2400, on the GPU.

    endog (n, V) or (n,); exog: list of (n,) / (n, k_i) dummy-coded variables;
    the design is [1, exog..., dmy_covariates], rows permuted by rand_array.
    Returns the reference's tuples: F (model), the drop-one F of every exog
    variable, t of every coefficient, P values (scipy, as the reference),
    reduced residuals.  Model F and t run on the FP32 CUDA-core GLM (TSS around
    each column's mean); the drop-one F runs on the tensor-core GLM in its
    exact Wald form (glm_stat_tc mode 2: no difference of residual sums)."""
    from .glm import WHAT_RESID, glm_fstat, glm_stat_tc
    y = np.asarray(endog)
    one = y.ndim == 1
    Y = np.ascontiguousarray(y.reshape(y.shape[0], -1), np.float32)
    n = Y.shape[0]
    X, kvars = _typeI_design(n, exog, dmy_covariates)
    if rand_array is not None:
        if use_reduced_residuals:
            Y = glm_stat(Y, DesignBatch([X]), WHAT_RESID)[0].cpu().numpy()
        X = X[np.asarray(rand_array)]
    reduced_data = None
    if output_reduced_residuals:
        reduced_data = glm_stat(Y, DesignBatch([X]), WHAT_RESID)[0].cpu().numpy()
    k = X.shape[1]
    df_between, df_within, df_total = k - 1, n - k, n - 1
    db = DesignBatch([X])

    Fvalues = Fvar = Tvalues = None
    Pvar = []
    if output_fvalues:
        Fvalues = glm_fstat(Y, db)[0].cpu().numpy()
        if verbose:
            print("Source\t\tDF\tF(Max)")
            print("Model\t\t(%d,%d)\t%.2f" % (df_between, df_within, Fvalues.max()))
        groups, start = [], 1
        for kv in kvars:
            groups.append((start, kv))
            start += kv
        Fvar = glm_stat_tc(Y, db, "f", groups=groups)[0].cpu().numpy()
        for i, col in enumerate(kvars):
            if verbose:
                name = exog_names[i] if exog_names is not None else "Exog%d" % (i + 1)
                print("%s\t\t(%d,%d)\t%.2f" % (name, col, df_within, Fvar[i].max()))
    if output_tvalues:
        Tvalues = glm_stat(Y, db, WHAT_T)[0].cpu().numpy()
    if one:
        Fvalues = None if Fvalues is None else Fvalues[0]
        Fvar = None if Fvar is None else Fvar[:, 0]
        Tvalues = None if Tvalues is None else Tvalues[:, 0]
    if output_fvalues and output_pvalues:
        from scipy.stats import f as fdist
        Pvar = [fdist.sf(Fvar[i], col, df_within) for i, col in enumerate(kvars)]
    if output_tvalues and output_fvalues:
        if output_pvalues:
            from scipy.stats import f as fdist
            from scipy.stats import t as tdist
            return (Fvalues, np.array(Fvar), Tvalues, fdist.sf(Fvalues, df_between, df_within), np.array(Pvar),
                    tdist.sf(np.abs(Tvalues), df_total) * 2)
        if output_reduced_residuals:
            return (Fvalues, np.array(Fvar), Tvalues, reduced_data)
        return (Fvalues, np.array(Fvar), Tvalues)
    if output_tvalues:
        if output_pvalues:
            from scipy.stats import t as tdist
            return (Tvalues, tdist.sf(np.abs(Tvalues), df_total) * 2)
        if output_reduced_residuals:
            return (Tvalues, reduced_data)
        return Tvalues
    if output_fvalues:
        if output_pvalues:
            from scipy.stats import f as fdist
            return (Fvalues, np.array(Fvar), fdist.sf(Fvalues, df_between, df_within), np.array(Pvar))
        if output_reduced_residuals:
            return (Fvalues, np.array(Fvar), reduced_data)
        return (Fvalues, np.array(Fvar))
    print("No output has been selected")
    return None


def cosinor_design(time_var, period, exog=None, dmy_covariates=None):
    """The cosinor design [1, cos(2 pi t / p), sin(2 pi t / p) per period,
    exog..., covariates] (pyfunc.py:2428-2457), float64."""
    t = np.asarray(time_var, np.float64)
    n = t.shape[0]
    cols = [np.ones((n, 1))]
    for p in period:
        cols.append(np.cos(np.divide(2.0 * np.pi * t, p)).reshape(n, 1))
        cols.append(np.sin(np.divide(2.0 * np.pi * t, p)).reshape(n, 1))
    for var in exog or []:
        cols.append(np.asarray(var, np.float64).reshape(n, -1))
    if dmy_covariates is not None:
        cols.append(np.asarray(dmy_covariates, np.float64).reshape(n, -1))
    return np.column_stack(cols)


def _acrophase(b_cos, b_sin, quadrant):
    """arctan(|b_sin / b_cos|), with the reference's sign/quadrant rule when
    `quadrant` (pyfunc.py:2475-2490)."""
    with np.errstate(divide="ignore", invalid="ignore"):
        acro = np.arctan(np.abs(np.divide(-b_sin, b_cos)))
    if quadrant:
        acro = acro.copy()
        m = (b_sin > 0) & (b_cos >= 0)
        acro[m] = -acro[m]
        m = (b_sin > 0) & (b_cos < 0)
        acro[m] = -np.pi + acro[m]
        m = (b_sin < 0) & (b_cos <= 0)
        acro[m] = -np.pi - acro[m]
        m = (b_sin <= 0) & (b_cos > 0)
        acro[m] = -2.0 * np.pi + acro[m]
    return acro


def glm_cosinor(endog, time_var, exog=None, dmy_covariates=None, rand_array=None, interaction_var=None,
                period=[24.0], calc_MESOR=True, output_fit_only=False):
    """Cosinor GLM of the tm-models path, pyfunc.py:2406-2560, on the GPU.

    Design [1, (cos, sin) per period, exog..., dmy_covariates], rows permuted
    by rand_array.  Returns the reference's tuple (R2, MESOR, SE_MESOR,
    AMPLITUDE, SE_AMPLITUDE, ACROPHASE, SE_ACROPHASE, Fmodel, tMESOR,
    |tAMPLITUDE|, |tACROPHASE|, tEXOG), or (MESOR, AMPLITUDE, ACROPHASE) with
    output_fit_only.  Betas, RSS, t and the model F (TSS around each column's
    mean) come from the FP32 CUDA-core GLM; the amplitude/acrophase error
    propagation is the reference's elementwise FP64 arithmetic on those.  The
    permutation loop does not call this: its maps come from the tensor-core
    GLM's programmed epilogue (randomise.tm_models_cosinor_run).
    interaction_var: the reference multiplies a design ROW by it
    (exog_vars[i+1] * interaction_var), which only broadcasts for degenerate
    sizes; it is refused here."""
    from .glm import WHAT_BETA, WHAT_RSS, glm_fstat
    if interaction_var is not None:
        raise ValueError("interaction_var is not supported (the reference's interaction term indexes a design row)")
    y = np.asarray(endog)
    one = y.ndim == 1
    Y = np.ascontiguousarray(y.reshape(y.shape[0], -1), np.float32)
    n = Y.shape[0]
    n_per = len(period)
    X = cosinor_design(time_var, period, exog, dmy_covariates)
    if rand_array is not None:
        X = X[np.asarray(rand_array)]
    k = X.shape[1]
    db = DesignBatch([X])
    a = glm_stat(Y, db, WHAT_BETA)[0].cpu().numpy().astype(np.float64)  # (k, V)

    def out(v):
        return v[..., 0] if one else v

    if output_fit_only:
        amp = np.asarray([np.sqrt(a[1 + 2 * i] ** 2 + a[2 + 2 * i] ** 2) for i in range(n_per)])
        acro = np.asarray([_acrophase(a[1 + 2 * i], a[2 + 2 * i], True) for i in range(n_per)])
        return out(a[0]), out(amp), out(acro)
    rss = glm_stat(Y, db, WHAT_RSS)[0].cpu().numpy().astype(np.float64)
    F = glm_fstat(Y, db)[0].cpu().numpy().astype(np.float64)
    df_between, df_within = k - 1, n - k
    sigma = np.sqrt(rss / df_within)
    invXX = db.inverse()[0]
    MESOR = tMESOR = SE_MESOR = tEXOG = None
    if calc_MESOR or exog is not None:
        if one:
            se = np.sqrt(sigma[None, :] ** 2 * np.diag(invXX)[:, None])
        else:
            se = np.sqrt((rss / df_within)[None, :] * np.diag(invXX)[:, None]).astype(np.float32)
        T = a / se
        MESOR, tMESOR, SE_MESOR = out(a[0]), out(T[0]), out(se[0])
        if exog is not None:
            tEXOG = out(T[3 + 2 * (n_per - 1):])
    amp, acro, se_amp, se_acro, t_amp, t_acro = [], [], [], [], [], []
    for i in range(n_per):
        c, s = 1 + 2 * i, 2 + 2 * i
        A = np.sqrt(a[c] ** 2 + a[s] ** 2)
        ph = _acrophase(a[c], a[s], False)
        sn, cs = np.sin(ph), np.cos(ph)
        with np.errstate(divide="ignore", invalid="ignore"):
            sp = sigma * np.sqrt(invXX[c, c] * sn ** 2 + 2 * invXX[c, s] * sn * cs + invXX[s, s] * cs ** 2) / A
            sa = sigma * np.sqrt(invXX[c, c] * cs ** 2 - 2 * invXX[c, s] * sn * cs + invXX[s, s] * sn ** 2)
            t_amp.append(np.abs(A / sa))
            t_acro.append(np.abs(1.0 / sp))
        amp.append(A)
        acro.append(_acrophase(a[c], a[s], True) if rand_array is None else ph)
        se_amp.append(sa)
        se_acro.append(sp)
    R2 = None
    if rand_array is None:
        ssb = F * rss * df_between / df_within
        R2 = out(ssb / (ssb + rss))
    arr = [out(np.asarray(v)) for v in (amp, se_amp, acro, se_acro, t_amp, t_acro)]
    return (R2, MESOR, SE_MESOR, arr[0], arr[1], arr[2], arr[3], out(F), tMESOR, arr[4], arr[5], tEXOG)


# -- tm-models repeated-measures ANCOVA ----------------------------------------


def _rm_anova(data, factors, dmy_subjects, dmy_covariates, data_format, output_sig, verbose, rand_array,
              use_reduced_residuals, output_reduced_residuals, labels):
    """Shared body of the two reg_rm_ancova_* drop-ins (see there)."""
    from .glm import WHAT_RESID
    from .rm_anova import RMAncovaEngine, RMModel, long_data
    endog, n, s = long_data(data, data_format, len(factors[0]))
    squeeze = endog.shape[1] == 1
    N = n * s
    facs = [np.asarray(f) for f in factors]
    cov = None if dmy_covariates is None else np.asarray(dmy_covariates)

    def long_exog(fs, cv):
        cols = [np.tile(np.asarray(f, np.float64).reshape(n, -1), (s, 1)) for f in fs]
        if len(fs) == 2:
            cols.append(np.tile(column_product(fs[0], fs[1]).reshape(n, -1), (s, 1)))
        if cv is not None:
            cols.append(np.tile(np.asarray(cv, np.float64).reshape(n, -1), (s, 1)))
        return stack_ones(np.column_stack(cols))

    if rand_array is not None:
        if use_reduced_residuals:
            X = long_exog(facs, cov)
            endog = glm_stat(np.ascontiguousarray(endog, np.float32), DesignBatch([X]), WHAT_RESID)[0].cpu().numpy()
        # the reference shuffles the long rows in place: the caller's array
        # when the long form is a view of it
        np.random.shuffle(endog)
        facs = [f[rand_array] for f in facs]
        cov = None if cov is None else cov[rand_array]
    model = RMModel(n, s, facs[0], dmy_subjects, dmy_factor2=facs[1] if len(facs) == 2 else None,
                    dmy_covariates=cov)
    eng = RMAncovaEngine(np.ascontiguousarray(endog, np.float32), model)
    F = eng.fmaps([None], np.arange(N)[None])[0].cpu().numpy().astype(np.float64)
    eng.status()
    if verbose:
        print("Source\t\tDF\tF(Max)")
        for (nm, df, err), lab, Fi in zip(model.f_maps, labels, F):
            tab = "\t" if len(lab) >= 8 else "\t\t"
            print("%s%s(%d,%d)\t%.2f" % (lab, tab, df, model.df_w if err else model.df_b, Fi.max()))
    Fs = [Fi[0] if squeeze else Fi for Fi in F]
    if output_sig:
        from scipy.stats import f as fdist
        Ps = [1 - fdist.cdf(Fi, df, model.df_w if err else model.df_b) for Fi, (_, df, err) in zip(Fs, model.f_maps)]
        return tuple(Fs) + tuple(Ps)
    if output_reduced_residuals:
        X = long_exog(facs if len(facs) == 2 else facs[:1], cov)
        reduced = glm_stat(np.ascontiguousarray(endog, np.float32), DesignBatch([X]), WHAT_RESID)[0].cpu().numpy()
        return tuple(Fs) + (reduced,)
    return tuple(Fs)


def reg_rm_ancova_one_bs_factor(data, dmy_factor1, dmy_subjects, data_format="short", dmy_covariates=None,
                                output_sig=False, verbose=True, rand_array=None, use_reduced_residuals=False,
                                output_reduced_residuals=False):
    """One between-subject factor repeated-measures ANCOVA, pyfunc.py:2067-2280,
    on the GPU: (F_a, F_s, F_sa) [+ (P_a, P_s, P_sa) with output_sig, or the
    reduced residuals].  data: (s intervals, n subjects[, V]) ('short') or
    (n*s[, V]) ('long', interval-major rows).  Effect sums of squares in exact
    Wald form on the tensor-core GLM, subject split and F on the device
    (tfce_mediation_gb300.rm_anova).  With rand_array the long data rows are
    shuffled in place with np.random.shuffle (the caller's array when the long
    form is a view of it) and the factor / covariate rows permuted, as the
    reference does.  'long' data is accepted with an integer interval count
    (the reference's own long path divides with / and fails on Python 3)."""
    return _rm_anova(data, [dmy_factor1], dmy_subjects, dmy_covariates, data_format, output_sig, verbose,
                     rand_array, use_reduced_residuals, output_reduced_residuals,
                     ["Factor", "Time", "Factor*Time"])


def reg_rm_ancova_two_bs_factor(data, dmy_factor1, dmy_factor2, dmy_subjects, dmy_covariates=None,
                                data_format="short", output_sig=False, verbose=True, rand_array=None,
                                use_reduced_residuals=False, output_reduced_residuals=False):
    """Two between-subject factor repeated-measures ANCOVA (type I sums of
    squares), pyfunc.py:1712-2060, on the GPU: (F_a, F_b, F_ab, F_s, F_sa, F_sb,
    F_sab) [+ P values or the reduced residuals]; see
    reg_rm_ancova_one_bs_factor."""
    return _rm_anova(data, [dmy_factor1, dmy_factor2], dmy_subjects, dmy_covariates, data_format, output_sig,
                     verbose, rand_array, use_reduced_residuals, output_reduced_residuals,
                     ["Factor1", "Factor2", "F1*F2", "Time", "F1*Time", "F2*Time", "F1*F2*Time"])
