"""ORACLE -- test infrastructure, not product code.

CPU restatement of the reference's permutation-inference path.  Each function
cites the reference lines it follows.  Only ``tests/``, ``__graft_entry__``'s
smoke check and ``bench.py``'s CPU-baseline leg may import this module.

Pinning: ``tests/test_oracle_pin.py`` checks every function here against
golden vectors produced by the reference itself (``tests/golden/``, made by
``tests/golden/make_golden.py`` from the reference's compiled Cython modules
and unmodified ``pyfunc``/``tm_func``), and -- where ``oracle/_ref`` was built
from a reference checkout -- against the reference sweep directly.
"""
from __future__ import annotations

import ctypes
import ctypes.util
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(HERE, "_build")
_LIB = None
_REF = None

_f32p = ctypes.POINTER(ctypes.c_float)
_i32p = ctypes.POINTER(ctypes.c_int32)
_i64p = ctypes.POINTER(ctypes.c_int64)


# --------------------------------------------------------------------------
# native pieces
# --------------------------------------------------------------------------
def build() -> str:
    """Compile the C restatement of the sweep (gcc, -O2, no -march flags so the
    same recipe works on x86_64 and aarch64)."""
    os.makedirs(_BUILD, exist_ok=True)
    so = os.path.join(_BUILD, "libtfce_oracle.so")
    srcs = [os.path.join(HERE, "tfce_oracle.c"), os.path.join(HERE, "geodesic_oracle.c")]
    if not (os.path.exists(so) and all(os.path.getmtime(so) >= os.path.getmtime(x) for x in srcs)):
        tmp = so + f".{os.getpid()}.tmp"
        subprocess.check_call(["gcc", "-O2", "-std=c11", "-shared", "-fPIC"] + srcs + ["-o", tmp, "-lm"])
        os.replace(tmp, so)
    return so


def lib():
    global _LIB
    if _LIB is None:
        l = ctypes.CDLL(build())
        l.oracle_tfce.restype = ctypes.c_int
        l.oracle_tfce.argtypes = [ctypes.c_float, ctypes.c_float, ctypes.c_int32, _i64p, _i32p,
                                  _f32p, _f32p, _i32p, _i32p, ctypes.c_int]
        l.oracle_tfce_mode.restype = ctypes.c_int
        l.oracle_tfce_mode.argtypes = [ctypes.c_float, ctypes.c_float, ctypes.c_int32, _i64p, _i32p,
                                       _f32p, _f32p, _i32p, _i32p, ctypes.c_int, ctypes.c_int]
        l.oracle_tfce_max_batch.restype = ctypes.c_int
        l.oracle_tfce_max_batch.argtypes = [ctypes.c_float, ctypes.c_float, ctypes.c_int32, _i64p,
                                            _i32p, _f32p, ctypes.c_int32, ctypes.c_float, _f32p,
                                            ctypes.c_int, _f32p, ctypes.c_int]
        l.oracle_threshold_table.restype = ctypes.c_int
        l.oracle_threshold_table.argtypes = [ctypes.c_float, _f32p, ctypes.c_int]
        l.oracle_geodesic_lists.restype = ctypes.c_int
        l.oracle_geodesic_lists.argtypes = _GEO_ARGS
        _LIB = l
    return _LIB


_GEO_ARGS = [ctypes.c_int32, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_double, ctypes.c_int32,
             ctypes.c_int32, ctypes.c_int32, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
             ctypes.c_void_p]
_REF_GEO = None


def _geo_call(fn, v, f, threshold, only_greater, src_lo, src_hi, cap):
    v = np.ascontiguousarray(v, np.float32)
    f = np.ascontiguousarray(f, np.int32)
    src_hi = v.shape[0] if src_hi is None else int(src_hi)
    if cap is None:
        cap = 4096 + 256 * (src_hi - int(src_lo))
    while True:
        oi = np.empty(cap, np.int32)
        oj = np.empty(cap, np.int32)
        od = np.empty(cap, np.float64)
        n = ctypes.c_int64()
        rc = fn(v.shape[0], v.ctypes.data, f.shape[0], f.ctypes.data, float(threshold), int(bool(only_greater)),
                int(src_lo), src_hi, cap, oi.ctypes.data, oj.ctypes.data, od.ctypes.data, ctypes.byref(n))
        if rc == -4:
            cap *= 4
            continue
        if rc:
            raise ValueError(f"geodesic lists failed ({rc})")
        k = n.value
        return oi[:k].copy(), oj[:k].copy(), od[:k].copy()


def geodesic_lists(v, f, threshold, only_greater=True, src_lo=0, src_hi=None, cap=None):
    """Exact geodesic (i, j, d) for sources i in [src_lo, src_hi) and vertices
    j != i with d < threshold (j > i when only_greater), sorted by i then j:
    the pairs tfce_mediation/adjacency.pyx:83-106 lists, by the window
    propagation restated in oracle/geodesic_oracle.c."""
    return _geo_call(lib().oracle_geodesic_lists, v, f, threshold, only_greater, src_lo, src_hi, cap)


def ref_geodesic_lib():
    """The reference's exact geodesic library behind oracle/ref_geodesic_shim.cpp
    (oracle/_ref/libref_geodesic.so), when it was built from a reference
    checkout on this machine; otherwise None."""
    global _REF_GEO
    if _REF_GEO is None:
        so = os.path.join(HERE, "_ref", "libref_geodesic.so")
        if not os.path.exists(so):
            return None
        try:
            l = ctypes.CDLL(so)
        except OSError:
            return None
        l.ref_geodesic_lists.restype = ctypes.c_int
        l.ref_geodesic_lists.argtypes = _GEO_ARGS
        _REF_GEO = l
    return _REF_GEO


def ref_geodesic_lists(v, f, threshold, only_greater=True, src_lo=0, src_hi=None, cap=None):
    """The same lists from the reference's own library (None when it is not built)."""
    l = ref_geodesic_lib()
    if l is None:
        return None
    return _geo_call(l.ref_geodesic_lists, v, f, threshold, only_greater, src_lo, src_hi, cap)


def ref_lib():
    """The reference sweep itself (oracle/_ref/libref_tfce.so), when it was
    built from a reference checkout on this machine; otherwise None."""
    global _REF
    if _REF is None:
        so = os.path.join(HERE, "_ref", "libref_tfce.so")
        if not os.path.exists(so):
            return None
        try:
            l = ctypes.CDLL(so)
        except OSError:  # built for another architecture
            return None
        l.ref_tfce.restype = ctypes.c_int
        l.ref_tfce.argtypes = [ctypes.c_float, ctypes.c_float, ctypes.c_int32, _i64p, _i32p,
                               _f32p, _f32p]
        _REF = l
    return _REF


def _p(a, t):
    return a.ctypes.data_as(t)


def _csr(offsets, indices):
    return (np.ascontiguousarray(offsets, dtype=np.int64),
            np.ascontiguousarray(indices, dtype=np.int32))


def threshold_table(maxT: float) -> np.ndarray:
    """T = maxT, maxT - dT, ... >= 0 with dT = maxT/100, all in float32
    (tfce_mediation/lib/fast_tfce.hpp:32-39)."""
    buf = np.zeros(4096, np.float32)
    n = lib().oracle_threshold_table(ctypes.c_float(maxT), _p(buf, _f32p), 4096)
    if n < 0:
        raise ValueError("threshold table overflow")
    return buf[:n].copy()


def tfce(offsets, indices, image, H, E, enhn=None, hh_exact=False):
    """One sweep: tfce_mediation/lib/fast_tfce.hpp:11-95 as called by
    tfce_mediation/tfce.pyx:44-45.  Accumulates into ``enhn``.

    hh_exact=False uses powf(T, H) for the threshold weight as the reference
    does; hh_exact=True uses the correctly rounded power (the device's
    arithmetic), for bit-for-bit checks of the kernel."""
    offsets, indices = _csr(offsets, indices)
    image = np.ascontiguousarray(image, dtype=np.float32)
    V = image.shape[0]
    if enhn is None:
        enhn = np.zeros(V, np.float32)
    rc = lib().oracle_tfce_mode(H, E, V, _p(offsets, _i64p), _p(indices, _i32p), _p(image, _f32p),
                                _p(enhn, _f32p), None, None, -1, int(bool(hh_exact)))
    if rc < 0:
        raise ValueError("oracle sweep failed")
    return enhn


def tfce_labels(offsets, indices, image, H, E, hh_exact=False):
    """Sweep plus per-threshold component labels (root vertex id, -1 inactive)
    and extents; (enhn, labels[L,V], extents[L,V])."""
    offsets, indices = _csr(offsets, indices)
    image = np.ascontiguousarray(image, dtype=np.float32)
    V = image.shape[0]
    finite = image[np.isfinite(image)]
    L = len(threshold_table(float(finite.max()))) if finite.size else 0
    enhn = np.zeros(V, np.float32)
    labels = np.full((max(L, 1), V), -1, np.int32)
    extents = np.zeros((max(L, 1), V), np.int32)
    rc = lib().oracle_tfce_mode(H, E, V, _p(offsets, _i64p), _p(indices, _i32p), _p(image, _f32p),
                                _p(enhn, _f32p), _p(labels, _i32p), _p(extents, _i32p), -1,
                                int(bool(hh_exact)))
    if rc < 0:
        raise ValueError("oracle sweep failed")
    return enhn, labels[:rc], extents[:rc]


def ref_tfce(offsets, indices, image, H, E, enhn=None):
    """The reference's own sweep (needs oracle/_ref)."""
    l = ref_lib()
    if l is None:
        raise RuntimeError("reference sweep not built (oracle/build_ref.py)")
    offsets, indices = _csr(offsets, indices)
    image = np.ascontiguousarray(image, dtype=np.float32)
    if enhn is None:
        enhn = np.zeros(image.shape[0], np.float32)
    l.ref_tfce(H, E, image.shape[0], _p(offsets, _i64p), _p(indices, _i32p), _p(image, _f32p),
               _p(enhn, _f32p))
    return enhn


def tfce_max_batch(offsets, indices, maps, H, E, sign=1.0, vdensity=None, floor_zero=False,
                   hh_exact=False):
    """Per-map scaled max, the body of tfce_mediation/pyfunc.py:107-119 for one
    hemisphere (TFCE * max/100 * vdensity, then max)."""
    offsets, indices = _csr(offsets, indices)
    maps = np.ascontiguousarray(maps, dtype=np.float32)
    if maps.ndim == 1:
        maps = maps[None]
    out = np.zeros(maps.shape[0], np.float32)
    vd = None if vdensity is None else np.ascontiguousarray(vdensity, np.float32)
    rc = lib().oracle_tfce_max_batch(H, E, maps.shape[1], _p(offsets, _i64p), _p(indices, _i32p),
                                     _p(maps, _f32p), maps.shape[0], sign,
                                     None if vd is None else _p(vd, _f32p), int(floor_zero),
                                     _p(out, _f32p), int(bool(hh_exact)))
    if rc < 0:
        raise ValueError("oracle sweep failed")
    return out


# --------------------------------------------------------------------------
# GLM: tfce_mediation/cynumstats.pyx
# --------------------------------------------------------------------------
def lstsqr_mat(X, y):
    """cy_lin_lstsqr_mat: inv(X'X) X' y in FP64 (cynumstats.pyx:28-29)."""
    X = np.asarray(X, np.float64)
    return (np.linalg.inv(X.T.dot(X)).dot(X.T)).dot(y)


def tval_int_ref(X, invXX, y, n, k):
    """tval_int with the reference's precision (cynumstats.pyx:59-64): FP64
    betas and sigma^2, SE rounded to float32 (se_of_slope, :47-52), t = FP64
    beta / float32 SE."""
    a = lstsqr_mat(X, y)
    sigma2 = np.sum((y - np.dot(X, a)) ** 2, axis=0) / (n - k)
    se = np.sqrt(sigma2[None, :] * np.diag(invXX)[:, None]).astype(np.float32)
    return a / se


def tval_fp64(X, y):
    """t for every column of X, all in FP64 (the accuracy yardstick)."""
    X = np.asarray(X, np.float64)
    y = np.asarray(y, np.float64)
    n, k = X.shape
    invXX = np.linalg.inv(X.T @ X)
    a = invXX @ (X.T @ y)
    r = y - X @ a
    sigma2 = np.sum(r * r, axis=0) / (n - k)
    return a / np.sqrt(sigma2[None, :] * np.diag(invXX)[:, None])


def glm_typeI(endog, exog, dmy_covariates=None, rand_array=None):
    """glm_typeI with output_fvalues and output_tvalues (tm/pyfunc.py:2282-2400):
    design [1, exog..., covariates] (rows permuted by rand_array), model F
    ((SS_Total - RSS)/(k-1)) / (RSS/(n-k)) with SS_Total around each column's
    mean (formed in the data's own type, float32 for the reference's data),
    the drop-one F of every exogenous variable from the refit without its
    columns, and t of every coefficient with the SE rounded to float32
    (se_of_slope).  Returns (F_model, F_var (n_var, V), T (k, V))."""
    y = np.asarray(endog, np.float64)
    n = y.shape[0]
    kvars, cols = [], [np.ones(n)]
    for var in exog:
        var = np.asarray(var, np.float64)
        kvars.append(1 if var.ndim == 1 else var.shape[1])
        cols.append(var.reshape(n, -1))
    if dmy_covariates is not None:
        cols.append(np.asarray(dmy_covariates, np.float64).reshape(n, -1))
    X = np.column_stack(cols)
    if rand_array is not None:
        X = X[np.asarray(rand_array)]
    k = X.shape[1]

    def rss(Xm):
        a = np.linalg.lstsq(Xm, y, rcond=None)[0]
        r = y - Xm @ a
        return a, np.sum(r * r, axis=0)

    # SS_Total in the data's own type, as numpy forms it for float32 data
    y_in = np.asarray(endog)
    ss_total = np.sum((y_in - np.mean(y_in, 0)) ** 2, 0).astype(np.float64)
    a, rss_full = rss(X)
    ms_res = rss_full / (n - k)
    F_model = ((ss_total - rss_full) / (k - 1)) / ms_res
    F_var, start = [], 1
    for kv in kvars:
        _, rss_red = rss(np.delete(X, np.s_[start:start + kv], 1))
        F_var.append((rss_red - rss_full) / (ms_res * kv))
        start += kv
    invXX = np.linalg.inv(X.T @ X)
    se = np.sqrt((rss_full / (n - k))[None, :] * np.diag(invXX)[:, None]).astype(np.float32)
    return F_model, np.asarray(F_var), a / se


def partial_f_fp64(X, y, groups):
    """Drop-one F of column groups [(start, width), ...] of design X, FP64,
    from the refits without each group (the yardstick of glm_stat_tc mode 2)."""
    X = np.asarray(X, np.float64)
    y = np.asarray(y, np.float64)
    n, k = X.shape

    def rss(Xm):
        a = np.linalg.lstsq(Xm, y, rcond=None)[0]
        r = y - Xm @ a
        return np.sum(r * r, axis=0)

    full = rss(X)
    return np.asarray([(rss(np.delete(X, np.s_[s0:s0 + w], 1)) - full) / w / (full / (n - k))
                       for s0, w in groups])


def cosinor_design(time_var, period, exog=None, dmy_covariates=None):
    """[1, cos(2 pi t / p_i), sin(2 pi t / p_i) per period, exog..., covariates]
    (tm/pyfunc.py:2428-2457)."""
    t = np.asarray(time_var, np.float64)
    n = t.shape[0]
    cols = [np.ones(n)]
    for p in period:
        cols.append(np.cos(np.divide(2.0 * np.pi * t, p)))
        cols.append(np.sin(np.divide(2.0 * np.pi * t, p)))
    for var in exog or []:
        cols.append(np.asarray(var, np.float64).reshape(n, -1))
    if dmy_covariates is not None:
        cols.append(np.asarray(dmy_covariates, np.float64).reshape(n, -1))
    return np.column_stack(cols)


def _acrophase_quadrant(acro, b_cos, b_sin):
    """The sign/quadrant rule of tm/pyfunc.py:2487-2490 (and 2545-2548)."""
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


def glm_cosinor(endog, time_var, exog=None, dmy_covariates=None, rand_array=None, period=(24.0,),
                calc_MESOR=True, output_fit_only=False):
    """glm_cosinor (tm/pyfunc.py:2406-2560), FP64, for 2-D endog (n, V):
    design rows permuted by rand_array; betas and RSS of the full fit
    (cy_lin_lstsqr_mat_residual); SS_Total in the data's own type; model F =
    ((SS_Total - RSS)/(k-1)) / (RSS/(n-k)); SE of the coefficients rounded to
    float32 (se_of_slope); per period the amplitude sqrt(b_cos^2 + b_sin^2),
    the acrophase arctan(|b_sin / b_cos|) with the error-propagation SEs taken
    before the quadrant rule, which only the unpermuted call applies; t of the
    amplitude A/SE_A and of the acrophase 1/SE_phi, returned as absolute values.
    Returns the reference's 12-tuple (3-tuple with output_fit_only)."""
    y_in = np.asarray(endog)
    y = np.asarray(endog, np.float64)
    n = y.shape[0]
    n_per = len(period)
    X = cosinor_design(time_var, period, exog, dmy_covariates)
    if rand_array is not None:
        X = X[np.asarray(rand_array)]
    k = X.shape[1]
    df_between, df_within = k - 1, n - k
    invXX = np.linalg.inv(X.T @ X)
    a = invXX @ X.T @ y
    r = y - X @ a
    rss = np.sum(r ** 2, axis=0)
    amp, acro = [], []
    for i in range(n_per):
        bc, bs = a[1 + 2 * i], a[2 + 2 * i]
        amp.append(np.sqrt(bc ** 2 + bs ** 2))
        with np.errstate(divide="ignore", invalid="ignore"):
            acro.append(np.arctan(np.abs(np.divide(-bs, bc))))
    if output_fit_only:
        acro_q = [_acrophase_quadrant(acro[i], a[1 + 2 * i], a[2 + 2 * i]) for i in range(n_per)]
        return a[0], np.asarray(amp), np.asarray(acro_q)
    ss_total = np.sum((y_in - np.mean(y_in, 0)) ** 2, 0).astype(np.float64)
    ms_res = rss / df_within
    F_model = ((ss_total - rss) / df_between) / ms_res
    sigma = np.sqrt(ms_res)
    MESOR = tMESOR = SE_MESOR = tEXOG = None
    if calc_MESOR or exog is not None:
        se = np.sqrt(ms_res[None, :] * np.diag(invXX)[:, None]).astype(np.float32)
        T = a / se
        MESOR, tMESOR, SE_MESOR = a[0], T[0], se[0]
        if exog is not None:
            tEXOG = T[3 + 2 * (n_per - 1):]
    se_amp, se_acro, t_amp, t_acro = [], [], [], []
    for i in range(n_per):
        c, s = 1 + 2 * i, 2 + 2 * i
        sn, cs = np.sin(acro[i]), np.cos(acro[i])
        with np.errstate(divide="ignore", invalid="ignore"):
            se_acro.append(sigma * np.sqrt(invXX[c, c] * sn ** 2 + 2 * invXX[c, s] * sn * cs
                                           + invXX[s, s] * cs ** 2) / amp[i])
            se_amp.append(sigma * np.sqrt(invXX[c, c] * cs ** 2 - 2 * invXX[c, s] * sn * cs
                                          + invXX[s, s] * sn ** 2))
            t_amp.append(amp[i] / se_amp[i])
            t_acro.append(1.0 / se_acro[i])
        if rand_array is None:
            acro[i] = _acrophase_quadrant(acro[i], a[c], a[s])
    R2 = 1 - rss / ss_total if rand_array is None else None
    return (R2, MESOR, SE_MESOR, np.asarray(amp), np.asarray(se_amp), np.asarray(acro), np.asarray(se_acro),
            F_model, tMESOR, np.abs(np.asarray(t_amp)), np.abs(np.asarray(t_acro)),
            None if tEXOG is None else np.asarray(tEXOG))


def calc_beta_se(x, y, n):
    """cynumstats.pyx:66-74: design [1, x]; returns (beta[1], se float32 k x V)."""
    X = np.column_stack([np.ones(n), x])
    invXX = np.linalg.inv(np.dot(X.T, X))
    k = X.shape[1]
    a = lstsqr_mat(X, y)
    sigma2 = np.sum((y - np.dot(X, a)) ** 2, axis=0) / (n - k)
    se = np.sqrt(sigma2[None, :] * np.diag(invXX)[:, None]).astype(np.float32)
    return a[1], se


def resid_covars(x_covars, data):
    """cynumstats.pyx:54-57 (data is V x n, returns n x V residuals)."""
    a_c = lstsqr_mat(x_covars, data.T)
    return data.T - np.dot(x_covars, a_c)


def calcF(X, y, n, k):
    """cynumstats.pyx:31-36.  TSS is taken around np.mean(y) -- the grand mean
    of the whole matrix, not each column's mean -- as the reference does."""
    a = lstsqr_mat(X, y)
    resids = y - np.dot(X, a)
    RSS = np.sum(resids ** 2, axis=0)
    TSS = np.sum((y - np.mean(y)) ** 2, axis=0)
    return ((TSS - RSS) / (k - 1)) / (RSS / (n - k))


def indirect(ta, tb, alg="aroian"):
    """Sobel/Aroian/Goodman z from path t values (pyfunc.py:146-161,
    pyfunc.py:2678-2709)."""
    ta = np.asarray(ta, np.float64)
    tb = np.asarray(tb, np.float64)
    if alg == "aroian":
        return 1 / np.sqrt((1 / (tb ** 2)) + (1 / (ta ** 2)) + (1 / (ta ** 2 * tb ** 2)))
    if alg == "sobel":
        return 1 / np.sqrt((1 / (tb ** 2)) + (1 / (ta ** 2)))
    if alg == "goodman":
        return 1 / np.sqrt((1 / (tb ** 2)) + (1 / (ta ** 2)) - (1 / (ta ** 2 * tb ** 2)))
    raise ValueError(alg)


def calc_sobelz(medtype, pred_x, depend_y, merge_y, n, alg="aroian"):
    """pyfunc.py:130-162 (medtype 'I', 'M' or 'Y')."""
    from scipy.stats import linregress
    if medtype == "I":
        a_b, a_se = calc_beta_se(pred_x, merge_y, n)
        b_b, b_se = calc_beta_se(np.column_stack([pred_x, depend_y]), merge_y, n)
        a_se, b_se = a_se[1], b_se[1]
    elif medtype == "M":
        a_b, a_se = calc_beta_se(pred_x, merge_y, n)
        b_b, b_se = calc_beta_se(np.column_stack([depend_y, pred_x]), merge_y, n)
        a_se, b_se = a_se[1], b_se[1]
    elif medtype == "Y":
        lr = linregress(pred_x, depend_y)
        a_b, a_se = lr.slope, lr.stderr
        b_b, b_se = calc_beta_se(np.column_stack([depend_y, pred_x]), merge_y, n)
        b_se = b_se[1]
    else:
        raise ValueError(medtype)
    return indirect(a_b / a_se, b_b / b_se, alg)


# --------------------------------------------------------------------------
# permutations, per-permutation max, FWER
# --------------------------------------------------------------------------
def permutation(n, seed, p):
    """Host-seeded index stream, the mmr-lr convention
    (tm_func.py:147-151): RandomState(seed + p).permutation(n)."""
    return np.random.RandomState(seed + p).permutation(n)


def perm_max_vertex(stat, segments, H, E, vdensity=None):
    """pyfunc.py:107-119 without the CSV: scatter, TFCE each segment
    (hemisphere), scale by the segment's max/100 and vdensity, max over
    segments.  segments: list of (offsets, indices, v0, v1)."""
    best = -np.inf
    for (off, idx, v0, v1) in segments:
        img = np.ascontiguousarray(stat[v0:v1], np.float32)
        enh = tfce(off, idx, img, H, E)
        scale = img[np.isfinite(img)].max() / np.float32(100)
        val = enh * scale
        if vdensity is not None:
            val = val * vdensity[v0:v1]
        best = max(best, float(val.max()))
    return np.float32(best)


def merge_adjacency(adjacency_array):
    """tm_func.merge_adjacency_array (tm_func.py:521-540) for the common call,
    adjacent_range = range(len(adjacency_array)): the surfaces' lists
    concatenated, each offset by the vertex count before it.  Returns a CSR."""
    offs, idxs, base = [np.zeros(1, np.int64)], [], 0
    e = 0
    for adj in adjacency_array:
        lens = np.array([len(list(a)) for a in adj], np.int64)
        offs.append(np.cumsum(lens) + e)
        e += int(lens.sum())
        idxs.append(np.concatenate([np.asarray(list(a), np.int64) for a in adj]) + base if len(adj) else
                    np.zeros(0, np.int64))
        base += len(adj)
    return np.concatenate(offs), np.concatenate(idxs).astype(np.int32)


def _full_mask(masking_array):
    """tm_func.create_full_mask (tm_func.py:502-510): surfaces ([V,1,1]
    masks) contribute their whole mask, volumes their in-mask voxels."""
    parts = []
    for m in masking_array:
        m = np.asarray(m)
        parts.append(m[:, 0, 0].astype(np.float64) if m.shape[2] == 1 else np.ones(int(m.sum())))
    return np.concatenate(parts)


def _positions(masking_array):
    """tm_func.create_position_array (tm_func.py:556-562)."""
    pos = [0]
    for m in masking_array:
        pos.append(pos[-1] + int(np.asarray(m).sum()))
    return pos


def _scaled(enh, tv, pos, vdensity):
    out = np.zeros_like(enh)
    for s in range(len(pos) - 1):
        a, b = pos[s], pos[s + 1]
        vd = vdensity if np.isscalar(vdensity) else np.asarray(vdensity)[a:b]
        out[a:b] = enh[a:b] * (tv[a:b].max() / 100) * vd
    return out


def calculate_tfce(merge_y, masking_array, pred_x, adjacency_array, H, E, vdensity=1, perm=None):
    """tm_func.calculate_tfce (tm_func.py:54-123), observed form: t of every
    non-intercept column (tval_int precision), each contrast scattered into the
    zero-filled merged image of all surfaces and swept once over the merged
    adjacency (one threshold table: dT = the merged image's max / 100, Q6),
    then every surface scaled by its own max / 100 and vdensity.
    perm: row permutation of the design (the randomised call's X[perm]).
    Returns (tvals, tfce_tvals, neg_tfce_tvals) float32 [C][V_masked]."""
    merge_y = np.asarray(merge_y)
    n = merge_y.shape[0]
    X = np.column_stack([np.ones(n), pred_x])
    if perm is not None:
        X = X[perm]
    k = X.shape[1]
    tv = tval_int_ref(X, np.linalg.inv(X.T @ X), merge_y, n, k)[1:].astype(np.float32)
    off, idx = merge_adjacency(adjacency_array)
    full = _full_mask(masking_array) == 1
    pos = _positions(masking_array)
    tp, tn = np.zeros_like(tv), np.zeros_like(tv)
    for c in range(tv.shape[0]):
        img = np.zeros(full.shape[0], np.float32)
        img[full] = tv[c]
        ep = tfce(off, idx, img, H, E)[full]
        en = tfce(off, idx, img * -1, H, E)[full]
        tp[c] = _scaled(ep, img[full], pos, vdensity)
        tn[c] = _scaled(en, (img * -1)[full], pos, vdensity)
    return tv, tp, tn


def surface_maxima(tfce_maps, position_array):
    """np.nanmax of a scaled map over each surface: the value the randomised
    call appends to perm_maxTFCE_surf<s>_* (tm_func.py:93-97)."""
    return np.array([np.nanmax(tfce_maps[..., a:b], axis=-1)
                     for a, b in zip(position_array[:-1], position_array[1:])]).T


def calc_mixed_tfce(assign, merge_y, masking_array, adjacency_array, settings, pred_x, vdensity=1, perm=None):
    """tm_func.calc_mixed_tfce (tm_func.py:327-378), observed form: the
    surfaces of each TFCE setting i (assign == i) are one calculate_tfce over
    their own merged adjacency with settings[i] = (H, E).  Returns the
    per-group (tvals, tfce, neg_tfce) placed in the full column range, plus
    the per-surface maxima of both signs [C][n_surf]."""
    assign = np.asarray(assign)
    pos = _positions(masking_array)
    merge_y = np.asarray(merge_y)
    C = np.asarray(pred_x).reshape(merge_y.shape[0], -1).shape[1]
    tv_all = np.zeros((C, merge_y.shape[1]), np.float32)
    tp_all, tn_all = np.zeros_like(tv_all), np.zeros_like(tv_all)
    for g in np.unique(assign):
        surf = np.flatnonzero(assign == g)
        cols = np.concatenate([np.arange(pos[s], pos[s + 1]) for s in surf])
        vd = vdensity if np.isscalar(vdensity) else np.asarray(vdensity)[cols]
        H, E = settings[int(g)]
        tv, tp, tn = calculate_tfce(merge_y[:, cols], [masking_array[s] for s in surf], pred_x,
                                    [adjacency_array[s] for s in surf], H, E, vd, perm=perm)
        tv_all[:, cols], tp_all[:, cols], tn_all[:, cols] = tv, tp, tn
    return tv_all, tp_all, tn_all


def calculate_mediation_tfce(medtype, merge_y, masking_array, pred_x, depend_y, adjacency_array, H, E,
                             vdensity=1, perm=None):
    """tm_func.calculate_mediation_tfce (tm_func.py:207-249), observed form:
    the Aroian z map (calc_sobelz) swept once over the merged adjacency and
    scaled per surface.  perm permutes pred_x (and depend_y for 'Y'), as the
    randomised call does.  Returns (SobelZ, tfce_SobelZ) float32."""
    merge_y = np.asarray(merge_y)
    n = merge_y.shape[0]
    x, dy = np.asarray(pred_x), np.asarray(depend_y)
    if perm is not None:
        x = x[perm]
        if medtype == "Y":
            dy = dy[perm]
    z = calc_sobelz(medtype, x, dy, merge_y, n).astype(np.float32)
    off, idx = merge_adjacency(adjacency_array)
    full = _full_mask(masking_array) == 1
    img = np.zeros(full.shape[0], np.float32)
    img[full] = z
    e = tfce(off, idx, img, H, E)[full]
    return z, _scaled(e, img[full], _positions(masking_array), vdensity)


def vert_stat_tfce_image(vertStat, bin_mask, offsets, indices, H, E, density=1):
    """The TFCE image of write_vertStat_img (pyfunc.py:80-92): the masked
    statistic scattered into a zero-filled hemisphere, swept, scaled by the max
    of its finite masked values / 100 and the density weight."""
    bin_mask = np.asarray(bin_mask, bool)
    out = np.zeros(bin_mask.shape[0], np.float32)
    out[bin_mask] = vertStat
    e = tfce(offsets, indices, out, H, E)
    vs = np.asarray(vertStat)
    return e * (vs[np.isfinite(vs)].max() / 100) * density


def voxel_stat_tfce_image(voxelStat, offsets, indices, H, E):
    """The TFCE values of write_voxelStat_img (pyfunc.py:94-103) over the
    mask's voxels: swept, scaled by the statistic's max / 100."""
    v = np.asarray(voxelStat).astype(np.float32)
    return tfce(offsets, indices, v, H, E) * (v.max() / 100)


def fwep_vertex(tfce_values, null):
    """1-p(FWER) as tfce_mediation/tmanalysis/calculate_fweP_vertex.py:37-69:
    sorted null, p_array[j] = j/N, idx = searchsorted(left),
    1-p = p_array[idx-1] (p_array[0] when idx == 0); computed where TFCE > 0."""
    srt = np.sort(np.asarray(null, np.float64))
    N = srt.shape[0]
    p_array = np.arange(N, dtype=np.float64) / N
    v = np.asarray(tfce_values)
    out = np.zeros(v.shape, np.float64)
    m = v > 0
    idx = np.searchsorted(srt, v[m], side="left")
    out[m] = p_array[np.maximum(idx - 1, 0)]
    return out


def find_nearest(array, value, p_array):
    """Nearest-rank lookup of tm_func.py:566-573 / pyfunc.py:254-261."""
    idx = np.searchsorted(array, value, side="left")
    if idx == len(p_array):
        return p_array[idx - 1]
    elif math.fabs(value - array[idx - 1]) < math.fabs(value - array[idx]):
        return p_array[idx - 1]
    else:
        return p_array[idx]


def apply_mfwer(pos_images, neg_images, perm_max, position_array, weight=None, mediation=False):
    """tm_func.py:403-491 with the permutation CSV contents passed in memory.

    pos_images/neg_images: (V_total, C) scaled TFCE images; perm_max:
    dict {(surface, contrast): 1-D array of permutation maxima}.  Returns
    (positive_1mp, negative_1mp)."""
    num_contrasts = pos_images.shape[1]
    num_surf = len(position_array) - 1
    num_perm = min(len(v) for v in perm_max.values())
    maxvalue_array = np.zeros((num_perm, num_contrasts))
    temp_max = np.zeros((num_perm, num_surf))
    positive_data = np.zeros((pos_images.shape[0], num_contrasts))
    negative_data = np.zeros((pos_images.shape[0], num_contrasts))
    if weight == "logmasksize":
        x = [position_array[i + 1] - position_array[i] for i in range(num_surf)]
        weights = (np.log(x) / np.log(x).sum()) / np.mean(np.log(x) / np.log(x).sum())
        w_temp_max = np.zeros((num_perm, num_surf))
    with np.errstate(divide="ignore", invalid="ignore"):
        for c in range(num_contrasts):
            for s in range(num_surf):
                lp = np.log(np.asarray(perm_max[(s, c)], np.float64)[:num_perm])
                lp[np.isinf(lp)] = 0
                start, end = position_array[s], position_array[s + 1]
                imgs = [(pos_images, positive_data)] + ([] if mediation else [(neg_images, negative_data)])
                for src, dst in imgs:
                    vm = np.log(src[start:end, c]) > 0
                    lt = np.log(src[start:end, c][vm])
                    lt -= lp.mean()
                    lt /= lp.std()
                    lt += 10
                    dst[start:end, c][vm] = lt
                lp -= lp.mean()
                lp /= lp.std()
                if weight == "logmasksize":
                    w = lp * weights[s]
                    w += 10
                    w_temp_max[:, s] = w
                lp += 10
                temp_max[:, s] = lp
            if weight is not None:
                w_temp_max[np.isnan(w_temp_max)] = 0
                mi = np.argmax(w_temp_max, axis=1)
                mv = np.zeros(len(mi), dtype=np.float32)
                for i in range(len(temp_max)):
                    mv[i] = temp_max[i, mi[i]]
                maxvalue_array[:, c] = np.sort(mv)
            else:
                maxvalue_array[:, c] = np.sort(temp_max.max(axis=1))
    for c in range(num_contrasts):
        srt = maxvalue_array[:, c]
        p_array = np.arange(num_perm, dtype=np.float64) / num_perm
        positive_data[:, c] = [find_nearest(srt, k, p_array) for k in positive_data[:, c]]
        if not mediation:
            negative_data[:, c] = [find_nearest(srt, k, p_array) for k in negative_data[:, c]]
    return positive_data, (None if mediation else negative_data)


# -- tm-models repeated-measures ANCOVA (reg_rm_ancova_*_bs_factor) ----------
def _dummy_code(variable, demean=True):
    """dummy_code(iscontinous=False) (tm/pyfunc.py:2564-2600): one column per
    level after the first, squeezed, optionally demeaned."""
    variable = np.asarray(variable)
    cols = [(variable == v).astype(np.float64) for v in np.unique(variable)]
    d = np.squeeze(np.array(cols)[1:]).astype(int).T
    return d - np.mean(d, 0) if demean else d


def _column_product(a1, a2):
    """column_product (tm/pyfunc.py:2622-2660): every column of a1 times every
    column of a2, a1-major."""
    a1, a2 = np.asarray(a1), np.asarray(a2)
    if a1.ndim == 1:
        return (a1 * a2.T).T
    if a2.ndim == 1:
        return (a2 * a1.T).T
    return np.concatenate([(a1[:, i] * a2.T).T.reshape(len(a1), -1) for i in range(a1.shape[1])], axis=1)


def _ones(a):
    return np.column_stack([np.ones(len(a)), a])


def _rss(X, y):
    a = np.linalg.inv(X.T @ X) @ X.T @ y
    return np.sum((y - X @ a) ** 2, axis=0)


def _rm_long(data, data_format, n_short):
    if data_format == "short":
        data = np.asarray(data)
        if data.ndim == 2:
            data = data[:, :, None]
        s, n = data.shape[0], data.shape[1]
        return data.reshape(s * n, data.shape[2]), n, s
    n = n_short
    return np.asarray(data), n, len(data) // n


def _tile(a, s):
    return None if a is None else np.concatenate([a] * s, 0)


def rm_ancova_one(data, dmy_factor1, dmy_subjects, dmy_covariates=None, data_format="short", rand_array=None,
                  shuffle=None):
    """reg_rm_ancova_one_bs_factor (tm/pyfunc.py:2067-2280) without p values:
    (F_a, F_s, F_sa).  Every SS is the reference's SS_Total - RSS difference
    (FP64 fits; SS_Total in the data's own type).  With rand_array the data's
    long rows are shuffled by the index array `shuffle` (what the reference's
    np.random.shuffle draws next from the global RNG) and the factor and
    covariate rows permuted by rand_array."""
    endog, n, s = _rm_long(data, data_format, len(dmy_factor1))
    f1 = np.asarray(dmy_factor1, np.float64)
    cov = None if dmy_covariates is None else np.asarray(dmy_covariates, np.float64)
    fa = 2 if f1.ndim == 1 else f1.shape[1] + 1
    if rand_array is not None:
        endog = endog[np.asarray(shuffle)]
        f1 = f1[rand_array]
        cov = None if cov is None else cov[rand_array]
    y_in = np.squeeze(endog)
    y = np.asarray(y_in, np.float64)
    interval = np.concatenate([np.full(n, float(i)) for i in range(s)])
    iv = _dummy_code(interval, demean=False)
    f1l, subl, covl = _tile(f1, s), _tile(np.asarray(dmy_subjects, np.float64), s), _tile(cov, s)
    sst = np.sum((y_in - np.mean(y_in, axis=0)) ** 2, axis=0).astype(np.float64)
    ss_ws = _rss(_ones(subl), y)
    ss_bs = sst - ss_ws
    X = _ones(f1l) if covl is None else np.column_stack([_ones(f1l), covl])
    ss_cells_a = sst - _rss(X, y)
    ss_cov = 0.0 if covl is None else sst - _rss(_ones(covl), y)
    ss_a = ss_cells_a - ss_cov
    ss_wf = ss_bs - ss_a - ss_cov
    ss_s = sst - _rss(_ones(iv), y)
    ss_scov = 0.0
    if covl is not None:
        cells = sst - _rss(np.column_stack([_ones(covl), _column_product(covl, iv), iv]), y)
        ss_scov = cells - (sst - _rss(np.column_stack([_ones(covl), iv]), y))
    X = np.column_stack([_ones(f1l), iv, _column_product(f1l, iv)])
    X2 = np.column_stack([_ones(f1l), iv])
    if covl is not None:
        X = np.column_stack([X, covl, _column_product(covl, iv)])
        X2 = np.column_stack([X2, covl, _column_product(covl, iv)])
    ss_sa = (sst - _rss(X, y)) - (sst - _rss(X2, y))
    ss_swf = ss_ws - ss_s - ss_sa - ss_scov
    df_a = fa - 1
    df_cov = 0 if cov is None else (1 if cov.ndim == 1 else cov.shape[1])
    df_wf = n - 1 - df_a - df_cov
    df_s = s - 1
    df_sa, df_swf = df_a * df_s, df_wf * df_s
    ms_wf, ms_swf = ss_wf / df_wf, ss_swf / df_swf
    return (ss_a / df_a) / ms_wf, (ss_s / df_s) / ms_swf, (ss_sa / df_sa) / ms_swf


def rm_ancova_two(data, dmy_factor1, dmy_factor2, dmy_subjects, dmy_covariates=None, data_format="short",
                  rand_array=None, shuffle=None):
    """reg_rm_ancova_two_bs_factor (tm/pyfunc.py:1712-2060) without p values:
    (F_a, F_b, F_ab, F_s, F_sa, F_sb, F_sab), type I sums of squares as the
    reference forms them (see rm_ancova_one for the permutation arguments)."""
    endog, n, s = _rm_long(data, data_format, len(dmy_factor1))
    f1 = np.asarray(dmy_factor1, np.float64)
    f2 = np.asarray(dmy_factor2, np.float64)
    cov = None if dmy_covariates is None else np.asarray(dmy_covariates, np.float64)
    fa = 2 if f1.ndim == 1 else f1.shape[1] + 1
    fb = 2 if f2.ndim == 1 else f2.shape[1] + 1
    if rand_array is not None:
        endog = endog[np.asarray(shuffle)]
        f1, f2 = f1[rand_array], f2[rand_array]
        cov = None if cov is None else cov[rand_array]
    y_in = endog
    y = np.asarray(y_in, np.float64)
    f12 = _column_product(f1, f2)
    interval = np.concatenate([np.full(n, float(i)) for i in range(s)])
    iv = _dummy_code(interval, demean=False)
    f1l, f2l, f12l = _tile(f1, s), _tile(f2, s), _tile(f12, s)
    subl, covl = _tile(np.asarray(dmy_subjects, np.float64), s), _tile(cov, s)

    def with_cov(X, cross=False):
        if covl is None:
            return X
        X = np.column_stack([X, covl])
        return np.column_stack([X, _column_product(covl, iv)]) if cross else X

    sst = np.sum((y_in - np.mean(y_in, axis=0)) ** 2, axis=0).astype(np.float64)
    ss_ws = _rss(_ones(subl), y)
    ss_bs = sst - ss_ws
    ss_cells_ab = sst - _rss(with_cov(np.column_stack([_ones(f1l), f2l, f12l])), y)
    ss_ab = ss_cells_ab - (sst - _rss(with_cov(_ones(np.column_stack([f1l, f2l]))), y))
    ss_cov = 0.0 if covl is None else sst - _rss(_ones(covl), y)
    ss_a = (sst - _rss(with_cov(_ones(f1l)), y)) - ss_cov
    ss_b = ss_cells_ab - ss_cov - ss_ab - ss_a
    ss_wf = ss_bs - ss_a - ss_b - ss_ab - ss_cov
    ss_s = sst - _rss(_ones(iv), y)
    base = np.column_stack([_ones(f1l), f2l, f12l, iv, _column_product(f1l, iv), _column_product(f2l, iv)])
    ss_sab = (sst - _rss(with_cov(np.column_stack([base, _column_product(f12l, iv)]), True), y)) \
        - (sst - _rss(with_cov(base, True), y))
    ss_scov = 0.0
    if covl is not None:
        cells = sst - _rss(np.column_stack([_ones(covl), _column_product(covl, iv), iv]), y)
        ss_scov = cells - (sst - _rss(np.column_stack([_ones(covl), iv]), y))
    ss_sa = (sst - _rss(with_cov(np.column_stack([_ones(f1l), iv, _column_product(f1l, iv)]), True), y)) \
        - (sst - _rss(with_cov(np.column_stack([_ones(f1l), iv]), True), y))
    Xb = np.column_stack([_ones(f1l), f2l, iv, _column_product(f1l, iv)])
    ss_sb = (sst - _rss(with_cov(np.column_stack([Xb, _column_product(f2l, iv)]), True), y)) \
        - (sst - _rss(with_cov(Xb, True), y))
    ss_swf = ss_ws - ss_s - ss_sa - ss_sb - ss_sab - ss_scov
    df_a, df_b = fa - 1, fb - 1
    df_ab = df_a * df_b
    df_cov = 0 if cov is None else (1 if cov.ndim == 1 else cov.shape[1])
    df_wf = n - 1 - df_a - df_b - df_ab - df_cov
    df_s = s - 1
    df_swf = df_wf * df_s
    ms_wf, ms_swf = ss_wf / df_wf, ss_swf / df_swf
    return ((ss_a / df_a) / ms_wf, (ss_b / df_b) / ms_wf, (ss_ab / df_ab) / ms_wf, (ss_s / df_s) / ms_swf,
            (ss_sa / (df_a * df_s)) / ms_swf, (ss_sb / (df_b * df_s)) / ms_swf,
            (ss_sab / (df_ab * df_s)) / ms_swf)


# -- geodesic FWHM smoothing (cynumstats.calc_gd_fwhm) -------------------------
_LIBM = None


def _libm():
    """The host C math library: the reference's compiled pdf_compute calls
    powf and, being C++, the float overload of exp (expf)."""
    global _LIBM
    if _LIBM is None:
        m = ctypes.CDLL(ctypes.util.find_library("m") or "libm.so.6")
        m.powf.restype, m.powf.argtypes = ctypes.c_float, [ctypes.c_float, ctypes.c_float]
        m.expf.restype, m.expf.argtypes = ctypes.c_float, [ctypes.c_float]
        _LIBM = m
    return _LIBM


def gd_weight(x, scale):
    """pdf_compute(x, 0, scale) as the reference's compiled Cython evaluates it
    (tm/cynumstats.pyx:76-81, C float arguments, result stored to a C float):
      norm     = float(sqrt((2.0 * M_PI) * scale))            double sqrt
      exponent = float((-1.0 * powf(x - 0, 2)) / (2.0 * scale)) double division
      weight   = float((1.0 / norm) * expf(exponent))          float exp (C++ overload)
    The reference's 'scale' acts as a variance."""
    m = _libm()
    s32 = np.float32(scale)
    norm = np.float32(math.sqrt((2.0 * math.pi) * float(s32)))
    p = np.float32(m.powf(float(np.float32(np.float32(x) - np.float32(0.0))), 2.0))
    ex = np.float32((-1.0 * float(p)) / (2.0 * float(s32)))
    return np.float32((1.0 / float(norm)) * float(m.expf(float(ex))))


def calc_gd_fwhm(indices, dist, data, sigma):
    """calc_gd_fwhm (tm/cynumstats.pyx:83-107), a pure-Python loop for small
    cases: every pair (i, j) adds weight*data[i] to j and weight*data[j] to i
    and the weight to both, then the self weight, then sumval / sum_weight.
    The product is a C float product; the accumulators are float32 arrays
    updated through numpy scalars, and with numpy >= 2 (NEP 50) a float32
    scalar plus a Python float stays float32: every update is one float32
    rounding of the product and one of the sum."""
    indices = np.asarray(indices)
    data = np.asarray(data, np.float32)
    V = data.shape[0]
    sumval = [np.float32(0.0)] * V
    sumw = [np.float32(0.0)] * V
    for x in range(len(dist)):
        i, j = int(indices[x, 0]), int(indices[x, 1])
        w = gd_weight(dist[x], sigma)
        sumval[j] = np.float32(sumval[j] + np.float32(w * data[i]))
        sumval[i] = np.float32(sumval[i] + np.float32(w * data[j]))
        sumw[i] = np.float32(sumw[i] + w)
        sumw[j] = np.float32(sumw[j] + w)
    w0 = gd_weight(0.0, sigma)
    for i in range(V):
        sumval[i] = np.float32(sumval[i] + np.float32(w0 * data[i]))
        sumw[i] = np.float32(sumw[i] + w0)
    return np.asarray(sumval, np.float32) / np.asarray(sumw, np.float32)
