"""ctypes binding of the native C-ABI (``include/tfce_gb300.h``).

The library is ``tfce_mediation_gb300/_native/libtfce_gb300.so`` built by
``tfce_mediation_gb300/build.py``.  There is no CPU fallback: if the library is
missing or cannot be loaded every entry point raises ``NativeLibraryError``.
"""
from __future__ import annotations

import ctypes
import os
import threading

from . import build as _build

_lock = threading.Lock()
_LIB = None

c_f32p = ctypes.POINTER(ctypes.c_float)
c_f64p = ctypes.POINTER(ctypes.c_double)
c_i32p = ctypes.POINTER(ctypes.c_int32)
c_i64p = ctypes.POINTER(ctypes.c_int64)
c_vp = ctypes.c_void_p

TFCE_OK, TFCE_EINVAL, TFCE_EDEVICE, TFCE_ETIMEOUT, TFCE_ENOMEM, TFCE_ERANGE = range(6)


class NativeLibraryError(RuntimeError):
    """The CUDA library is missing or failed to load."""


class TfceError(RuntimeError):
    """A native entry point returned a non-OK status."""

    def __init__(self, status: int, message: str):
        super().__init__(f"[status {status}] {message}")
        self.status = status


# name -> (restype, argtypes); mirrors include/tfce_gb300.h
SIGNATURES = {
    "tfce_version": (ctypes.c_int, []),
    "tfce_last_error": (ctypes.c_char_p, []),
    "tfce_adjset_create": (ctypes.c_int, [c_i64p, c_i32p, ctypes.c_int32, c_i64p, ctypes.c_int32,
                                          c_f32p, c_f32p, ctypes.POINTER(c_vp)]),
    "tfce_adjset_destroy": (None, [c_vp]),
    "tfce_adjset_set_params": (ctypes.c_int, [c_vp, c_f32p, c_f32p]),
    "tfce_adjset_is_symmetric": (ctypes.c_int, [c_vp]),
    "tfce_adjset_set_threshold_groups": (ctypes.c_int, [c_vp, c_i32p]),
    "tfce_adjset_set_sweep_shape": (ctypes.c_int, [c_vp, ctypes.c_int32]),
    "tfce_adjset_set_accumulation": (ctypes.c_int, [c_vp, ctypes.c_int32]),
    "tfce_adjset_run": (ctypes.c_int, [c_vp, c_f32p, c_f32p, ctypes.c_int32]),
    "tfce_adjset_run_labels": (ctypes.c_int, [c_vp, c_f32p, c_f32p, ctypes.c_int32, c_i32p, c_i32p,
                                              ctypes.c_int32, c_i32p]),
    "tfce_sweep_batch": (ctypes.c_int, [c_vp, c_vp, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32,
                                        c_vp, ctypes.c_int32, c_vp, c_vp, ctypes.c_int32, c_vp]),
    "tfce_sweep_status": (ctypes.c_int, [c_vp, c_vp]),
    "tfce_sweep_resident_slots": (ctypes.c_int, [c_vp, c_vp]),
    "tfce_sweep_batch_noalloc": (ctypes.c_int, [c_vp, c_vp, ctypes.c_int32, ctypes.c_int64, c_vp,
                                                ctypes.c_int32, ctypes.c_int32, c_vp, c_vp, c_vp,
                                                ctypes.c_int64, ctypes.c_int32, ctypes.c_int32, c_vp,
                                                ctypes.c_int32, c_vp, c_vp]),
    "geodesic_mesh_create": (ctypes.c_int, [c_f32p, ctypes.c_int32, c_i32p, ctypes.c_int32, ctypes.POINTER(c_vp)]),
    "geodesic_mesh_destroy": (None, [c_vp]),
    "geodesic_mesh_saddles": (ctypes.c_int, [c_vp, c_i32p]),
    "geodesic_distance_lists": (ctypes.c_int, [c_vp, ctypes.c_double, ctypes.c_int32, ctypes.c_int32,
                                               ctypes.c_int32, c_i64p]),
    "geodesic_take_lists": (ctypes.c_int, [c_vp, c_i32p, c_i32p, c_f64p, ctypes.c_int64]),
    "glm_tstat": (ctypes.c_int, [c_vp, ctypes.c_int64, ctypes.c_int32, ctypes.c_int64, c_vp, c_vp,
                                 c_vp, c_vp, ctypes.c_int32, ctypes.c_int32, c_vp, ctypes.c_int32,
                                 c_vp, ctypes.c_int64, c_vp]),
    "glm_stat": (ctypes.c_int, [c_vp, ctypes.c_int64, ctypes.c_int32, ctypes.c_int64, c_vp, c_vp,
                                c_vp, c_vp, ctypes.c_int32, ctypes.c_int32, c_vp, ctypes.c_int32,
                                ctypes.c_int32, c_vp, ctypes.c_int64, c_vp]),
    "glm_stat_f64": (ctypes.c_int, [c_vp, ctypes.c_int64, ctypes.c_int32, ctypes.c_int64, c_vp, c_vp, c_vp, c_vp,
                                    ctypes.c_int32, ctypes.c_int32, c_vp, ctypes.c_int32, ctypes.c_int32, c_vp,
                                    ctypes.c_int64, c_vp]),
    "glm_fstat": (ctypes.c_int, [c_vp, ctypes.c_int64, ctypes.c_int32, ctypes.c_int64, c_vp, c_vp,
                                 c_vp, ctypes.c_int32, ctypes.c_int32, c_vp, c_vp, ctypes.c_int64,
                                 c_vp]),
    "glm_tc_design_block": (ctypes.c_int, [ctypes.c_int32]),
    "glm_tile_bytes": (ctypes.c_int64, [ctypes.c_int64, ctypes.c_int32, ctypes.c_int32]),
    "glm_col_mean": (ctypes.c_int, [c_vp, ctypes.c_int64, ctypes.c_int32, ctypes.c_int64, c_vp, c_vp]),
    "glm_tile_split": (ctypes.c_int, [c_vp, ctypes.c_int64, ctypes.c_int32, ctypes.c_int64, ctypes.c_int32,
                                      c_vp, ctypes.c_int32, ctypes.c_int32, c_vp, c_vp, c_vp]),
    "glm_tstat_tc": (ctypes.c_int, [c_vp, c_vp, c_vp, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32,
                                    ctypes.c_int64, c_vp, c_vp, c_vp, ctypes.c_int32, c_vp, c_vp, ctypes.c_int32,
                                    ctypes.c_int32, c_vp, ctypes.c_int32, c_vp, ctypes.c_int64, c_vp, c_vp]),
    "perm_stream": (ctypes.c_int, [ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, c_vp,
                                   ctypes.c_int32]),
    "glm_qf_design_block": (ctypes.c_int, [ctypes.c_int32]),
    "glm_col_sumsq": (ctypes.c_int, [c_vp, ctypes.c_int64, ctypes.c_int32, ctypes.c_int64, c_vp, c_vp]),
    "glm_tstat_tc_qf": (ctypes.c_int, [c_vp, c_vp, ctypes.c_int32, ctypes.c_int32, ctypes.c_int64, c_vp, c_vp,
                                       c_vp, c_vp, ctypes.c_int32, ctypes.c_int32, c_vp, ctypes.c_int32, c_vp,
                                       ctypes.c_int64, c_vp, c_vp]),
    "glm_col_center": (ctypes.c_int, [c_vp, ctypes.c_int64, ctypes.c_int32, ctypes.c_int64, c_vp, c_vp, c_vp]),
    "glm_stat_tc": (ctypes.c_int, [c_vp, c_vp, c_vp, c_vp, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32,
                                   ctypes.c_int64, c_vp, c_vp, c_vp, ctypes.c_int32, c_vp, c_vp, ctypes.c_int32,
                                   ctypes.c_int32, ctypes.c_int32, c_vp, ctypes.c_int32, c_vp, ctypes.c_int32,
                                   c_vp, ctypes.c_int64, c_vp, c_vp]),
    "glm_stat_tc_block": (ctypes.c_int, [c_vp, c_vp, c_vp, c_vp, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32,
                                         ctypes.c_int64, c_vp, c_vp, c_vp, ctypes.c_int32, c_vp, c_vp, ctypes.c_int32,
                                         ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, c_vp, ctypes.c_int32, c_vp,
                                         ctypes.c_int32, c_vp, ctypes.c_int64, c_vp, c_vp]),
    "sobel_combine": (ctypes.c_int, [c_vp, ctypes.c_int64, c_vp, c_vp, ctypes.c_int64,
                                     ctypes.c_int32, ctypes.c_int64, ctypes.c_int32, c_vp,
                                     ctypes.c_int64, c_vp]),
    "rm_anova_max_rows": (ctypes.c_int, []),
    "rm_anova_combine": (ctypes.c_int, [c_vp, ctypes.c_int64, ctypes.c_int32, ctypes.c_int64, c_vp, ctypes.c_int32,
                                        c_vp, ctypes.c_int32, c_vp, c_vp, c_vp, ctypes.c_int32, c_vp,
                                        ctypes.c_int32, c_vp, ctypes.c_int32, ctypes.c_float, ctypes.c_float,
                                        c_vp, c_vp, c_vp, ctypes.c_int32, c_vp, ctypes.c_int64, c_vp, c_vp,
                                        c_vp]),
    "gd_fwhm_weights": (ctypes.c_int, [c_vp, ctypes.c_int64, ctypes.c_float, c_vp, c_vp]),
    "gd_fwhm_smooth": (ctypes.c_int, [c_vp, c_vp, c_vp, c_vp, ctypes.c_int64, c_vp, ctypes.c_int64,
                                      ctypes.c_int32, ctypes.c_int32, c_vp, ctypes.c_int64, c_vp, c_vp]),
    "fwer_sort": (ctypes.c_int, [c_vp, ctypes.c_int64, c_vp]),
    "fwer_lookup": (ctypes.c_int, [c_vp, ctypes.c_int64, c_vp, ctypes.c_int64, ctypes.c_int32,
                                   c_vp, c_vp]),
    "mlp_gemm": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                c_vp, ctypes.c_int32, c_vp, ctypes.c_int32, c_vp, ctypes.c_int32, c_vp,
                                ctypes.c_int32, c_vp, ctypes.c_int32, c_vp]),
    "mlp_gemm_bf16": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                     ctypes.c_int32, c_vp, ctypes.c_int32, c_vp, ctypes.c_int32, c_vp,
                                     ctypes.c_int32, c_vp, ctypes.c_int32, c_vp]),
    "mlp_to_bf16": (ctypes.c_int, [c_vp, c_vp, ctypes.c_int64, c_vp]),
    "mlp_gelu_backward": (ctypes.c_int, [c_vp, c_vp, c_vp, ctypes.c_int64, c_vp]),
    "mlp_bias_grad": (ctypes.c_int, [c_vp, ctypes.c_int32, ctypes.c_int32, c_vp, c_vp]),
    "mlp_mse_loss": (ctypes.c_int, [c_vp, c_vp, c_vp, ctypes.c_int64, ctypes.c_int32, c_vp, c_vp, c_vp]),
    "mlp_adam_step": (ctypes.c_int, [c_vp, c_vp, c_vp, c_vp, ctypes.c_int64, ctypes.c_float, ctypes.c_float,
                                     ctypes.c_float, ctypes.c_float, ctypes.c_int32, ctypes.c_float, c_vp]),
}


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load (building first if the .so is absent or stale) the native library."""
    global _LIB
    with _lock:
        if _LIB is not None:
            return _LIB
        path = _build.LIB
        if build_if_missing:
            try:
                path = _build.build()
            except Exception as exc:  # no silent fallback
                if not os.path.exists(path):
                    raise NativeLibraryError(f"cannot build {path}: {exc}") from exc
        if not os.path.exists(path):
            raise NativeLibraryError(f"native library not built: {path}")
        try:
            lib = ctypes.CDLL(path)
        except OSError as exc:
            raise NativeLibraryError(f"cannot load {path}: {exc}") from exc
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = lib
        return lib


def check(status: int) -> None:
    if status != TFCE_OK:
        msg = load().tfce_last_error()
        raise TfceError(status, msg.decode() if msg else "")


def ptr(arr, ctype):
    """ctypes pointer to a contiguous numpy array."""
    return arr.ctypes.data_as(ctype)
