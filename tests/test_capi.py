"""The C-ABI library builds for sm_103a, loads, and exports every entry point
that include/*.h declares (no compute calls: these run without a GPU)."""
import ctypes
import glob
import os
import re

from tfce_mediation_gb300 import _lib, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**\s+\**([a-z_][a-z0-9_]*)\s*\(",
                             src, flags=re.M):
            names.add(m.group(1))
    return names


def test_header_declares_entry_points():
    names = declared_functions()
    for n in ("tfce_adjset_create", "tfce_adjset_run", "tfce_sweep_batch", "glm_tstat", "fwer_lookup"):
        assert n in names


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    assert declared_functions() <= set(_lib.SIGNATURES)


def test_version_and_error_string():
    lib = _lib.load()
    assert lib.tfce_version() >= 100
    assert isinstance(lib.tfce_last_error(), bytes)


def test_invalid_arguments_are_rejected_on_host():
    """Argument validation happens before any device work."""
    lib = _lib.load()
    h = ctypes.c_void_p()
    import numpy as np
    off = np.array([0, 1, 2], np.int64)
    idx = np.array([1, 5], np.int32)  # 5 is out of range
    H = np.array([2.0], np.float32)
    E = np.array([1.0], np.float32)
    rc = lib.tfce_adjset_create(_lib.ptr(off, _lib.c_i64p), _lib.ptr(idx, _lib.c_i32p), 2, None, 1,
                                _lib.ptr(H, _lib.c_f32p), _lib.ptr(E, _lib.c_f32p), ctypes.byref(h))
    assert rc == _lib.TFCE_EINVAL
    assert b"outside" in lib.tfce_last_error()
    assert lib.tfce_sweep_batch(None, None, 0, 0, 2, None, 0, None, None, 0, None) == _lib.TFCE_EINVAL
    assert lib.glm_tstat(None, 1, 1, 1, None, None, None, None, 1, 1, None, 1, None, 1, None) == _lib.TFCE_EINVAL
    assert lib.fwer_lookup(None, 0, None, 1, 0, None, None) == _lib.TFCE_EINVAL


def test_new_entries_reject_invalid_arguments_on_host():
    """The tm-models, smoothing and slot-query entries validate before any
    device work."""
    lib = _lib.load()
    E = _lib.TFCE_EINVAL
    assert lib.tfce_sweep_resident_slots(None, None) == E
    # rm_anova_combine: NULL data, then N out of range
    assert lib.rm_anova_combine(None, 1, 2, 1, None, 1, None, 1, None, None, None, 0, None, 0, None, 0,
                                ctypes.c_float(1.0), ctypes.c_float(1.0), None, None, None, 0, None, 1, None,
                                None, None) == E
    one = ctypes.c_void_p(16)  # never dereferenced: the size checks fail first
    assert lib.rm_anova_combine(one, 1, 100000, 1, one, 1, one, 1, None, None, None, 0, None, 0, None, 0,
                                ctypes.c_float(1.0), ctypes.c_float(1.0), None, None, None, 0, one, 1, None,
                                one, None) == E
    assert b"N (data rows)" in lib.tfce_last_error()
    assert lib.gd_fwhm_weights(None, 1, ctypes.c_float(0.5), None, None) == E
    assert lib.gd_fwhm_weights(one, 1, ctypes.c_float(-1.0), one, None) == E
    assert lib.gd_fwhm_smooth(None, None, None, None, 0, None, 1, 1, 1, None, 1, None, None) == E
    # glm_stat_tc: mode out of range
    assert lib.glm_stat_tc(one, None, one, None, 16, 16, 16, 16, one, None, one, 32, one, one, 1, 5, 9, one, 1,
                           None, 0, one, 16, one, None) == E
    assert b"mode" in lib.tfce_last_error()


def test_quadratic_form_glm_arguments_are_rejected_on_host():
    """glm_tstat_tc_qf checks its sizes and pointers before any device work:
    kmax outside [2, 8], more than 8 coefficients, n_pad not a multiple of 16
    or below n, and NULL operands are TFCE_EINVAL."""
    lib = _lib.load()
    assert lib.glm_qf_design_block(5) == 64 and lib.glm_qf_design_block(8) == 32
    assert lib.glm_qf_design_block(1) == -1 and lib.glm_qf_design_block(9) == -1
    fake = ctypes.c_void_p(256)  # never dereferenced: every call below fails its host checks

    def call(n=100, n_pad=112, V=10, G=4, kmax=5, n_coef=2, ptrs=True, ldt=10):
        p = fake if ptrs else None
        return lib.glm_tstat_tc_qf(p, p, n, n_pad, V, p, p, p, p, G, kmax, p, n_coef, p, ldt, p, None)

    for kw in ({"kmax": 1}, {"kmax": 9}, {"n_coef": 0}, {"n_coef": 9}, {"n_pad": 100}, {"n_pad": 96},
               {"ptrs": False}, {"ldt": 5}, {"n": 5, "n_pad": 16}):
        assert call(**kw) == _lib.TFCE_EINVAL, kw
    assert lib.glm_col_sumsq(None, 10, 5, 10, None, None) == _lib.TFCE_EINVAL
