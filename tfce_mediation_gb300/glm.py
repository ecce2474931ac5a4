"""Batched OLS on the device (glm_stat / glm_tstat of the C-ABI).

Host side keeps FP64 for what is k x k: for every design the pseudoinverse
inv(X'X) X' and diag(inv(X'X)) are formed in float64 with numpy (as
cy_lin_lstsqr_mat does, tfce_mediation/cynumstats.pyx:28-29) and handed to the
kernel as float32 operands; the n x V contraction, residuals, RSS, SE and t run
in the kernel.
"""
from __future__ import annotations

import numpy as np

from . import _lib
from .device import dev, ptr, require_cuda, stream_handle

WHAT_T, WHAT_BETA, WHAT_SE, WHAT_RESID, WHAT_F, WHAT_RSS = range(6)


class DesignBatch:
    """Stacked operators of G designs padded to kmax columns.

    designs: array (G, n, k) or list of (n, k_g) arrays (float64).
    invXX: optional (G, k, k) matrices whose diagonal gives the SE factor (the
    reference passes its own invXX to tval_int); default inv(X'X)."""

    def __init__(self, designs, invXX=None, kmax=None):
        if isinstance(designs, np.ndarray) and designs.ndim == 3:
            mats = [designs[g] for g in range(designs.shape[0])]
        else:
            mats = [np.asarray(d, np.float64) for d in designs]
        G = len(mats)
        n = mats[0].shape[0]
        ks = [m.shape[1] for m in mats]
        kmax = kmax or max(ks)
        if kmax > 8:
            raise ValueError("at most 8 regressors per design")
        pinv = np.zeros((G, kmax, n), np.float64)
        Xp = np.zeros((G, n, kmax), np.float64)
        invdiag = np.zeros((G, kmax), np.float64)
        same_k = len(set(ks)) == 1
        if same_k:
            Xs = np.stack(mats).astype(np.float64)
            inv = np.linalg.inv(np.einsum("gsi,gsj->gij", Xs, Xs))
            k = ks[0]
            pinv[:, :k, :] = np.einsum("gij,gsj->gis", inv, Xs)
            Xp[:, :, :k] = Xs
            di = np.diagonal(inv if invXX is None else np.asarray(invXX, np.float64), axis1=1, axis2=2)
            invdiag[:, :k] = di
        else:
            for g, m in enumerate(mats):
                k = m.shape[1]
                inv = np.linalg.inv(m.T @ m)
                pinv[g, :k] = inv @ m.T
                Xp[g, :, :k] = m
                invdiag[g, :k] = np.diag(inv if invXX is None else np.asarray(invXX[g], np.float64))
        self.G, self.n, self.kmax, self.ks = G, n, kmax, ks
        self.pinv64, self.X64, self.invdiag64 = pinv, Xp, invdiag
        self.dof = np.asarray([n - k for k in ks], np.float64)

    def to_device(self):
        return (dev(self.pinv64.astype(np.float32)), dev(self.X64.astype(np.float32)),
                dev(self.invdiag64.astype(np.float32)), dev(self.dof.astype(np.float32)))


def glm_stat(Y, designs, what=WHAT_T, coef=None, out=None, stream=None):
    """Run one of the fitted outputs for every design of a DesignBatch.

    Y: CUDA float32 tensor (n, V) (or host array, uploaded).  Returns a CUDA
    tensor: (G, n_coef, V) for t/beta/se, (G, n, V) for residuals, (G, V) for
    F/RSS."""
    t = require_cuda()
    Yd = dev(Y, t.float32)
    n, V = Yd.shape
    db = designs if isinstance(designs, DesignBatch) else DesignBatch(designs)
    if db.n != n:
        raise ValueError(f"design has {db.n} rows, data has {n}")
    pinv, Xp, invd, dof = db.to_device()
    if what in (WHAT_T, WHAT_BETA, WHAT_SE):
        coef = list(range(db.kmax)) if coef is None else list(coef)
        coef_d = dev(np.asarray(coef, np.int32))
        shape = (db.G, len(coef), V)
    else:
        coef_d = None
        coef = []
        shape = (db.G, n, V) if what == WHAT_RESID else (db.G, V)
    if out is None:
        out = t.empty(shape, device="cuda", dtype=t.float32)
    lib = _lib.load()
    _lib.check(lib.glm_stat(ptr(Yd), V, n, V, ptr(pinv), ptr(Xp), ptr(invd), ptr(dof), db.G, db.kmax,
                            ptr(coef_d), len(coef), what, ptr(out), V, stream_handle(stream)))
    return out


def glm_fstat(Y, designs, centre=None, stream=None):
    """Model F (G, V) with TSS around `centre` (None: each column's mean)."""
    t = require_cuda()
    Yd = dev(Y, t.float32)
    n, V = Yd.shape
    db = designs if isinstance(designs, DesignBatch) else DesignBatch(designs)
    pinv, Xp, _, dof = db.to_device()
    c = None if centre is None else dev(np.asarray([centre], np.float32))
    out = t.empty((db.G, V), device="cuda", dtype=t.float32)
    _lib.check(_lib.load().glm_fstat(ptr(Yd), V, n, V, ptr(pinv), ptr(Xp), ptr(dof), db.G, db.kmax,
                                     ptr(c), ptr(out), V, stream_handle(stream)))
    return out


class TensorCoreOperands:
    """Split-BF16 operands of the tcgen05 GLM (glm_tstat_tc): the data once,
    as per-vertex rows [V][n_pad] (hi and lo), and each batch's stacked
    pseudoinverses as [G*8][n_pad] (hi and lo)."""

    def __init__(self, Yd):
        t = require_cuda()
        self.t = t
        self.n, self.V = Yd.shape
        self.n_pad = (self.n + 31) // 32 * 32
        if self.n_pad > 640:
            raise ValueError("the tensor-core GLM holds at most 640 subjects per tile")
        self.y_hi = t.empty((self.V, self.n_pad), dtype=t.bfloat16, device="cuda")
        self.y_lo = t.empty_like(self.y_hi)
        self.lib = _lib.load()
        _lib.check(self.lib.glm_split_bf16(ptr(Yd), self.V, 1, self.V, self.n, self.n_pad, ptr(self.y_hi),
                                           ptr(self.y_lo), stream_handle()))
        self.err = t.zeros(1, dtype=t.int32, device="cuda")

    def stacked(self, db: DesignBatch):
        """Host float32 [G][8][n_pad] of the pseudoinverse rows (zero padded)."""
        P8 = np.zeros((db.G, 8, self.n_pad), np.float32)
        P8[:, :db.kmax, :db.n] = db.pinv64
        return P8

    def split(self, P8_dev, G, p_hi=None, p_lo=None):
        t = self.t
        p_hi = t.empty((G * 8, self.n_pad), dtype=t.bfloat16, device="cuda") if p_hi is None else p_hi
        p_lo = t.empty_like(p_hi) if p_lo is None else p_lo
        _lib.check(self.lib.glm_split_bf16(ptr(P8_dev), self.n_pad, 0, G * 8, self.n_pad, self.n_pad, ptr(p_hi),
                                           ptr(p_lo), stream_handle()))
        return p_hi, p_lo

    def tstat(self, p_hi, p_lo, X, invd, dof, G, kmax, coef_d, n_coef, out, ldt):
        _lib.check(self.lib.glm_tstat_tc(ptr(self.y_hi), ptr(self.y_lo), self.n, self.n_pad, self.V, ptr(p_hi),
                                         ptr(p_lo), ptr(X), ptr(invd), ptr(dof), G, kmax, ptr(coef_d), n_coef,
                                         ptr(out), ldt, ptr(self.err), stream_handle()))

    def status(self):
        e = int(self.err.item())
        if e:
            self.err.zero_()
            raise RuntimeError("tensor-core GLM: MMA completion wait ran out (device code %d)" % e)


def glm_tstat_tc(Y, designs, coef, ops=None):
    """t maps (G, n_coef, V) through the tcgen05 split-BF16 GLM."""
    t = require_cuda()
    Yd = dev(Y, t.float32)
    ops = ops or TensorCoreOperands(Yd)
    db = designs if isinstance(designs, DesignBatch) else DesignBatch(designs)
    if db.kmax > 8:
        raise ValueError("at most 8 regressors per design")
    P8 = dev(ops.stacked(db))
    p_hi, p_lo = ops.split(P8, db.G)
    _, Xp, invd, dof = db.to_device()
    coef_d = dev(np.asarray(coef, np.int32))
    out = t.empty((db.G, len(coef), ops.V), device="cuda", dtype=t.float32)
    ops.tstat(p_hi, p_lo, Xp, invd, dof, db.G, db.kmax, coef_d, len(coef), out, ops.V)
    t.cuda.synchronize()
    ops.status()
    return out
