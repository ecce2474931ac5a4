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
# typed output rows of the tensor-core GLM's programmed epilogue (glm_stat_tc mode 3)
OUT_T, OUT_NEG_T, OUT_F, OUT_AMP, OUT_ACRO, OUT_ESS = range(6)
_OUT_KIND = {"t": OUT_T, "-t": OUT_NEG_T, "f": OUT_F, "amp": OUT_AMP, "acro": OUT_ACRO, "ess": OUT_ESS}


def output_program(outputs):
    """Rows (kind, column, width, weight offset) int32 (C, 4) and the weight
    stride of a list of typed outputs:
      ("t", j) / ("-t", j): t (negated t) of coefficient j;
      ("f", j, w): partial F of the columns [j, j+w) (Wald form);
      ("ess", j, w): the extra sum of squares of the columns [j, j+w) (the
        Wald form alone: glm_stat_tc mode 4 needs no residuals for it);
      ("amp", j) / ("acro", j): cosinor amplitude / acrophase t of the
        (cos, sin) coefficient pair (j, j+1) (glm_cosinor, pyfunc.py:2406-2560).
    The model F of an intercept design with k columns is ("f", 1, k-1)."""
    rows, o = [], 0
    for spec in outputs:
        kind = _OUT_KIND.get(spec[0])
        if kind is None:
            raise ValueError(f"unknown output kind {spec[0]!r}")
        j = int(spec[1])
        if kind in (OUT_T, OUT_NEG_T):
            rows.append((kind, j, 1, 0))
        elif kind in (OUT_F, OUT_ESS):
            w = int(spec[2])
            if w < 1:
                raise ValueError("an 'f' / 'ess' row needs a width >= 1")
            rows.append((kind, j, w, o))
            o += w * w
        else:
            rows.append((kind, j, 2, o))
            o += 3
    return np.asarray(rows, np.int32).reshape(-1, 4), o


def output_columns(outputs):
    """The design columns an output program reads."""
    cols = set()
    for kind, j, w, _ in output_program(outputs)[0]:
        cols.update(range(j, j + (1 if kind in (OUT_T, OUT_NEG_T) else w)))
    return cols


class DesignBatch:
    """Stacked operators of G designs padded to kmax columns.

    designs: array (G, n, k) or list of (n, k_g) arrays (float64).
    invXX: optional (G, k, k) matrices whose diagonal gives the SE factor (the
    reference passes its own invXX to tval_int); default inv(X'X)."""

    def __init__(self, designs, invXX=None, kmax=None):
        if isinstance(designs, np.ndarray) and designs.ndim == 3:
            Xs = np.array(designs, np.float64)
            mats = None
            G, n = Xs.shape[0], Xs.shape[1]
            ks = [Xs.shape[2]] * G
        else:
            mats = [np.asarray(d, np.float64) for d in designs]
            G = len(mats)
            n = mats[0].shape[0]
            ks = [m.shape[1] for m in mats]
        kmax = kmax or max(ks)
        if kmax > 8:
            raise ValueError("at most 8 regressors per design")
        invdiag = np.zeros((G, kmax), np.float64)
        inv_p = np.zeros((G, kmax, kmax), np.float64)  # inv(X'X), zero padded
        same_k = len(set(ks)) == 1
        self._pinv64 = None
        if same_k:
            if mats is not None:
                Xs = np.stack(mats)
            k = ks[0]
            inv = np.linalg.inv(np.einsum("gsi,gsj->gij", Xs, Xs))
            # the stacked pseudoinverses are formed on first use (the
            # quadratic-form GLM does not need them)
            self._pinv_src = (inv, Xs, k)
            if k == kmax:
                Xp = Xs
            else:
                Xp = np.zeros((G, n, kmax), np.float64)
                Xp[:, :, :k] = Xs
            di = np.diagonal(inv if invXX is None else np.asarray(invXX, np.float64), axis1=1, axis2=2)
            invdiag[:, :k] = di
            inv_p[:, :k, :k] = inv
        else:
            pinv = np.zeros((G, kmax, n), np.float64)
            Xp = np.zeros((G, n, kmax), np.float64)
            for g, m in enumerate(mats):
                k = m.shape[1]
                inv = np.linalg.inv(m.T @ m)
                inv_p[g, :k, :k] = inv
                pinv[g, :k] = inv @ m.T
                Xp[g, :, :k] = m
                invdiag[g, :k] = np.diag(inv if invXX is None else np.asarray(invXX[g], np.float64))
            self._pinv64 = pinv
        self.G, self.n, self.kmax, self.ks = G, n, kmax, ks
        self.X64, self.invdiag64 = Xp, invdiag
        self._inv64 = inv_p
        self.dof = np.asarray([n - k for k in ks], np.float64)

    @property
    def pinv64(self):
        """(G, kmax, n) pinv(X_d) = inv(X'X) X' per design (zero padded), FP64."""
        if self._pinv64 is None:
            inv, Xs, k = self._pinv_src
            pinv = np.zeros((self.G, self.kmax, self.n), np.float64)
            pinv[:, :k, :] = np.einsum("gij,gsj->gis", inv, Xs)
            self._pinv64 = pinv
        return self._pinv64

    def inverse(self):
        """(G, kmax, kmax) inv(X'X) per design (zero padded), FP64."""
        return self._inv64

    def group_blocks(self, groups):
        """(G, sum w^2) float32: per design, inv(inv(X'X)_SS) of every column
        group S = (start, width), row-major, concatenated -- the Wald form of
        the extra sum of squares of dropping S."""
        return self.program_weights([("f", s0, w) for s0, w in groups])

    def program_weights(self, outputs, out=None):
        """(G, w_stride) float32 per-design weights of an output program
        (output_program): inv(inv(X'X)_SS) for an 'f' row, the inv(X'X)
        entries (jj, j j+1, j+1 j+1) for an 'amp' / 'acro' row; written into
        `out` (G, w_stride) when given."""
        rows, stride = output_program(outputs)
        inv = self.inverse()
        w64 = np.zeros((self.G, stride), np.float64)
        for kind, j, w, o in rows:
            if j < 0 or j + w > self.kmax:
                continue  # outside the designs: the kernel returns NaN for the row
            if kind in (OUT_F, OUT_ESS):
                w64[:, o:o + w * w] = np.linalg.inv(inv[:, j:j + w, j:j + w]).reshape(self.G, w * w)
            elif kind in (OUT_AMP, OUT_ACRO):
                w64[:, o], w64[:, o + 1], w64[:, o + 2] = inv[:, j, j], inv[:, j, j + 1], inv[:, j + 1, j + 1]
        if out is None:
            return w64.astype(np.float32)
        out[...] = w64
        return out

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


def glm_stat_f64(Y, designs, what=WHAT_T, coef=None, stream=None):
    """t (what=WHAT_T), betas or SE of every design in FP64 with the
    reference's precision (glm_stat_f64: double betas and sigma^2, SE rounded
    to float32 as se_of_slope stores it, t = beta / SE); a CUDA float64 tensor
    (G, n_coef, V).  Used for the observed statistic and the one-off helpers,
    where the map is compared with the reference's own."""
    t = require_cuda()
    if what not in (WHAT_T, WHAT_BETA, WHAT_SE):
        raise ValueError("glm_stat_f64 computes t, betas or SE")
    Yd = dev(Y, t.float32)
    n, V = Yd.shape
    db = designs if isinstance(designs, DesignBatch) else DesignBatch(designs)
    if db.n != n:
        raise ValueError(f"design has {db.n} rows, data has {n}")
    coef = list(range(db.kmax)) if coef is None else list(coef)
    out = t.empty((db.G, len(coef), V), device="cuda", dtype=t.float64)
    # the operands stay referenced until the launch is queued (a temporary's
    # memory goes back to the caching allocator as soon as it is released)
    pinv, Xd, invd, dof = (dev(a, t.float64) for a in (db.pinv64, db.X64, db.invdiag64, db.dof))
    coef_d = dev(np.asarray(coef, np.int32))
    _lib.check(_lib.load().glm_stat_f64(ptr(Yd), V, n, V, ptr(pinv), ptr(Xd), ptr(invd), ptr(dof), db.G, db.kmax,
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
    """Operands of the tensor-core GLM (glm_tstat_tc).

    The data is centred per vertex (FP64 mean), split into BF16 hi/lo and
    pre-tiled once (128-vertex row blocks of Y', 16-subject K steps).  Per
    design batch: the stacked pseudoinverse rows [G_pad*8][n_pad] (tiled on
    the device), u = pinv(X_d).1 [G_pad][kmax] (restores the betas of the
    uncentred data) and the negated design rows [G_pad/DB][n_sc][kmax][DB]
    for the residual epilogue.

    The quadratic form (glm_tstat_tc_qf) serves t of coefficients >= 1 of
    designs whose first column is all ones: its operands are the centred
    design columns [G_pad*R][n_pad] (tiled on the device) and inv(Xc'Xc)
    [G_pad][k-1][k-1], with the data's centred sum of squares yy [V] kept
    beside the tiles."""

    ROW_BLOCK = 128

    def __init__(self, Yd, centre=True):
        t = require_cuda()
        self.t = t
        self.lib = _lib.load()
        self.Yd = Yd
        self.n, self.V = Yd.shape
        self.n_pad = (self.n + 15) // 16 * 16
        self.n_sc = (self.n + 31) // 32 * 32
        nbytes = int(self.lib.glm_tile_bytes(self.V, self.ROW_BLOCK, self.n_pad))
        self.yt = t.empty(nbytes, dtype=t.uint8, device="cuda")
        self.shift = t.empty(self.V, dtype=t.float32, device="cuda") if centre else None
        # the data minus its centre: residuals of intercept designs skip the intercept term
        self.Yc = t.empty_like(Yd) if centre else None
        self.yy = t.empty(self.V, dtype=t.float32, device="cuda") if centre else None
        self.err = t.zeros(1, dtype=t.int32, device="cuda")
        # t of coefficients >= 1 of intercept designs through the quadratic
        # form (False: the residual epilogue; the autotuner times both)
        self.quadratic_form = True
        # designs per tile: None = the library's default for kmax (32 for kmax <= 5, else 16);
        # 16 or 32 to choose (the autotuner times both)
        self.design_block = None
        self.retile()

    def retile(self):
        """Centre, split and tile the resident data again (after new data was copied in)."""
        if self.shift is not None:
            _lib.check(self.lib.glm_col_mean(ptr(self.Yd), self.V, self.n, self.V, ptr(self.shift),
                                             stream_handle()))
        # tiles of the centred data, and the centred FP32 copy in the same pass
        _lib.check(self.lib.glm_tile_split(ptr(self.Yd), self.V, 1, self.V, self.n, ptr(self.shift),
                                           self.ROW_BLOCK, self.n_pad, ptr(self.yt), ptr(self.Yc), stream_handle()))
        if self.yy is not None:
            _lib.check(self.lib.glm_col_sumsq(ptr(self.Yc), self.V, self.n, self.V, ptr(self.yy), stream_handle()))

    def block(self, kmax):
        if self.design_block is not None and (kmax <= 5 or self.design_block == 16):
            return int(self.design_block)
        return int(self.lib.glm_tc_design_block(kmax))

    def padded(self, G, kmax):
        DB = self.block(kmax)
        return (G + DB - 1) // DB * DB

    def centred_ok(self, db: DesignBatch, first_column_used=False):
        """Whether the centred residual form applies: a centred data copy
        exists, every design's first column is all ones, and no requested
        output uses coefficient 0."""
        return self.Yc is not None and not first_column_used and bool(np.all(db.X64[:, :, 0] == 1.0))

    def qf_ok(self, db: DesignBatch, coef):
        """Whether the quadratic form serves t of `coef` for these designs:
        centred data, every design's first column all ones, kmax in [2, 8]
        and no coefficient 0 (designs with fewer columns are zero padded:
        their missing columns get zero cross products and inverse rows)."""
        return (self.quadratic_form and self.yy is not None and 2 <= db.kmax <= 8 and 1 <= len(coef) <= 8
                and min(int(c) for c in coef) >= 1 and self.centred_ok(db))

    def qf_rows(self, kmax):
        return 4 if kmax <= 5 else 8

    def qf_padded(self, G, kmax):
        DB = int(self.lib.glm_qf_design_block(kmax))
        return (G + DB - 1) // DB * DB

    def host_operands_qf(self, db: DesignBatch, XR=None, GI=None):
        """Host float32 operands of the quadratic form: the centred design
        columns 1..k-1 stacked [G_pad*R][n_pad] (design d, column j at row
        d*R + j - 1) and inv(Xc'Xc) = inv(X'X)[1:, 1:] zero padded to
        [G_pad][R][R]; written into XR / GI when given (e.g. pinned buffers of
        those sizes)."""
        G, k, n = db.G, db.kmax, db.n
        R, Gp = self.qf_rows(k), self.qf_padded(G, k)
        xr = np.zeros((Gp, R, self.n_pad), np.float32) if XR is None else XR.reshape(Gp, R, self.n_pad)
        gi = np.zeros((Gp, R, R), np.float32) if GI is None else GI.reshape(Gp, R, R)
        if XR is not None:
            xr[...] = 0.0
            gi[...] = 0.0
        xc = db.X64[:, :, 1:] - db.X64[:, :, 1:].mean(axis=1, keepdims=True)
        xr[:G, :k - 1, :n] = xc.transpose(0, 2, 1)
        gi[:G, :k - 1, :k - 1] = db.inverse()[:, 1:, 1:]
        return xr.reshape(Gp * R, self.n_pad), gi

    def tile_designs_qf(self, XR_dev, G, kmax, out=None):
        """Device tiles of the stacked centred design columns XR_dev (G_pad*R, n_pad)."""
        t = self.t
        rows = self.qf_padded(G, kmax) * self.qf_rows(kmax)
        nbytes = int(self.lib.glm_tile_bytes(rows, 256, self.n_pad))
        out = t.empty(nbytes, dtype=t.uint8, device="cuda") if out is None else out
        _lib.check(self.lib.glm_tile_split(ptr(XR_dev), self.n_pad, 0, rows, self.n_pad, None, 256, self.n_pad,
                                           ptr(out), None, stream_handle()))
        return out

    def tstat_qf(self, x_tiles, ginv, invd, dof, G, kmax, coef_d, n_coef, out, ldt):
        _lib.check(self.lib.glm_tstat_tc_qf(ptr(self.yt), ptr(self.yy), self.n, self.n_pad, self.V, ptr(x_tiles),
                                            ptr(ginv), ptr(invd), ptr(dof), G, kmax, ptr(coef_d), n_coef, ptr(out),
                                            ldt, ptr(self.err), stream_handle()))

    def host_operands(self, db: DesignBatch, P8=None, U=None, Xt=None, centred=False):
        """Host float32 operands of a DesignBatch: stacked pseudoinverse rows
        (G_pad*8, n_pad), u = pinv.1 (G_pad, kmax) and negated design rows
        (G_pad/DB, n_sc, kmax, DB) -- with `centred`, the columns after the
        first minus their means and the first column zero; written into P8 /
        U / Xt when given (e.g. pinned buffers of exactly those sizes)."""
        G, kmax, n = db.G, db.kmax, db.n
        DB = self.block(kmax)
        Gp = self.padded(G, kmax)
        p = np.zeros((Gp, 8, self.n_pad), np.float32) if P8 is None else P8.reshape(Gp, 8, self.n_pad)
        if P8 is not None:
            p[...] = 0.0
        p[:G, :kmax, :n] = db.pinv64
        u = np.zeros((Gp, kmax), np.float32) if U is None else U.reshape(Gp, kmax)
        u[...] = 0.0
        u[:G] = db.pinv64.sum(axis=2)
        x = np.zeros((Gp // DB, self.n_sc, kmax, DB), np.float32) if Xt is None else \
            Xt.reshape(Gp // DB, self.n_sc, kmax, DB)
        xg = np.zeros((Gp, self.n_sc, kmax), np.float32)
        if centred:
            xc = db.X64[:, :, 1:] - db.X64[:, :, 1:].mean(axis=1, keepdims=True)
            xg[:G, :n, 1:] = -xc
        else:
            xg[:G, :n] = -db.X64
        x[...] = xg.reshape(Gp // DB, DB, self.n_sc, kmax).transpose(0, 2, 3, 1)
        return p.reshape(Gp * 8, self.n_pad), u, x

    def tile_designs(self, P8_dev, G, kmax, out=None):
        """Device tiles of stacked pseudoinverse rows P8_dev (G_pad*8, n_pad)."""
        t = self.t
        rows = self.padded(G, kmax) * 8
        rb = self.block(kmax) * 8
        nbytes = int(self.lib.glm_tile_bytes(rows, rb, self.n_pad))
        out = t.empty(nbytes, dtype=t.uint8, device="cuda") if out is None else out
        _lib.check(self.lib.glm_tile_split(ptr(P8_dev), self.n_pad, 0, rows, self.n_pad, None, rb, self.n_pad,
                                           ptr(out), None, stream_handle()))
        return out

    def tstat(self, p_tiles, u_rows, x_rows, invd, dof, G, kmax, coef_d, n_coef, out, ldt):
        self.stat(0, p_tiles, u_rows, x_rows, invd, dof, G, kmax, coef_d, n_coef, out, ldt)

    def stat(self, mode, p_tiles, u_rows, x_rows, invd, dof, G, kmax, coef_d, n_coef, out, ldt, wmat=None,
             centred=False):
        """mode 0: t of coefficients coef_d; 1: RSS; 2: partial F of the column
        groups coef_d = (start, width) pairs, wmat from DesignBatch.group_blocks;
        3: output program rows coef_d (output_program), wmat from
        DesignBatch.program_weights.
        centred: x_rows came from host_operands(..., centred=True)."""
        w_stride = 0 if wmat is None else int(wmat.shape[-1])
        _lib.check(self.lib.glm_stat_tc_block(ptr(self.yt), ptr(self.shift), ptr(self.Yd),
                                              ptr(self.Yc) if centred else None, self.V, self.n, self.n_pad,
                                              self.V, ptr(p_tiles), ptr(u_rows), ptr(x_rows), self.n_sc, ptr(invd),
                                              ptr(dof), G, kmax, self.block(kmax), mode, ptr(coef_d), n_coef,
                                              ptr(wmat), w_stride, ptr(out), ldt, ptr(self.err), stream_handle()))

    def status(self):
        e = int(self.err.item())
        if e:
            self.err.zero_()
            raise RuntimeError("tensor-core GLM: a copy or MMA completion wait ran out (device code %d)" % e)


def glm_tstat_tc(Y, designs, coef, ops=None, centre=True, quadratic_form=None):
    """t maps (G, n_coef, V) through the tcgen05 split-BF16 GLM: the quadratic
    form (glm_tstat_tc_qf) where it applies and quadratic_form is not False
    (None: the operands' setting), else the residual epilogue (glm_tstat_tc)."""
    t = require_cuda()
    db = designs if isinstance(designs, DesignBatch) else DesignBatch(designs)
    ops = ops or TensorCoreOperands(dev(Y, t.float32), centre=centre)
    keep = ops.quadratic_form
    if quadratic_form is not None:
        ops.quadratic_form = bool(quadratic_form)
    try:
        use_qf = ops.qf_ok(db, coef)
    finally:
        ops.quadratic_form = keep
    if use_qf:
        XR, GI = ops.host_operands_qf(db)
        xt = ops.tile_designs_qf(dev(XR), db.G, db.kmax)
        out = t.empty((db.G, len(coef), ops.V), device="cuda", dtype=t.float32)
        ops.tstat_qf(xt, dev(GI), dev(db.invdiag64.astype(np.float32)), dev(db.dof.astype(np.float32)), db.G,
                     db.kmax, dev(np.asarray(coef, np.int32)), len(coef), out, ops.V)
        t.cuda.synchronize()
        ops.status()
        return out
    centred = ops.centred_ok(db, first_column_used=0 in list(coef))
    P8, U, Xt = ops.host_operands(db, centred=centred)
    pt = ops.tile_designs(dev(P8), db.G, db.kmax)
    u, xt = dev(U), dev(Xt)
    invd = dev(db.invdiag64.astype(np.float32))
    dof = dev(db.dof.astype(np.float32))
    coef_d = dev(np.asarray(coef, np.int32))
    out = t.empty((db.G, len(coef), ops.V), device="cuda", dtype=t.float32)
    ops.stat(0, pt, u, xt, invd, dof, db.G, db.kmax, coef_d, len(coef), out, ops.V, centred=centred)
    t.cuda.synchronize()
    ops.status()
    return out


def glm_stat_tc(Y, designs, mode, coef=None, groups=None, ops=None, outputs=None):
    """Tensor-core GLM outputs for a DesignBatch: mode 't' -> (G, len(coef), V)
    t maps; 'rss' -> (G, V) residual sums of squares; 'f' -> (G, len(groups), V)
    partial F of the column groups [(start, width), ...] (glm_typeI's drop-one
    F, tm/pyfunc.py:2282-2400); 'program' -> (G, len(outputs), V) typed output
    rows (output_program)."""
    t = require_cuda()
    db = designs if isinstance(designs, DesignBatch) else DesignBatch(designs)
    ops = ops or TensorCoreOperands(dev(Y, t.float32))
    uses0 = ((mode == "t" and 0 in list(coef)) or (mode == "f" and min(s0 for s0, _ in groups) < 1)
             or (mode == "program" and 0 in output_columns(outputs)))
    centred = ops.centred_ok(db, first_column_used=uses0)
    P8, U, Xt = ops.host_operands(db, centred=centred)
    pt = ops.tile_designs(dev(P8), db.G, db.kmax)
    u, xt = dev(U), dev(Xt)
    invd = dev(db.invdiag64.astype(np.float32))
    dof = dev(db.dof.astype(np.float32))
    wmat = None
    if mode == "t":
        m, rows, coef_d = 0, len(coef), dev(np.asarray(coef, np.int32))
    elif mode == "rss":
        m, rows, coef_d = 1, 1, None
    elif mode == "f":
        m, rows = 2, len(groups)
        coef_d = dev(np.asarray(groups, np.int32).reshape(-1))
        wmat = dev(db.group_blocks(groups))
    elif mode == "program":
        rows_i, stride = output_program(outputs)
        m, rows, coef_d = 3, len(outputs), dev(rows_i.reshape(-1))
        wmat = dev(db.program_weights(outputs)) if stride else None
    else:
        raise ValueError("mode must be 't', 'rss', 'f' or 'program'")
    out = t.empty((db.G, rows, ops.V), device="cuda", dtype=t.float32)
    ops.stat(m, pt, u, xt, invd, dof, db.G, db.kmax, coef_d, rows, out, ops.V, wmat=wmat, centred=centred)
    t.cuda.synchronize()
    ops.status()
    return out[:, 0] if mode == "rss" else out
