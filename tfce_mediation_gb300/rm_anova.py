"""Repeated-measures ANCOVA of the tm-models path on the GPU: the statistics of
reg_rm_ancova_one_bs_factor / reg_rm_ancova_two_bs_factor
(tfce_mediation/pyfunc.py:2067-2280, 1712-2060) for many permutations at once,
as tmanalysis/tm_models_randomise.py:522-684 draws them.

The reference forms every effect sum of squares as a difference SS_Total - RSS
of two least-squares fits.  Each of them is the extra sum of squares of
dropping one column group S from one design D, which has the exact Wald form
b_S' inv(inv(D'D)_SS) b_S with b_S = (pinv D)_S y.  So per permutation only
the pseudoinverse rows of the S columns are needed (a handful per design); they
are packed into stacks of at most 8 rows and run through the tensor-core GLM
(glm_stat_tc mode 4: GEMM + quadratic forms, no residual pass).  The fit on
the subject dummies (SS within subjects) is the sum of squares around the
subject means; rm_anova_combine forms it and SS between subjects directly from
the permuted data rows, subtracts the error terms' effect rows exactly as the
reference does, and writes the F maps.  One tfce_sweep_batch launch then
TFCEs every map with one sign.

Row permutation.  A permuted reference call shuffles all n*s long data rows
with np.random.shuffle (after rand_array permuted the subjects' factor and
covariate rows), and because the long form is a view of the caller's array the
shuffle persists: the k-th call of a loop sees the data shuffled k times.  A
statistic is invariant under one permutation of all rows of data and designs
together, so the resident data stays in place and every design is permuted
instead (row i of the permuted design is row argsort(c)[i] of the built one,
c the cumulative shuffle)."""
from __future__ import annotations

import numpy as np

from . import _lib
from .device import dev, ptr, require_cuda, stream_handle
from .glm import TensorCoreOperands, output_program

SLOT_ROWS = 8  # pseudoinverse rows per stack (one tensor-core "design")


def dummy_code(variable, iscontinous=False, demean=True):
    """pyfunc.py:2564-2600: one column per level after the first (squeezed to
    1-D for two levels), optionally demeaned; or the variable itself
    (demeaned) when continuous."""
    variable = np.asarray(variable)
    if iscontinous:
        return variable - np.mean(variable, 0) if demean else variable
    cols = [(variable == v).astype(np.float64) for v in np.unique(variable)]
    d = np.squeeze(np.array(cols)[1:]).astype(int).T
    return d - np.mean(d, 0) if demean else d


def column_product(arr1, arr2):
    """pyfunc.py:2622-2660: every column of arr1 times every column of arr2
    (arr1-major)."""
    a1, a2 = np.asarray(arr1), np.asarray(arr2)
    if len(a1) != len(a2):
        raise ValueError("arrays must be of same length")
    if a1.ndim == 1:
        return (a1 * a2.T).T
    if a2.ndim == 1:
        return (a2 * a1.T).T
    return np.concatenate([(a1[:, i] * a2.T).T.reshape(len(a1), -1) for i in range(a1.shape[1])], axis=1)


def stack_ones(arr):
    """pyfunc.py:2662-2676."""
    return np.column_stack([np.ones(len(arr)), arr])


def _cols(a):
    return None if a is None else np.asarray(a, np.float64).reshape(len(a), -1)


def subject_groups(dmy_subjects):
    """Group label of every short row: the distinct rows of the subject
    dummies.  The fit on [1, dummies] is the fit on the group indicators only
    if the dummies span them, i.e. rank([1, dummies]) == number of groups."""
    S = np.asarray(dmy_subjects, np.float64).reshape(len(dmy_subjects), -1)
    _, labels = np.unique(S, axis=0, return_inverse=True)
    labels = labels.reshape(-1)
    n_groups = int(labels.max()) + 1
    if np.linalg.matrix_rank(stack_ones(S)) != n_groups:
        raise ValueError("dmy_subjects must dummy-code the subjects (its rows must span the subject indicators)")
    return labels, n_groups


class RMModel:
    """Designs, sums-of-squares rows and F maps of a one- or two-factor
    repeated-measures ANCOVA with n subjects and s intervals (long row
    t*n + j = subject j at interval t).

    blocks: (name, build, width, ess) -- build(f1, f2, cov) returns the long
    design whose LAST `width` columns are the block's rows; ess lists the sums
    of squares read from them as (ess name, first row, number of rows)."""

    def __init__(self, n, s, dmy_factor1, dmy_subjects, dmy_factor2=None, dmy_covariates=None):
        self.n, self.s, self.N = int(n), int(s), int(n) * int(s)
        if self.s < 2:
            raise ValueError("a repeated-measures design needs at least two intervals")
        self.two = dmy_factor2 is not None
        self.f1 = _cols(dmy_factor1)
        self.f2 = _cols(dmy_factor2)
        self.cov = _cols(dmy_covariates)
        self.A = self.f1.shape[1]
        self.B = 0 if self.f2 is None else self.f2.shape[1]
        self.AB = self.A * self.B
        self.c = 0 if self.cov is None else self.cov.shape[1]
        self.T = self.s - 1
        interval = np.concatenate([np.full(self.n, float(i)) for i in range(self.s)])
        self.iv = np.asarray(dummy_code(interval, demean=False), np.float64).reshape(self.N, -1)
        labels, self.n_groups = subject_groups(dmy_subjects)
        long_labels = np.tile(labels, self.s)
        self.gpos = np.argsort(long_labels, kind="stable").astype(np.int64)
        self.goff = np.concatenate([[0], np.cumsum(np.bincount(long_labels, minlength=self.n_groups))]).astype(
            np.int32)
        self._define()
        L = self.long_columns([None])
        for name, build, _, _ in self.blocks:
            D = np.concatenate([np.ones((1, self.N, 1))] + [x for x in build(L) if x is not None], axis=2)[0]
            if np.linalg.matrix_rank(D) < D.shape[1]:
                raise ValueError(f"the '{name}' design is rank deficient (an empty factor cell or collinear "
                                 "covariates); its sums of squares are not defined")
        self.df_b = float(self.n - 1 - self.A - self.B - self.AB - self.c)
        self.df_w = self.df_b * self.T
        if self.df_b <= 0:
            raise ValueError("no between-subject error degrees of freedom left")

    def _define(self):
        A, B, AB, c, T = self.A, self.B, self.AB, self.c, self.T
        blocks = []
        if not self.two:
            blocks.append(("a", lambda L: [L["f1"], L["cov"]], A + c, [("a", 0, A), ("cells", 0, A + c)]))
        else:
            blocks.append(("ab", lambda L: [L["f1"], L["f2"], L["cov"], L["f12"]], A + B + c + AB,
                           [("cells", 0, A + B + c + AB), ("ab", A + B + c, AB)]))
            blocks.append(("a", lambda L: [L["cov"], L["f1"]], A, [("a", 0, A)]))
            blocks.append(("b", lambda L: [L["f1"], L["cov"], L["f2"]], B, [("b", 0, B)]))
        blocks.append(("s", lambda L: [L["iv"]], T, [("s", 0, T)]))
        if c:
            blocks.append(("scov", lambda L: [L["cov"], L["iv"], L["cov_iv"]], c * T, [("scov", 0, c * T)]))
        if not self.two:
            blocks.append(("sa", lambda L: [L["iv"], L["cov"], L["cov_iv"], L["f1"], L["f1_iv"]], A * T,
                           [("sa", 0, A * T)]))
        else:
            blocks.append(("sab", lambda L: [L["f1"], L["f2"], L["f12"], L["iv"], L["f1_iv"], L["f2_iv"], L["cov"],
                                             L["cov_iv"], L["f12_iv"]], AB * T, [("sab", 0, AB * T)]))
            blocks.append(("sa", lambda L: [L["iv"], L["cov"], L["cov_iv"], L["f1"], L["f1_iv"]], A * T,
                           [("sa", 0, A * T)]))
            blocks.append(("sb", lambda L: [L["f1"], L["iv"], L["f1_iv"], L["cov"], L["cov_iv"], L["f2"],
                                            L["f2_iv"]], B * T, [("sb", 0, B * T)]))
        for name, _, w, _ in blocks:
            if w > SLOT_ROWS:
                raise ValueError(f"the '{name}' block needs {w} pseudoinverse rows (at most {SLOT_ROWS})")
        self.blocks = blocks
        if not self.two:
            self.f_maps = [("a", A, 0), ("s", T, 1), ("sa", A * T, 1)]
            self.within = ["s", "sa"] + (["scov"] if c else [])
        else:
            self.f_maps = [("a", A, 0), ("b", B, 0), ("ab", AB, 0), ("s", T, 1), ("sa", A * T, 1),
                           ("sb", B * T, 1), ("sab", AB * T, 1)]
            self.within = ["s", "sa", "sb", "sab"] + (["scov"] if c else [])
        self.between = ["cells"]
        # first-fit decreasing packing of the blocks into stacks of <= 8 rows
        order = sorted(range(len(blocks)), key=lambda i: -blocks[i][2])
        slots = []
        for i in order:
            for sl in slots:
                if sum(blocks[j][2] for j in sl) + blocks[i][2] <= SLOT_ROWS:
                    sl.append(i)
                    break
            else:
                slots.append([i])
        self.slots = [sorted(sl) for sl in slots]
        # program rows per slot: ("ess", first row in the stack, width); ESS id -> (slot, program row)
        self.slot_outputs, self.ess_at = [], {}
        for si, sl in enumerate(self.slots):
            outs, r0 = [], 0
            for bi in sl:
                _, _, w, ess = blocks[bi]
                for nm, off, width in ess:
                    self.ess_at[nm] = (si, len(outs))
                    outs.append(("ess", r0 + off, width))
                r0 += w
            self.slot_outputs.append(outs)

    def long_columns(self, ras):
        """Long-form column groups (P, N, q) of the factors / covariates with
        their subject rows permuted by ras (P, n) (None: unpermuted)."""
        P, n, s = len(ras), self.n, self.s
        idx = np.stack([np.arange(n) if ra is None else np.asarray(ra) for ra in ras])  # (P, n)

        def tile(a):
            return None if a is None else np.tile(a[idx], (1, s, 1))  # (P, N, q)

        def prod(x, y):
            return None if x is None else np.einsum("pna,pnb->pnab", x, y).reshape(P, self.N, -1)

        iv = np.broadcast_to(self.iv, (P,) + self.iv.shape)
        L = {"f1": tile(self.f1), "f2": tile(self.f2), "cov": tile(self.cov), "iv": iv}
        L["f12"] = None if self.f2 is None else prod(L["f1"], L["f2"])
        for k in ("f1", "f2", "f12", "cov"):
            L[k + "_iv"] = prod(L[k], iv)
        return L

    def slot_operands(self, ras, cums):
        """Per slot: stacked pseudoinverse rows (P, rows, N) and per-design
        weights (P, w_stride) (FP64) of the permutations given by the subject
        permutations `ras` (P entries, None = unpermuted) and the cumulative
        data-row shuffles `cums` (P, N)."""
        P = len(ras)
        inv_order = np.argsort(np.asarray(cums), axis=1)  # (P, N)
        L = self.long_columns(ras)
        per_block = {}
        for bi, (name, build, w, ess) in enumerate(self.blocks):
            parts = [np.ones((P, self.N, 1))] + [x for x in build(L) if x is not None]
            D = np.concatenate(parts, axis=2)
            Dt = D.transpose(0, 2, 1)
            inv = np.linalg.inv(Dt @ D)  # the row shuffle leaves D'D unchanged
            k = D.shape[2]
            # pseudoinverse rows of the block on the built rows, then columns in
            # the shuffled order: column i <- built row argsort(c)[i]
            rows = np.take_along_axis(inv[:, k - w:, :] @ Dt, inv_order[:, None, :], axis=2)  # (P, w, N)
            blocks_w = []
            for _, off, width in ess:
                a = k - w + off
                blocks_w.append(np.linalg.inv(inv[:, a:a + width, a:a + width]).reshape(P, width * width))
            per_block[bi] = (rows, blocks_w)
        out = []
        for sl in self.slots:
            rows = np.concatenate([per_block[bi][0] for bi in sl], axis=1)
            W = np.concatenate([wb for bi in sl for wb in per_block[bi][1]], axis=1)
            out.append((rows, W))
        return out

    def grouped_rows(self, cums):
        """(P, N) int32: data rows of every permutation grouped by subject."""
        return np.ascontiguousarray(np.asarray(cums)[:, self.gpos], np.int32)


class RMAncovaEngine:
    """F maps and TFCE null maxima of a repeated-measures ANCOVA on one GPU.

    data: long data (N = n*s, V) float32 (row t*n + j = subject j, interval t);
    model: RMModel.  Per batch of P permutations -- subject permutations ras
    (P, n) and cumulative long-row shuffles cums (P, N) -- the host forms the
    pseudoinverse rows of every effect block (FP64), one glm_stat_tc mode-4
    launch per stack of rows gives the effect sums of squares, rm_anova_combine
    the F maps, and one sweep their maxima (one sign each)."""

    def __init__(self, data, model: RMModel, adjacency=None, segments=None, H=2.0, E=1.0, vdensity=None,
                 floor_zero=False, batch=64, accumulation="component"):
        from .adjacency import AdjacencySet, to_csr
        t = require_cuda()
        self.t = t
        self.lib = _lib.load()
        self.model = model
        self.Yd = dev(np.ascontiguousarray(data, np.float32) if not isinstance(data, t.Tensor) else data, t.float32)
        self.N, self.V = self.Yd.shape
        if self.N != model.N:
            raise ValueError(f"data has {self.N} rows, the model {model.N}")
        if self.N > int(self.lib.rm_anova_max_rows()):
            raise ValueError(f"at most {int(self.lib.rm_anova_max_rows())} long rows")
        self.tc = TensorCoreOperands(self.Yd, centre=True)
        self.adj = None
        if adjacency is not None:
            if isinstance(adjacency, AdjacencySet):
                self.adj = adjacency
                self.adj.set_params(H, E)
            else:
                off, idx = to_csr(adjacency)
                seg = np.array([0, off.shape[0] - 1], np.int64) if segments is None else np.asarray(segments)
                self.adj = AdjacencySet((off, idx), H, E, seg)
            self.adj.set_accumulation(accumulation)
        self.n_seg = 1 if self.adj is None else self.adj.n_seg
        self.vd = None if vdensity is None else dev(np.asarray(vdensity, np.float32))
        self.floor_zero = bool(floor_zero)
        self.batch = int(batch)
        self.n_f = len(model.f_maps)
        self.goff_d = dev(model.goff)
        self.err = t.zeros(1, dtype=t.int32, device="cuda")
        m = model
        self._progs = [output_program(outs) for outs in m.slot_outputs]
        self._coef_d = [dev(rows.reshape(-1)) for rows, _ in self._progs]
        self._R = [len(outs) for outs in m.slot_outputs]
        names = sorted(m.ess_at, key=lambda k: m.ess_at[k])
        self._ess_names = names
        self._ess_index = {nm: i for i, nm in enumerate(names)}

    def _tables(self, P):
        """Host tables of rm_anova_combine for a batch of P (ESS buffer layout:
        slot j's rows [P][R_j][V] one after the other)."""
        m, V = self.model, self.V
        slot_off = np.concatenate([[0], np.cumsum([P * R * V for R in self._R])]).astype(np.int64)
        row_off = np.zeros(len(self._ess_names), np.int64)
        row_ps = np.zeros(len(self._ess_names), np.int64)
        for nm, (si, q) in m.ess_at.items():
            i = self._ess_index[nm]
            row_off[i] = slot_off[si] + q * V
            row_ps[i] = self._R[si] * V
        eb = np.asarray([self._ess_index[x] for x in m.between], np.int32)
        ew = np.asarray([self._ess_index[x] for x in m.within], np.int32)
        f_num = np.asarray([self._ess_index[x] for x, _, _ in m.f_maps], np.int32)
        f_err = np.asarray([e for _, _, e in m.f_maps], np.int32)
        f_df = np.asarray([d for _, d, _ in m.f_maps], np.float32)
        return int(slot_off[-1]), row_off, row_ps, eb, ew, f_num, f_err, f_df

    def fmaps(self, ras, cums, out=None, ss_out=None):
        """F maps (P, n_f, V) on the device for subject permutations `ras`
        (P entries, None = unpermuted) and cumulative long-row shuffles
        `cums` (P, N)."""
        t, m, tc = self.t, self.model, self.tc
        P = len(ras)
        cums = np.asarray(cums)
        if cums.shape != (P, self.N):
            raise ValueError("cums must be (P, N) row shuffles")
        total, row_off, row_ps, eb, ew, f_num, f_err, f_df = self._tables(P)
        ess = t.empty(max(total, 1), device="cuda", dtype=t.float32)
        base = 0
        for si, (rows, W) in enumerate(m.slot_operands(ras, cums)):
            kr = rows.shape[1]
            Gp = tc.padded(P, kr)
            P8 = np.zeros((Gp, 8, tc.n_pad), np.float32)
            P8[:P, :kr, :self.N] = rows
            U = np.zeros((Gp, kr), np.float32)
            U[:P] = rows.sum(axis=2)
            pt = tc.tile_designs(dev(P8.reshape(Gp * 8, tc.n_pad)), P, kr)
            R = self._R[si]
            view = ess[base:base + P * R * self.V].view(P, R, self.V)
            tc.stat(4, pt, dev(U), None, None, None, P, kr, self._coef_d[si], R, view, self.V,
                    wmat=dev(np.ascontiguousarray(W, np.float32)))
            base += P * R * self.V
        rows_d = dev(m.grouped_rows(cums))
        out = t.empty((P, self.n_f, self.V), device="cuda", dtype=t.float32) if out is None else out
        _lib.check(self.lib.rm_anova_combine(
            ptr(tc.Yc), self.V, self.N, self.V, ptr(rows_d), P, ptr(self.goff_d), m.n_groups, ptr(ess),
            row_off.ctypes.data, row_ps.ctypes.data, len(row_off), eb.ctypes.data, len(eb), ew.ctypes.data,
            len(ew), m.df_b, m.df_w, f_num.ctypes.data, f_err.ctypes.data, f_df.ctypes.data, len(f_num), ptr(out),
            self.V, ptr(ss_out), ptr(self.err), stream_handle()))
        return out

    def status(self):
        e = int(self.err.item())
        if e:
            self.err.zero_()
            raise RuntimeError("rm_anova_combine: a data row index or group bound was out of range")
        self.tc.status()
        if self.adj is not None:
            self.adj.status()

    def maxima(self, ras, cums):
        """TFCE null maxima (P, n_f, n_seg), one sign per map.  A batch's
        maxima are read back after the next batch is launched, so the host
        forms the next batch's designs while the GPU runs the current one."""
        t = self.t
        P = len(ras)
        res, prev = [], None

        def collect(item):
            mx, nb = item
            res.append(mx.cpu().numpy().reshape(nb, self.n_f, self.n_seg))
            self.status()

        for b in range(0, P, self.batch):
            Fm = self.fmaps(ras[b:b + self.batch], cums[b:b + self.batch])
            nb = Fm.shape[0]
            mx = t.empty(nb * self.n_f * self.n_seg, device="cuda", dtype=t.float32)
            self.adj.sweep_batch(ptr(Fm), self.V, nb * self.n_f, 1, ptr(self.vd), int(self.floor_zero), ptr(mx),
                                 None, 0, stream_handle())
            if prev is not None:
                collect(prev)
            prev = (mx, nb)
        if prev is not None:
            collect(prev)
        return np.concatenate(res) if res else np.zeros((0, self.n_f, self.n_seg), np.float32)


def long_data(data, data_format, n):
    """Long (N, V) view of the reference's data argument and (n, s):
    'short' (s, n[, V]) -> rows t*n + j; 'long' (N[, V]) with n subjects.  A
    view where numpy allows one (the reference's in-place shuffle acts on the
    caller's array through it)."""
    if data_format == "short":
        d = np.asarray(data)
        if d.ndim == 2:
            d = d[:, :, np.newaxis]
        s, n_ = d.shape[0], d.shape[1]
        return d.reshape(s * n_, d.shape[2]), n_, s
    if data_format == "long":
        d = np.asarray(data)
        d2 = d.reshape(d.shape[0], -1)
        if d2.shape[0] % n:
            raise ValueError("long data rows must be a multiple of the number of subjects")
        return d2, n, d2.shape[0] // n
    raise ValueError("data format must be short or long")
