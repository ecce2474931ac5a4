"""Batched permutation engine: the GB300 form of the reference's randomise loops
(tfce_mediation/tmanalysis/vertex_tfce_multiple_regression_randomise.py:90-117,
voxel_tfce_multiple_regression_randomise.py:95-118,
vertex_tfce_mediation_randomise.py:79-91,
tfce_mediation/tm_func.py:144-185 and 269-305).

Per launch, P permutations:
  1. host: permutation indices RandomState(seed + p).permutation(n) and, in
     float64, each permuted design's inv(X'X) X' and diag(inv(X'X));
  2. device: one GLM launch -> t maps [P][C][V] (float32, resident): the
     tcgen05 split-BF16 GEMM with the fused residual epilogue (precision
     'bf16x3', default) or the FP32 CUDA-core kernel ('fp32'); with
     `outputs` / `f_groups` the epilogue's programmed rows instead (partial F,
     cosinor amplitude / acrophase t, +/- t), swept with one sign;
  3. device: one tfce_sweep_batch launch over P x C maps x (+,-) x segments
     -> the scaled per-segment maximum of every sweep;
  4. host: max over segments (hemispheres) gives the reference's per-permutation
     CSV values (2 per contrast: + then -).
Y stays resident in HBM for the whole run; per launch only the P design
operators go up and P x C x 2 x S maxima come down.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .adjacency import AdjacencySet, is_symmetric, locality_order, relabel_csr, to_csr
from .device import dev, ptr, require_cuda, stream_handle
from .glm import OUT_NEG_T, OUT_T, DesignBatch, TensorCoreOperands, output_columns, output_program


def permutations(n, seed, start, stop):
    """Index streams of the mmr-lr convention (tm_func.py:147-151): row p is
    numpy.random.RandomState(seed + p).permutation(n), generated by the
    native library (perm_stream, bit-identical to numpy's)."""
    if stop <= start:
        return np.zeros((0, n), np.int64)
    out = np.empty((stop - start, n), np.int64)
    _lib.check(_lib.load().perm_stream(int(n), int(seed), int(start), int(stop),
                                       out.ctypes.data_as(ctypes.c_void_p), 0))
    return out


class PermutationEngine:
    """Mass-univariate GLM + TFCE null distribution on one GPU.

    Y: (n, V) float32 data (subjects x vertices, concatenated segments).
    batch: permutations per launch, or "auto" (timed candidates, cached;
    tfce_mediation_gb300.autotune).
    pred_x: (n, k-1) regressors; the design is [1, pred_x] (randomise :88).
    adjacency: (offsets, indices) CSR over V, or an AdjacencySet.
    segments: vertex offsets of the segments (hemispheres / surfaces).
    contrasts: coefficient indices to test (default 1..k-1: every
    non-intercept column, randomise :113-117).
    floor_zero: the segment maxima count the zero fill of masked vertices
    (vertex path: the statistic is scattered into zero-filled hemispheres).
    accumulation: 'component' (default; per-component double sums, within
    ~1e-7 of the reference's float sums) or 'exact' (the reference's float
    arithmetic, bit-identical; slower).
    f_groups: [(start, width), ...] column groups of the design: the maps are
    then the drop-one F of each group (glm_typeI's F per variable,
    tm/pyfunc.py:2282-2400, as tm_models_randomise.py:205-210 permutes it),
    swept with one sign; needs precision 'bf16x3'.  Shorthand for
    outputs=[("f", start, width), ...].
    outputs: typed output maps of the tensor-core GLM's programmed epilogue
    (glm.output_program: ("t", j), ("-t", j), ("f", j, w), ("amp", j),
    ("acro", j)), each swept with one sign -- e.g. the cosinor path's model F,
    amplitude and acrophase t and +/- t of the other regressors
    (tm_models_randomise.py:274-372); needs precision 'bf16x3'.
    precision: GLM arithmetic of the permutation t maps: 'bf16x3' (default;
    tensor cores, split BF16 with FP32 accumulation, t within ~3e-5 relative
    of FP64) or 'fp32' (CUDA cores, ~1e-6).  The observed (unpermuted) t map
    always uses 'fp32'.
    threshold_groups: one group id per segment, or None.  Segments of one
    group share one threshold table per map and sign, from the largest of
    their maxima: the sweep of one merged adjacency over several surfaces
    (tm_func.calculate_tfce, tm_func.py:54-123: dT = the merged image's
    max / 100) or of one TFCE setting's surfaces (calc_mixed_tfce,
    tm_func.py:327-378); each segment is still scaled by its own max / 100.
    None: every segment its own table (the hemispheres of the vertex path,
    the surfaces of mmr-lr).
    reorder: renumber vertices inside every segment for memory locality
    (reverse Cuthill-McKee); Y's columns are permuted once here and every map
    handed back is in the caller's order.  Only symmetric adjacency is
    renumbered (for one-way entries the tie rule depends on vertex order), so
    results do not depend on it."""

    def __init__(self, Y, pred_x, adjacency, segments=None, H=2.0, E=1.0, vdensity=None,
                 contrasts=None, floor_zero=False, batch=64, signs=2, reorder=False,
                 accumulation="component", precision="bf16x3", f_groups=None, outputs=None,
                 threshold_groups=None):
        t = require_cuda()
        if precision not in ("bf16x3", "fp32"):
            raise ValueError("precision must be 'bf16x3' (tensor cores) or 'fp32' (CUDA cores)")
        self.precision = precision
        self.f_groups = None if f_groups is None else [(int(a), int(b)) for a, b in f_groups]
        if self.f_groups is not None:
            if outputs is not None:
                raise ValueError("give f_groups or outputs, not both")
            outputs = [("f", s0, w) for s0, w in self.f_groups]
        self.outputs = None if outputs is None else [tuple(o) for o in outputs]
        if self.outputs is not None:
            if precision != "bf16x3":
                raise ValueError("programmed output maps run on the tensor-core GLM (precision='bf16x3')")
            signs = 1
        self.t = t
        Yh = Y if isinstance(Y, t.Tensor) else np.asarray(Y, np.float32)
        V = Yh.shape[1]
        self.order = None
        if isinstance(adjacency, AdjacencySet):
            self.adj = adjacency
            self.adj.set_params(H, E)
        else:
            off, idx = to_csr(adjacency)
            seg = np.array([0, off.shape[0] - 1], np.int64) if segments is None else np.asarray(segments)
            if reorder and off.shape[0] - 1 == V and is_symmetric(off, idx):
                self.order = locality_order(off, idx, seg)
                off, idx = relabel_csr(off, idx, self.order)
            self.adj = AdjacencySet((off, idx), H, E, seg)
        if self.order is not None:
            order_t = t.from_numpy(self.order)
            Yh = (Yh[:, order_t] if isinstance(Yh, t.Tensor) else Yh[:, self.order])
            if vdensity is not None:
                vdensity = np.asarray(vdensity, np.float32)[self.order]
        self.Yd = dev(Yh, t.float32)
        self.n, self.V = self.Yd.shape
        px = np.asarray(pred_x, np.float64)
        self.X = np.column_stack([np.ones(self.n), px.reshape(self.n, -1)])
        self.k = self.X.shape[1]
        if self.adj.n_vertices != self.V:
            raise ValueError(f"adjacency has {self.adj.n_vertices} vertices, data {self.V}")
        self.adj.set_accumulation(accumulation)
        self.n_seg = self.adj.n_seg
        if threshold_groups is not None:
            self.adj.set_threshold_groups(threshold_groups)
        self.contrasts = list(range(1, self.k)) if contrasts is None else list(contrasts)
        self._w_stride = 0
        if self.f_groups is not None:
            for s0, w in self.f_groups:
                if s0 < 1 or w < 1 or s0 + w > self.k:
                    raise ValueError(f"column group ({s0}, {w}) outside the design's {self.k} columns")
        if self.outputs is not None:
            prog, self._w_stride = output_program(self.outputs)
            for kind, j, w, _ in prog:
                last = j + (0 if kind in (OUT_T, OUT_NEG_T) else w - 1)
                if j < 0 or last >= self.k:
                    raise ValueError(f"output {tuple(int(x) for x in (kind, j, w))} outside the design's "
                                     f"{self.k} columns")
            self.contrasts = list(range(len(self.outputs)))
        self.C = len(self.contrasts)
        self.signs = signs
        self.floor_zero = bool(floor_zero)
        self.vd = None if vdensity is None else dev(np.asarray(vdensity, np.float32))
        self.lib = _lib.load()
        self._coef = dev(np.asarray(self.contrasts, np.int32) if self.outputs is None
                         else output_program(self.outputs)[0].reshape(-1))
        self._tc = TensorCoreOperands(self.Yd) if precision == "bf16x3" else None
        # the designs [1, pred_x] have an intercept: the tensor-core residuals
        # use the centred form unless an output needs coefficient 0
        uses0 = (0 in self.contrasts) if self.outputs is None else 0 in output_columns(self.outputs)
        self._centred = self._tc is not None and self._tc.Yc is not None and not uses0
        if batch == "auto":
            from .autotune import choose_batch
            batch = choose_batch(self)
        self.batch = int(batch)
        self._alloc_buffers()

    def _alloc_buffers(self):
        t = self.t
        self._tbuf = t.empty((self.batch, self.C, self.V), device="cuda", dtype=t.float32)
        self._maxbuf = t.empty((self.batch, self.C, self.signs, self.n_seg), device="cuda",
                               dtype=t.float32)
        self._host_max = t.empty((self.batch, self.C, self.signs, self.n_seg), dtype=t.float32,
                                 pin_memory=True)

    # -- device steps -------------------------------------------------------
    def _designs(self, perms):
        return DesignBatch(self.X[perms])

    def tmaps(self, designs: DesignBatch, out=None, precision=None):
        """t maps [G][C][V] for a DesignBatch (device tensor)."""
        G = designs.G
        out = self._tbuf[:G] if out is None else out
        if (precision or self.precision) == "bf16x3":
            tc = self._tc if self._tc is not None else TensorCoreOperands(self.Yd)
            self._tc = tc
            if self.outputs is None and tc.qf_ok(designs, self.contrasts):
                XR, GI = tc.host_operands_qf(designs)
                xt = tc.tile_designs_qf(dev(XR), G, designs.kmax)
                tc.tstat_qf(xt, dev(GI), dev(designs.invdiag64.astype(np.float32)),
                            dev(designs.dof.astype(np.float32)), G, designs.kmax, self._coef, self.C, out, self.V)
                return out
            centred = self._centred and tc.centred_ok(designs)
            P8, U, Xt = tc.host_operands(designs, centred=centred)
            pt = tc.tile_designs(dev(P8), G, designs.kmax)
            mode, wmat = 0, None
            if self.outputs is not None:
                mode = 3
                wmat = dev(designs.program_weights(self.outputs)) if self._w_stride else None
            tc.stat(mode, pt, dev(U), dev(Xt), dev(designs.invdiag64.astype(np.float32)),
                    dev(designs.dof.astype(np.float32)), G, designs.kmax, self._coef, self.C, out, self.V,
                    wmat=wmat, centred=centred)
            return out
        pinv, Xp, invd, dof = designs.to_device()
        _lib.check(self.lib.glm_tstat(ptr(self.Yd), self.V, self.n, self.V, ptr(pinv), ptr(Xp),
                                      ptr(invd), ptr(dof), G, designs.kmax, ptr(self._coef),
                                      self.C, ptr(out), self.V, stream_handle()))
        return out

    def sweep_max(self, maps, n_maps, out=None):
        """Scaled per-segment TFCE maxima of n_maps maps (device tensor
        [n_maps][signs][n_seg])."""
        out = self._maxbuf.view(-1)[: n_maps * self.signs * self.n_seg] if out is None else out
        self.adj.sweep_batch(ptr(maps), self.V, n_maps, self.signs, ptr(self.vd),
                             int(self.floor_zero), ptr(out), None, 0, stream_handle())
        return out

    def upload(self, Y_host):
        """Copy new data (n, V) in the caller's vertex order into the resident
        buffer (pinned host memory makes this asynchronous)."""
        t = self.t
        if self.order is not None:
            if not hasattr(self, "_order_d"):
                self._order_d = t.from_numpy(self.order).cuda()
            staged = getattr(self, "_stage", None)
            if staged is None or staged.shape != self.Yd.shape:
                self._stage = staged = t.empty_like(self.Yd)
            staged.copy_(Y_host, non_blocking=True)
            t.index_select(staged, 1, self._order_d, out=self.Yd)
        else:
            self.Yd.copy_(Y_host, non_blocking=True)
        if self._tc is not None:
            self._tc.retile()

    def status(self):
        """Raise if a device wait of the last launches ran out (sweep or GLM)."""
        self.adj.status()
        if self._tc is not None:
            self._tc.status()

    def run_batch(self, perms):
        """Maxima (P, C, signs, n_seg) for the permutation index rows `perms`."""
        P = perms.shape[0]
        if P > self.batch:
            raise ValueError("batch larger than the engine's buffers")
        tm = self.tmaps(self._designs(perms))
        mx = self.sweep_max(tm, P * self.C)
        hm = self._host_max.view(-1)[: mx.numel()]
        hm.copy_(mx, non_blocking=True)
        self.t.cuda.current_stream().synchronize()
        self.status()
        return hm.numpy().reshape(P, self.C, self.signs, self.n_seg).copy()

    def run(self, n_perm=None, seed=0, start=0, stop=None, perms=None):
        """Null maxima for permutations [start, stop) of the seeded stream (or
        explicit index rows `perms`): array (n_perm, C, signs, n_seg)."""
        if perms is None:
            stop = start + n_perm if stop is None else stop
            perms = permutations(self.n, seed, start, stop)
        out = []
        for b in range(0, perms.shape[0], self.batch):
            out.append(self.run_batch(perms[b:b + self.batch]))
        return np.concatenate(out) if out else np.zeros((0, self.C, self.signs, self.n_seg), np.float32)

    # -- CUDA-graph path ----------------------------------------------------
    def _graph_qf(self):
        """Whether the captured batches run the quadratic-form GLM: t of
        coefficients >= 1 of the intercept designs [1, pred_x], no output
        program, and the operands' setting on."""
        tc = self._tc
        return (tc is not None and self.outputs is None and self._centred and tc.quadratic_form
                and tc.yy is not None and 2 <= self.k <= 8 and min(self.contrasts) >= 1)

    def _graph_slot(self, P):
        """One captured batch: pinned design operators -> device, glm_tstat,
        the sweep (counter reset included), maxima -> pinned host memory."""
        t = self.t
        n, kmax = self.n, self.k
        tc = self._tc
        slot = {"P": P}
        qf = self._graph_qf()
        slot["QF"] = qf
        if qf:
            R, Gp = tc.qf_rows(kmax), tc.qf_padded(P, kmax)
            keys = ("XR", "GI", "invd", "dof")
            slot["h_XR"] = t.zeros((Gp * R, tc.n_pad), dtype=t.float32, pin_memory=True)
            slot["h_GI"] = t.zeros((Gp, R, R), dtype=t.float32, pin_memory=True)
            slot["d_xt"] = t.empty(int(self.lib.glm_tile_bytes(Gp * R, 256, tc.n_pad)), dtype=t.uint8,
                                   device="cuda")
        elif tc is not None:
            Gp, DB = tc.padded(P, kmax), tc.block(kmax)
            slot["DB"] = DB
            keys = ("P8", "U", "Xt", "invd", "dof") + (("W",) if self._w_stride else ())
            if self._w_stride:
                slot["h_W"] = t.zeros((P, self._w_stride), dtype=t.float32, pin_memory=True)
            slot["h_P8"] = t.zeros((Gp * 8, tc.n_pad), dtype=t.float32, pin_memory=True)
            slot["h_U"] = t.zeros((Gp, kmax), dtype=t.float32, pin_memory=True)
            slot["h_Xt"] = t.zeros((Gp // DB, tc.n_sc, kmax, DB), dtype=t.float32, pin_memory=True)
            slot["d_pt"] = t.empty(int(self.lib.glm_tile_bytes(Gp * 8, DB * 8, tc.n_pad)), dtype=t.uint8,
                                   device="cuda")
        else:
            keys = ("pinv", "X", "invd", "dof")
            slot["h_pinv"] = t.zeros((P, kmax, n), dtype=t.float32, pin_memory=True)
            slot["h_X"] = t.zeros((P, n, kmax), dtype=t.float32, pin_memory=True)
        # the capture warm-up runs on these before the first fill: a harmless design
        slot["h_invd"] = t.ones((P, kmax), dtype=t.float32, pin_memory=True)
        slot["h_dof"] = t.ones((P,), dtype=t.float32, pin_memory=True)
        slot["h_max"] = t.empty((P, self.C, self.signs, self.n_seg), dtype=t.float32, pin_memory=True)
        for key in keys:
            slot["d_" + key] = t.empty(slot["h_" + key].shape, device="cuda", dtype=t.float32)
        slot["d_t"] = t.empty((P, self.C, self.V), device="cuda", dtype=t.float32)
        slot["d_max"] = t.empty((P, self.C, self.signs, self.n_seg), device="cuda", dtype=t.float32)

        def body_glm():
            for key in keys:
                slot["d_" + key].copy_(slot["h_" + key], non_blocking=True)
            if qf:
                tc.tile_designs_qf(slot["d_XR"], P, kmax, out=slot["d_xt"])
                tc.tstat_qf(slot["d_xt"], slot["d_GI"], slot["d_invd"], slot["d_dof"], P, kmax, self._coef, self.C,
                            slot["d_t"], self.V)
            elif tc is not None:
                tc.tile_designs(slot["d_P8"], P, kmax, out=slot["d_pt"])
                tc.stat(3 if self.outputs is not None else 0, slot["d_pt"], slot["d_U"], slot["d_Xt"],
                        slot["d_invd"], slot["d_dof"], P, kmax, self._coef, self.C, slot["d_t"], self.V,
                        wmat=slot.get("d_W"), centred=self._centred)
            else:
                _lib.check(self.lib.glm_tstat(ptr(self.Yd), self.V, n, self.V, ptr(slot["d_pinv"]),
                                              ptr(slot["d_X"]), ptr(slot["d_invd"]), ptr(slot["d_dof"]), P,
                                              kmax, ptr(self._coef), self.C, ptr(slot["d_t"]), self.V,
                                              stream_handle()))

        def body_sweep():
            self.adj.sweep_batch(ptr(slot["d_t"]), self.V, P * self.C, self.signs, ptr(self.vd),
                                 int(self.floor_zero), ptr(slot["d_max"]), None, 0, stream_handle())
            slot["h_max"].copy_(slot["d_max"], non_blocking=True)

        # warm-up outside capture (allocates the sweep workspace), then capture
        # two graphs: the GLM part (the last reader of the resident data) and
        # the sweep part, so new data can be uploaded while a sweep runs
        side = t.cuda.Stream()
        side.wait_stream(t.cuda.current_stream())
        with t.cuda.stream(side):
            body_glm()
            body_sweep()
        t.cuda.current_stream().wait_stream(side)
        t.cuda.synchronize()
        self.status()
        g1, g2 = t.cuda.CUDAGraph(), t.cuda.CUDAGraph()
        with t.cuda.graph(g1):
            body_glm()
        with t.cuda.graph(g2):
            body_sweep()
        slot["graph_glm"], slot["graph_sweep"] = g1, g2
        slot["event"] = t.cuda.Event()
        slot["glm_done"] = t.cuda.Event()
        return slot

    def _fill(self, slot, perms):
        db = DesignBatch(self.X[perms])
        P = perms.shape[0]
        if slot["QF"]:
            self._tc.host_operands_qf(db, XR=slot["h_XR"].numpy(), GI=slot["h_GI"].numpy())
        elif self._tc is not None:
            self._tc.host_operands(db, P8=slot["h_P8"].numpy(), U=slot["h_U"].numpy(), Xt=slot["h_Xt"].numpy(),
                                   centred=self._centred)
            if self._w_stride:
                db.program_weights(self.outputs, out=slot["h_W"].numpy()[:P])
        else:
            slot["h_pinv"].numpy()[:P] = db.pinv64
            slot["h_X"].numpy()[:P] = db.X64
        slot["h_invd"].numpy()[:P] = db.invdiag64
        slot["h_dof"].numpy()[:P] = db.dof

    def run_graph(self, n_perm=None, seed=0, start=0, stop=None, perms=None):
        """Same result as run(), through two captured batch graphs replayed in
        turn: while one batch runs on the GPU the host forms the next batch's
        design inverses (run_stream over the batches)."""
        if perms is None:
            stop = start + n_perm if stop is None else stop
            perms = permutations(self.n, seed, start, stop)
        P = self.batch
        res = self.run_stream((None, perms[b:b + P]) for b in range(0, perms.shape[0], P))
        return np.concatenate(res) if res else np.zeros((0, self.C, self.signs, self.n_seg), np.float32)

    def run_stream(self, steps, on_batch=None):
        """The pipelined public entry: one batch per item of `steps`, each a
        pair (data, perms) -- data: new (n, V) host data in the caller's
        vertex order (pinned memory keeps the copy asynchronous) or None to
        keep the resident data; perms: at most `batch` permutation index rows.
        Two captured batch slots are replayed in turn, each as a GLM graph and
        a sweep graph.  The host forms a batch's design operators while the
        GPU runs the previous batch; new data is copied and re-tiled on a side
        stream once the previous batch's GLM (the last reader of the resident
        data) is done, so the upload overlaps that batch's sweep, and this
        batch's GLM waits for it; each batch's maxima come back when its slot
        is reused or at the end.  A short batch is padded with its last row
        inside the captured graph and the padding discarded.
        on_batch (optional): called as on_batch(i, maxima) as soon as step i's
        maxima are back on the host, while later steps run on the device --
        host work placed there overlaps the device.
        Returns the per-batch maxima, (rows, C, signs, n_seg) each."""
        t = self.t
        P = self.batch
        DB = None if self._tc is None else self._tc.block(self.k)
        if (not hasattr(self, "_slots") or self._slots[0]["P"] != P or self._slots[0].get("DB") != DB
                or self._slots[0]["QF"] != self._graph_qf()):
            self._slots = [self._graph_slot(P), self._graph_slot(P)]
        if not hasattr(self, "_up_stream"):
            self._up_stream = t.cuda.Stream()
            self._up_done = t.cuda.Event()
        for slot in self._slots:
            if slot.get("busy"):  # left by a call that raised: drain it, its maxima are not this call's
                slot["event"].synchronize()
                slot["busy"] = False
        main = t.cuda.current_stream()
        results = {}
        prev = None

        def collect(slot):
            slot["event"].synchronize()
            results[slot["order"]] = slot["h_max"].numpy()[: slot["rows"]].copy()
            slot["busy"] = False
            if on_batch is not None:
                on_batch(slot["order"], results[slot["order"]])

        n_steps = 0
        for s_, (data, perms) in enumerate(steps):
            perms = np.asarray(perms)
            rows = perms.shape[0]
            if rows == 0:
                results[s_] = np.zeros((0, self.C, self.signs, self.n_seg), np.float32)
                n_steps = s_ + 1
                continue
            if rows > P:
                raise ValueError("a step has more permutations than the engine's batch")
            if rows < P:
                perms = np.concatenate([perms, np.repeat(perms[-1:], P - rows, axis=0)])
            slot = self._slots[s_ % 2]
            if slot.get("busy"):
                collect(slot)
            self._fill(slot, perms)
            if data is not None:
                up = self._up_stream
                up.wait_stream(main) if prev is None else up.wait_event(prev["glm_done"])
                with t.cuda.stream(up):
                    self.upload(data)
                self._up_done.record(up)
                main.wait_event(self._up_done)
            slot["graph_glm"].replay()
            slot["glm_done"].record(main)
            slot["graph_sweep"].replay()
            slot["event"].record(main)
            slot["busy"], slot["order"], slot["rows"] = True, s_, rows
            prev = slot
            n_steps = s_ + 1
        for slot in self._slots:
            if slot.get("busy"):
                collect(slot)
        self.status()
        return [results[i] for i in range(n_steps)]

    def observed(self):
        """Unpermuted t maps (C, V) and scaled TFCE maps (C, signs, V) as host arrays
        (write_vertStat_img's TFCE image, pyfunc.py:80-92)."""
        t = self.t
        db = DesignBatch(self.X[None])
        if self.outputs is None:
            # the observed map in FP64 with the reference's precision (tval_int): it is the
            # image the reference writes and compares against its null
            from .glm import WHAT_T, glm_stat_f64
            tm = glm_stat_f64(self.Yd, db, WHAT_T, coef=self.contrasts).float().contiguous()
        else:
            # programmed outputs exist on the tensor-core GLM only
            tm = t.empty((1, self.C, self.V), device="cuda", dtype=t.float32)
            self.tmaps(db, out=tm)
        maps = t.empty((self.C, self.signs, self.V), device="cuda", dtype=t.float32)
        mx = t.empty((self.C, self.signs, self.n_seg), device="cuda", dtype=t.float32)
        # the observed image is swept once: use the reference's exact arithmetic
        mode = getattr(self.adj, "accumulation", "exact")
        self.adj.set_accumulation("exact")
        try:
            self.adj.sweep_batch(ptr(tm), self.V, self.C, self.signs, ptr(self.vd),
                                 int(self.floor_zero), ptr(mx), ptr(maps), 1, stream_handle())
            self.adj.status()
        finally:
            self.adj.set_accumulation(mode)
        return self.to_caller(tm[0].cpu().numpy()), self.to_caller(maps.cpu().numpy()), mx.cpu().numpy()

    def to_caller(self, a):
        """Maps in the engine's internal vertex order -> the caller's order."""
        if self.order is None:
            return a
        out = np.empty_like(a)
        out[..., self.order] = a
        return out


def reduce_vertex(maxima):
    """Per-permutation CSV values of the vertex path: max over segments
    (hemispheres), pyfunc.py:118.  (P, C, signs, S) -> (P, C, signs)."""
    return maxima.max(axis=-1)


def null_distribution(maxima, contrast):
    """Interleave + and - maxima as the reference appends them to one CSV
    (randomise :115-116): (P, C, 2) -> (2P,)."""
    return np.asarray(maxima)[:, contrast, :].reshape(-1)


class MediationEngine:
    """Indirect-effect (Sobel/Aroian/Goodman) z + TFCE null distribution: the
    batched form of vertex_tfce_mediation_randomise.py:79-91 and
    tm_func.low_ram_calculate_mediation_tfce (tm_func.py:269-305).

    Per permutation the reference permutes pred_x (and, for medtype 'Y', also
    depend_y) and regresses the data on the path-a design [1, x] and the
    path-b design ([1, x, y] for 'I', [1, y, x] for 'M' and 'Y'; pyfunc.py:131-145),
    taking coefficient 1 of each.  Here both designs of P permutations go into
    one glm_tstat launch (2P designs, kmax 3), sobel_combine forms z, and one
    sweep launch gives the maxima (one sign: z >= 0 for Aroian/Sobel).  For
    medtype 'Y' path a is a host regression of depend_y on pred_x (scipy
    linregress), as in the reference.  covariates: unpermuted columns appended
    to both designs (the tm-models mediation branch,
    tm_models_randomise.py:430-503, where path a of 'Y' is glm_typeI's t)."""

    def __init__(self, Y, pred_x, depend_y, medtype, adjacency, segments=None, H=2.0, E=1.0, vdensity=None,
                 floor_zero=False, batch=64, alg="aroian", accumulation="component", precision="bf16x3",
                 covariates=None, threshold_groups=None):
        from .pyfunc import ALG
        if medtype not in ("I", "M", "Y"):
            raise ValueError("Invalid mediation type")
        if alg not in ALG:
            raise ValueError("Unknown indirect test algorithm")
        self.inner = PermutationEngine(Y, np.zeros((np.asarray(Y).shape[0], 1)), adjacency, segments, H, E,
                                       vdensity, contrasts=[1], floor_zero=floor_zero, batch=2 * batch, signs=1,
                                       reorder=False, accumulation=accumulation, precision=precision,
                                       threshold_groups=threshold_groups)
        self.t = self.inner.t
        self.medtype, self.alg, self.alg_code, self.batch = medtype, alg, ALG[alg], int(batch)
        self.pred_x = np.asarray(pred_x, np.float64)
        self.depend_y = np.asarray(depend_y, np.float64)
        self.cov = None if covariates is None else np.asarray(covariates, np.float64)
        self.n, self.V, self.n_seg = self.inner.n, self.inner.V, self.inner.n_seg
        n_cov = 0 if self.cov is None else self.cov.reshape(self.n, -1).shape[1]
        width = self.pred_x.reshape(self.n, -1).shape[1] + self.depend_y.reshape(self.n, -1).shape[1]
        self.kmax = 1 + width + n_cov
        if self.kmax > 8:
            raise ValueError("at most 8 design columns (intercept, pred_x, depend_y, covariates)")
        self._z = self.t.empty((self.batch, self.V), device="cuda", dtype=self.t.float32)
        self._max = self.t.empty((self.batch, 1, self.inner.n_seg), device="cuda", dtype=self.t.float32)

    def _paths(self, perms):
        from .pyfunc import mediation_designs
        A, B, ta = [], [], []
        for p in perms:
            x = self.pred_x[p]
            dy = self.depend_y if self.medtype in ("M", "I") else self.depend_y[p]
            Xa, Xb, tas = mediation_designs(self.medtype, x, dy, self.n, covariates=self.cov)
            A.append(Xa)
            B.append(Xb)
            ta.append(tas)
        return A, B, ta

    def _designs(self, perms):
        """Host work of a batch: the path designs (FP64 inverses) of the
        permutation rows, as (DesignBatch, path-a t of medtype 'Y' or None)."""
        A, B, ta = self._paths(perms)
        if self.medtype == "Y":
            return DesignBatch(B, kmax=self.kmax), np.asarray(ta, np.float32)
        return DesignBatch([m for pair in zip(A, B) for m in pair], kmax=self.kmax), None

    def _zmaps_from(self, db, ta, P, out=None):
        inner = self.inner
        z = self._z[:P] if out is None else out
        lib = inner.lib
        tm = inner.tmaps(db)
        if self.medtype == "Y":  # tm (P, 1, V): path b
            tas = dev(ta)
            _lib.check(lib.sobel_combine(None, self.V, ptr(tas), ptr(tm), self.V, P, self.V, self.alg_code,
                                         ptr(z), self.V, stream_handle()))
        else:  # tm (2P, 1, V): a, b, a, b ...
            _lib.check(lib.sobel_combine(ptr(tm), 2 * self.V, None, ptr(tm) + 4 * self.V, 2 * self.V, P,
                                         self.V, self.alg_code, ptr(z), self.V, stream_handle()))
        return z

    def zmaps(self, perms, out=None):
        """Indirect-effect z maps (P, V) on the device for permutation rows."""
        db, ta = self._designs(perms)
        return self._zmaps_from(db, ta, len(perms), out)

    def run_batch(self, perms):
        """Maxima (P, 1, 1, n_seg) for the permutation index rows `perms`."""
        P = len(perms)
        if P > self.batch:
            raise ValueError("batch larger than the engine's buffers")
        z = self.zmaps(perms)
        mx = self._max.view(-1)[: P * self.n_seg]
        self.inner.adj.sweep_batch(ptr(z), self.V, P, 1, ptr(self.inner.vd), int(self.inner.floor_zero),
                                   ptr(mx), None, 0, stream_handle())
        out = mx.cpu().numpy().reshape(P, 1, 1, self.n_seg)
        self.inner.status()
        return out

    def run(self, n_perm=None, seed=0, start=0, stop=None, perms=None):
        """Null maxima (n_perm, 1, 1, n_seg).  A batch's maxima are read back
        after the next batch is queued, so the host forms the next batch's
        path designs (FP64 inverses) while the GPU runs the current one."""
        if perms is None:
            stop = start + n_perm if stop is None else stop
            perms = permutations(self.n, seed, start, stop)
        res = self.run_stream((None, perms[b:b + self.batch]) for b in range(0, perms.shape[0], self.batch))
        return np.concatenate(res) if res else np.zeros((0, 1, 1, self.n_seg), np.float32)

    def run_stream(self, steps):
        """The pipelined public entry, as PermutationEngine.run_stream: one
        batch per item (data, perms) of `steps` -- data: new (n, V) mediator
        data from the host (pinned memory keeps the copy asynchronous) or None
        to keep the resident data; perms: at most `batch` permutation rows.
        A batch's path designs are formed on the host while the previous batch
        runs on the device; new data is copied and re-tiled on a side stream
        once the previous batch's GLM (the last reader of the resident data)
        is done, and this batch's GLM waits for it; each batch's maxima are
        read back after the next batch is queued.  Returns the per-batch
        maxima, (rows, 1, 1, n_seg) each."""
        t = self.t
        inner = self.inner
        if not hasattr(self, "_host_max"):
            self._host_max = [t.empty(self.batch * self.n_seg, dtype=t.float32, pin_memory=True) for _ in range(2)]
            self._max2 = [self._max.view(-1), t.empty_like(self._max.view(-1))]
            self._done = [t.cuda.Event(), t.cuda.Event()]
            self._glm_done = [t.cuda.Event(), t.cuda.Event()]
            self._up_stream = t.cuda.Stream()
            self._up_done = t.cuda.Event()
        main = t.cuda.current_stream()
        out, prev = [], None

        def collect(item):
            k, P = item
            self._done[k].synchronize()
            out.append(self._host_max[k][: P * self.n_seg].numpy().reshape(P, 1, 1, self.n_seg).copy())

        for i, (data, rows) in enumerate(steps):
            rows = np.asarray(rows)
            P, k = len(rows), i % 2
            if P > self.batch:
                raise ValueError("a step has more permutations than the engine's batch")
            if P == 0:
                out.append(np.zeros((0, 1, 1, self.n_seg), np.float32))
                continue
            db, ta = self._designs(rows)  # host work, overlapping the previous batch
            if data is not None:
                up = self._up_stream
                up.wait_stream(main) if prev is None else up.wait_event(self._glm_done[prev[0]])
                with t.cuda.stream(up):
                    inner.upload(data)
                self._up_done.record(up)
                main.wait_event(self._up_done)
            z = self._zmaps_from(db, ta, P)
            self._glm_done[k].record(main)
            mx = self._max2[k][: P * self.n_seg]
            inner.adj.sweep_batch(ptr(z), self.V, P, 1, ptr(inner.vd), int(inner.floor_zero),
                                  ptr(mx), None, 0, stream_handle())
            self._host_max[k][: P * self.n_seg].copy_(mx, non_blocking=True)
            self._done[k].record(main)
            if prev is not None:
                collect(prev)
            prev = (k, P)
        if prev is not None:
            collect(prev)
        inner.status()
        return out

    def observed(self):
        """Unpermuted z map (V,) and scaled TFCE map (V,) on the host."""
        t = self.t
        from .pyfunc import sobel_z_device
        # the observed z from FP64 path t maps (the reference's precision)
        z = sobel_z_device(self.medtype, self.pred_x, self.depend_y, self.inner.Yd, self.n,
                           alg=self.alg, covariates=self.cov)
        maps = t.empty((1, 1, self.V), device="cuda", dtype=t.float32)
        mx = t.empty((1, 1, self.n_seg), device="cuda", dtype=t.float32)
        adj = self.inner.adj
        mode = getattr(adj, "accumulation", "exact")
        adj.set_accumulation("exact")
        try:
            adj.sweep_batch(ptr(z), self.V, 1, 1, ptr(self.inner.vd), int(self.inner.floor_zero), ptr(mx),
                            ptr(maps), 1, stream_handle())
            adj.status()
        finally:
            adj.set_accumulation(mode)
        return z[0].cpu().numpy(), maps[0, 0].cpu().numpy(), mx[0, 0].cpu().numpy()
