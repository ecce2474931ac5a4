"""Batched permutation engine: the GB300 form of the reference's randomise loops
(tfce_mediation/tmanalysis/vertex_tfce_multiple_regression_randomise.py:90-117,
voxel_tfce_multiple_regression_randomise.py:95-118,
vertex_tfce_mediation_randomise.py:79-91,
tfce_mediation/tm_func.py:144-185 and 269-305).

Per launch, P permutations:
  1. host: permutation indices RandomState(seed + p).permutation(n) and, in
     float64, each permuted design's inv(X'X) X' and diag(inv(X'X));
  2. device: one glm_tstat launch -> t maps [P][C][V] (float32, resident);
  3. device: one tfce_sweep_batch launch over P x C maps x (+,-) x segments
     -> the scaled per-segment maximum of every sweep;
  4. host: max over segments (hemispheres) gives the reference's per-permutation
     CSV values (2 per contrast: + then -).
Y stays resident in HBM for the whole run; per launch only the P design
operators go up and P x C x 2 x S maxima come down.
"""
from __future__ import annotations

import numpy as np

from . import _lib
from .adjacency import AdjacencySet, is_symmetric, locality_order, relabel_csr, to_csr
from .device import dev, ptr, require_cuda, stream_handle
from .glm import DesignBatch


def permutations(n, seed, start, stop):
    """Index streams of the mmr-lr convention (tm_func.py:147-151)."""
    return np.stack([np.random.RandomState(seed + p).permutation(n) for p in range(start, stop)])


class PermutationEngine:
    """Mass-univariate GLM + TFCE null distribution on one GPU.

    Y: (n, V) float32 data (subjects x vertices, concatenated segments).
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
    reorder: renumber vertices inside every segment for memory locality
    (reverse Cuthill-McKee); Y's columns are permuted once here and every map
    handed back is in the caller's order.  Only symmetric adjacency is
    renumbered (for one-way entries the tie rule depends on vertex order), so
    results do not depend on it."""

    def __init__(self, Y, pred_x, adjacency, segments=None, H=2.0, E=1.0, vdensity=None,
                 contrasts=None, floor_zero=False, batch=64, signs=2, reorder=False,
                 accumulation="component"):
        t = require_cuda()
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
        self.contrasts = list(range(1, self.k)) if contrasts is None else list(contrasts)
        self.C = len(self.contrasts)
        self.signs = signs
        self.floor_zero = bool(floor_zero)
        self.vd = None if vdensity is None else dev(np.asarray(vdensity, np.float32))
        self.batch = int(batch)
        self._coef = dev(np.asarray(self.contrasts, np.int32))
        self._tbuf = t.empty((self.batch, self.C, self.V), device="cuda", dtype=t.float32)
        self._maxbuf = t.empty((self.batch, self.C, self.signs, self.n_seg), device="cuda",
                               dtype=t.float32)
        self._host_max = t.empty((self.batch, self.C, self.signs, self.n_seg), dtype=t.float32,
                                 pin_memory=True)
        self.lib = _lib.load()

    # -- device steps -------------------------------------------------------
    def _designs(self, perms):
        return DesignBatch(self.X[perms])

    def tmaps(self, designs: DesignBatch, out=None):
        """t maps [G][C][V] for a DesignBatch (device tensor)."""
        G = designs.G
        out = self._tbuf[:G] if out is None else out
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
        self.adj.status()
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

    def observed(self):
        """Unpermuted t maps (C, V) and scaled TFCE maps (C, signs, V) as host arrays
        (write_vertStat_img's TFCE image, pyfunc.py:80-92)."""
        t = self.t
        db = DesignBatch(self.X[None])
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
