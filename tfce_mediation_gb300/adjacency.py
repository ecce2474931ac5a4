"""Adjacency sets: builders, CSR conversion and the device handle.

Builders reproduce the reference's adjacency lists exactly (same entries,
same quirks), vectorised with numpy instead of per-vertex Python loops:

* ``create_adjac_vertex``  -- tfce_mediation/pyfunc.py:37-46 (triangle edges,
  symmetric);
* ``create_adjac_voxel``   -- tfce_mediation/pyfunc.py:48-76 (6/26-neighbour
  voxels in ``np.where`` order; label 0 is never anyone's neighbour and its own
  list is emptied; with 6 neighbours, voxels on the grid faces get no
  neighbours);
* ``create_adjac_voxel_mmr`` -- tfce_mediation/tools/tm_mulitmodality_adjacency.py:40-67
  (keeps self entries and voxel 0's outgoing list, so it is asymmetric);
* ``merge_adjacency_array`` -- tfce_mediation/tm_func.py:521-540.

``compute`` and ``compute_distance_parallel`` (the reference's own
``tfce_mediation.adjacency`` module, adjacency.pyx:44-106: exact geodesic
neighbour lists) are the GPU drop-ins of ``geodesic.py``, importable from here
under the reference's module name.

``AdjacencySet`` owns the device CSR (the C-ABI ``tfce_adjset`` handle).
"""
from __future__ import annotations

import ctypes
import itertools

import numpy as np

from . import _lib
from .geodesic import compute, compute_distance_parallel  # noqa: F401  (adjacency.pyx:44-106)


# ---------------------------------------------------------------------------
# CSR helpers
# ---------------------------------------------------------------------------
def to_csr(adjacency):
    """List-of-iterables (sets, lists, arrays, numpy object array) -> CSR
    (offsets int64[V+1], indices int32[D]).  Entry order inside a list is kept."""
    if isinstance(adjacency, tuple) and len(adjacency) == 2 and isinstance(adjacency[0], np.ndarray) \
            and adjacency[0].dtype.kind in "iu" and adjacency[0].ndim == 1:
        off, idx = adjacency
        return np.ascontiguousarray(off, np.int64), np.ascontiguousarray(idx, np.int32)
    lens = np.fromiter((len(a) for a in adjacency), dtype=np.int64, count=len(adjacency))
    off = np.zeros(len(adjacency) + 1, np.int64)
    np.cumsum(lens, out=off[1:])
    idx = np.fromiter(itertools.chain.from_iterable(adjacency), dtype=np.int64, count=int(off[-1]))
    if idx.size and (idx.min() < -2 ** 31 or idx.max() >= 2 ** 31):
        raise ValueError("adjacency index out of int32 range")
    return off, idx.astype(np.int32)


def from_csr(offsets, indices, as_sets=False):
    """CSR -> list of lists (or sets)."""
    out = np.split(np.asarray(indices), np.asarray(offsets)[1:-1])
    return [set(a.tolist()) for a in out] if as_sets else [a.tolist() for a in out]


def _csr_from_pairs(src, dst, V, sort=True):
    """Directed pairs -> CSR with duplicates removed, lists sorted."""
    key = np.unique(src.astype(np.int64) * V + dst.astype(np.int64)) if sort else \
        src.astype(np.int64) * V + dst.astype(np.int64)
    s = key // V
    d = (key % V).astype(np.int32)
    off = np.zeros(V + 1, np.int64)
    np.add.at(off, s + 1, 1)
    np.cumsum(off, out=off)
    return off, d


# ---------------------------------------------------------------------------
# builders
# ---------------------------------------------------------------------------
def mesh_csr(faces, n_vertices):
    """Triangle-edge adjacency as CSR (sorted lists; the same entry sets as
    create_adjac_vertex)."""
    f = np.asarray(faces, np.int64)
    src = np.concatenate([f[:, 0], f[:, 0], f[:, 1], f[:, 1], f[:, 2], f[:, 2]])
    dst = np.concatenate([f[:, 1], f[:, 2], f[:, 0], f[:, 2], f[:, 0], f[:, 1]])
    return _csr_from_pairs(src, dst, int(n_vertices))


def create_adjac_vertex(vertices, faces):
    """tfce_mediation/pyfunc.py:37-46: list of neighbour sets from triangles."""
    off, idx = mesh_csr(faces, np.asarray(vertices).shape[0])
    return from_csr(off, idx, as_sets=True)


_SIX = np.array([0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 1, 0, 1, 1, 1, 0, 1, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0],
                bool).reshape(3, 3, 3)


def _voxel_pairs(mask, dirtype, six_wall_rule):
    mask = np.asarray(mask).astype(bool)
    X, Y, Z = mask.shape
    coords = np.array(np.where(mask)).T  # np.where order == label order
    nvox = coords.shape[0]
    lab = np.full(mask.shape, -1, np.int64)
    lab[mask] = np.arange(nvox)
    src_l, dst_l = [], []
    if int(dirtype) == 6:
        offs = [tuple(np.array(o) - 1) for o in zip(*np.where(_SIX))]
    else:
        offs = [(dx, dy, dz) for dx in (-1, 0, 1) for dy in (-1, 0, 1) for dz in (-1, 0, 1)]
    if int(dirtype) == 6 and six_wall_rule:
        # the reference keeps only the voxel itself when its 3x3x3 window is
        # clipped by the grid
        interior = ((coords[:, 0] > 0) & (coords[:, 0] < X - 1) & (coords[:, 1] > 0) &
                    (coords[:, 1] < Y - 1) & (coords[:, 2] > 0) & (coords[:, 2] < Z - 1))
    else:
        interior = np.ones(nvox, bool)
    for dx, dy, dz in offs:
        nx, ny, nz = coords[:, 0] + dx, coords[:, 1] + dy, coords[:, 2] + dz
        ok = (nx >= 0) & (nx < X) & (ny >= 0) & (ny < Y) & (nz >= 0) & (nz < Z) & interior
        src = np.nonzero(ok)[0]
        nb = lab[nx[ok], ny[ok], nz[ok]]
        keep = nb >= 0
        src_l.append(src[keep])
        dst_l.append(nb[keep])
    wall = np.nonzero(~interior)[0]  # their window is the voxel itself
    src_l.append(wall)
    dst_l.append(wall)
    return np.concatenate(src_l), np.concatenate(dst_l), nvox


def voxel_csr(mask, dirtype=26, variant="pyfunc"):
    """Voxel adjacency as CSR in np.where (C) order.

    variant "pyfunc": tfce_mediation/pyfunc.py:48-76 -- no self entries, label 0
    neither has nor is a neighbour, 6-neighbour grid-face voxels have none.
    variant "mmr": tfce_mediation/tools/tm_mulitmodality_adjacency.py:40-67 --
    self entries kept (label > 0), label 0 is nobody's neighbour but keeps its
    own list."""
    src, dst, nvox = _voxel_pairs(mask, dirtype, six_wall_rule=True)
    keep = dst > 0  # the reference filters local_area > 0: label 0 is never listed
    src, dst = src[keep], dst[keep]
    if variant == "pyfunc":
        keep = (src != dst) & (src != 0)
        src, dst = src[keep], dst[keep]
    elif variant != "mmr":
        raise ValueError(variant)
    return _csr_from_pairs(src, dst, nvox)


def create_adjac_voxel(data_index, data_mask=None, num_voxel=None, dirtype=26):
    """tfce_mediation/pyfunc.py:48-76 (object array of sorted lists)."""
    off, idx = voxel_csr(data_index, dirtype, "pyfunc")
    lists = from_csr(off, idx)
    out = np.empty(len(lists), dtype=object)
    for i, l in enumerate(lists):
        out[i] = l
    return out


def create_adjac_voxel_mmr(data_index, dirtype=26):
    """tfce_mediation/tools/tm_mulitmodality_adjacency.py:40-67 (list of sets)."""
    off, idx = voxel_csr(data_index, dirtype, "mmr")
    return from_csr(off, idx, as_sets=True)


def merge_adjacency_array(adjacent_range, adjacency_array):
    """tfce_mediation/tm_func.py:521-540.  As in the reference, the first merged
    block is always adjacency_array[0] (whatever adjacent_range starts with)
    while the offset advances by the size of the listed entry."""
    adjacent_range = list(adjacent_range)
    pieces = []
    v_count = 0
    if len(adjacent_range) == 1:
        return [list(a) for a in adjacency_array[0]]
    for i, e in enumerate(adjacent_range):
        src = adjacency_array[0] if v_count == 0 else adjacency_array[e]
        pieces.extend([(np.asarray(list(a), np.int64) + v_count).tolist() for a in src])
        v_count += len(adjacency_array[e])
    return pieces


def induced_csr(adjacency, mask):
    """CSR of the subgraph on the vertices where `mask` is true, renumbered in
    order; entries to vertices outside the mask are dropped.  Sweeping a masked
    statistic on it equals sweeping the statistic scattered into a zero-filled
    array on the full adjacency: zeros are never above a threshold >= 0, so they
    never join a component (the max over the zero fill is kept by the
    sweep's floor_zero option)."""
    off, idx = to_csr(adjacency)
    mask = np.asarray(mask, bool)
    V = off.shape[0] - 1
    new = np.full(V, -1, np.int64)
    new[mask] = np.arange(int(mask.sum()))
    rows = np.repeat(np.arange(V), np.diff(off))
    ok = (idx >= 0) & (idx < V)
    ok[ok] &= mask[rows[ok]] & mask[idx[ok]]
    src, dst = new[rows[ok]], new[idx[ok]]
    n = int(mask.sum())
    order = np.argsort(src, kind="stable")
    src, dst = src[order], dst[order]
    o = np.zeros(n + 1, np.int64)
    np.add.at(o, src + 1, 1)
    np.cumsum(o, out=o)
    return o, dst.astype(np.int32)


def vertex_density(adjacency):
    """Vertex-density weight 1 - deg/max + mean/max (float32), as
    tfce_mediation/tmanalysis/STEP_1_vertex_tfce_multiple_regression.py:166-173."""
    off, _ = to_csr(adjacency)
    deg = np.diff(off).astype(np.float64)
    return np.array((1 - (deg / deg.max()) + (deg.mean() / deg.max())), dtype=np.float32)


def concat_csr(parts):
    """Concatenate per-segment CSRs (local indices) into one CSR with global
    indices and segment offsets -- the offset table of a multisurface launch."""
    offs, idxs, segs = [np.zeros(1, np.int64)], [], [0]
    base_v, base_e = 0, 0
    for off, idx in parts:
        off = np.asarray(off, np.int64)
        offs.append(off[1:] + base_e)
        idxs.append(np.asarray(idx, np.int64) + base_v)
        base_v += off.shape[0] - 1
        base_e += int(off[-1])
        segs.append(base_v)
    return (np.concatenate(offs), np.concatenate(idxs).astype(np.int32) if idxs else np.zeros(0, np.int32),
            np.asarray(segs, np.int64))


def locality_order(offsets, indices, segments):
    """A vertex numbering that keeps mesh neighbours close in memory: reverse
    Cuthill-McKee inside every segment (segments stay in place).  Returns
    `order` with new vertex u = old vertex order[u]."""
    import scipy.sparse as sp
    from scipy.sparse.csgraph import reverse_cuthill_mckee
    offsets = np.asarray(offsets, np.int64)
    indices = np.asarray(indices, np.int64)
    order = []
    for s in range(len(segments) - 1):
        v0, v1 = int(segments[s]), int(segments[s + 1])
        n = v1 - v0
        if n == 0:
            continue
        e0, e1 = offsets[v0], offsets[v1]
        loc = indices[e0:e1] - v0
        ok = (loc >= 0) & (loc < n)
        rows = np.repeat(np.arange(n), np.diff(offsets[v0:v1 + 1]))[ok]
        A = sp.csr_matrix((np.ones(rows.shape[0], np.int8), (rows, loc[ok])), shape=(n, n))
        A = ((A + A.T) > 0).astype(np.int8).tocsr()
        order.append(np.asarray(reverse_cuthill_mckee(A, symmetric_mode=True), np.int64) + v0)
    return np.concatenate(order) if order else np.zeros(0, np.int64)


def is_symmetric(offsets, indices):
    """True when every entry b in list a has a in list b (self entries aside)."""
    import scipy.sparse as sp
    offsets = np.asarray(offsets, np.int64)
    indices = np.asarray(indices, np.int64)
    V = offsets.shape[0] - 1
    rows = np.repeat(np.arange(V), np.diff(offsets))
    ok = (indices >= 0) & (indices < V) & (indices != rows)
    A = sp.csr_matrix((np.ones(int(ok.sum()), np.int8), (rows[ok], indices[ok])), shape=(V, V))
    A.data[:] = 1
    return (A != A.T).nnz == 0


def relabel_csr(offsets, indices, order):
    """CSR of the same graph with vertex u_new = order[u_new] renamed; lists
    keep their entries (renamed), out-of-range entries are kept as they are so
    the handle still rejects them."""
    offsets = np.asarray(offsets, np.int64)
    indices = np.asarray(indices, np.int64)
    V = offsets.shape[0] - 1
    inv = np.empty(V, np.int64)
    inv[order] = np.arange(V)
    deg = np.diff(offsets)[order]
    off = np.zeros(V + 1, np.int64)
    np.cumsum(deg, out=off[1:])
    starts = offsets[order]
    src = np.repeat(starts - off[:-1], deg) + np.arange(int(off[-1]))
    old = indices[src]
    ok = (old >= 0) & (old < V)
    new = old.copy()
    new[ok] = inv[old[ok]]
    return off, new.astype(np.int32)


# ---------------------------------------------------------------------------
# device handle
# ---------------------------------------------------------------------------
class AdjacencySet:
    """Device CSR + per-segment TFCE parameters (the ``tfce_adjset`` handle).

    ``adjacency``: list-of-iterables or (offsets, indices).  ``segments``:
    vertex offsets [n_seg+1] (default: one segment).  ``H``/``E``: scalars or
    per-segment sequences."""

    def __init__(self, adjacency, H=2.0, E=1.0, segments=None):
        self._lib = _lib.load()
        off, idx = to_csr(adjacency)
        V = off.shape[0] - 1
        if segments is None:
            segments = np.array([0, V], np.int64)
        segments = np.ascontiguousarray(segments, np.int64)
        n_seg = segments.shape[0] - 1
        Hs = np.ascontiguousarray(np.broadcast_to(np.asarray(H, np.float32), (n_seg,)))
        Es = np.ascontiguousarray(np.broadcast_to(np.asarray(E, np.float32), (n_seg,)))
        h = ctypes.c_void_p()
        _lib.check(self._lib.tfce_adjset_create(
            _lib.ptr(off, _lib.c_i64p), _lib.ptr(idx, _lib.c_i32p), V,
            _lib.ptr(segments, _lib.c_i64p), n_seg, _lib.ptr(Hs, _lib.c_f32p),
            _lib.ptr(Es, _lib.c_f32p), ctypes.byref(h)))
        self._h = h
        self.csr = (off, idx)  # host copy: the in-memory multisurface bodies re-cut it into segments
        self.n_vertices = V
        self.n_entries = int(off[-1])
        self.segments = segments
        self.n_seg = n_seg
        self.H = Hs.copy()
        self.E = Es.copy()
        self.accumulation = "exact"  # the native handle's defaults
        self.ctas_per_sm = 3
        self.threshold_groups = None

    @property
    def handle(self):
        return self._h

    @property
    def symmetric(self) -> bool:
        return bool(self._lib.tfce_adjset_is_symmetric(self._h))

    def set_params(self, H, E):
        Hs = np.ascontiguousarray(np.broadcast_to(np.asarray(H, np.float32), (self.n_seg,)))
        Es = np.ascontiguousarray(np.broadcast_to(np.asarray(E, np.float32), (self.n_seg,)))
        _lib.check(self._lib.tfce_adjset_set_params(self._h, _lib.ptr(Hs, _lib.c_f32p),
                                                    _lib.ptr(Es, _lib.c_f32p)))
        self.H, self.E = Hs.copy(), Es.copy()

    def set_threshold_groups(self, groups):
        """Segments sharing a group id share one threshold table per map and
        sign, built from the largest of their maxima (one merged adjacency
        over several surfaces, tm_func.py:68-91); None: one table per segment."""
        if groups is None:
            _lib.check(self._lib.tfce_adjset_set_threshold_groups(self._h, None))
            self.threshold_groups = None
            return
        g = np.ascontiguousarray(np.asarray(groups, np.int32))
        if g.shape != (self.n_seg,):
            raise ValueError(f"threshold groups: {self.n_seg} ids expected, got shape {g.shape}")
        _lib.check(self._lib.tfce_adjset_set_threshold_groups(self._h, _lib.ptr(g, _lib.c_i32p)))
        self.threshold_groups = g.copy()

    def set_sweep_shape(self, ctas_per_sm: int):
        """Resident CTAs per SM of the per-component sweeps: 3 (40 registers,
        most items in flight) or 2 (64 registers, no spills)."""
        _lib.check(self._lib.tfce_adjset_set_sweep_shape(self._h, int(ctas_per_sm)))
        self.ctas_per_sm = int(ctas_per_sm)

    def set_accumulation(self, mode: str):
        """'exact' (the reference's float arithmetic, bit-identical),
        'component' (per-component double accumulation for batched sweeps;
        maxima-only launches keep each component's largest sum) or
        'component-chain' (per-component, every vertex resolved along its
        chain of potentials even when only maxima are asked for)."""
        code = {"exact": 0, "component": 1, "component-chain": 2}[mode]
        _lib.check(self._lib.tfce_adjset_set_accumulation(self._h, code))
        self.accumulation = mode

    def run(self, image: np.ndarray, enhn: np.ndarray) -> None:
        """Sweep one host map, accumulating into enhn (float32, length V)."""
        _lib.check(self._lib.tfce_adjset_run(self._h, _lib.ptr(image, _lib.c_f32p),
                                             _lib.ptr(enhn, _lib.c_f32p), self.n_vertices))

    def run_labels(self, image, max_steps=128):
        """Sweep with per-threshold labels/extents (debug; one segment)."""
        V = self.n_vertices
        image = np.ascontiguousarray(image, np.float32)
        enhn = np.zeros(V, np.float32)
        labels = np.full((max_steps, V), -1, np.int32)
        extents = np.zeros((max_steps, V), np.int32)
        steps = ctypes.c_int32(0)
        _lib.check(self._lib.tfce_adjset_run_labels(
            self._h, _lib.ptr(image, _lib.c_f32p), _lib.ptr(enhn, _lib.c_f32p), V,
            _lib.ptr(labels, _lib.c_i32p), _lib.ptr(extents, _lib.c_i32p), max_steps,
            ctypes.byref(steps)))
        L = steps.value
        return enhn, labels[:L], extents[:L]

    def sweep_batch(self, stats_ptr, map_stride, n_maps, signs, vdensity_ptr, floor_zero,
                    out_max_ptr, out_maps_ptr=None, out_mode=0, stream=None):
        """Raw device-pointer batch sweep (stream-ordered)."""
        _lib.check(self._lib.tfce_sweep_batch(self._h, stats_ptr, int(map_stride), int(n_maps),
                                              int(signs), vdensity_ptr, int(floor_zero),
                                              out_max_ptr, out_maps_ptr, int(out_mode), stream))

    def resident_slots(self):
        """Sweep items run at once (the persistent grid's CTAs)."""
        n = ctypes.c_int32(0)
        _lib.check(self._lib.tfce_sweep_resident_slots(self._h, ctypes.byref(n)))
        return int(n.value)

    def status(self, stream=None):
        """Synchronise and raise if a queued sweep set the device error word."""
        _lib.check(self._lib.tfce_sweep_status(self._h, stream))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                self._lib.tfce_adjset_destroy(h)
            except Exception:
                pass
            self._h = None
