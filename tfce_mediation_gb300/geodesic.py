"""Exact geodesic distance lists on the GPU: drop-ins for the reference's
``tfce_mediation.adjacency`` module (tfce_mediation/adjacency.pyx:44-106).

The reference propagates its exact geodesic library (tfce_mediation/lib/geodesic)
from one source vertex at a time on one CPU core and then asks for the
distance of every vertex j > i.  Here every source of the mesh is propagated
in one launch (``csrc/geodesic.cu``: one warp per source, exact window
propagation with double-precision distances) and only the vertices reached
within the radius are listed.

* ``compute(v, f, thresholds)`` -- adjacency.pyx:44-80: for every threshold,
  the list of vertices within that geodesic distance of each vertex (Python
  lists, ascending, the order the reference's appends produce).
* ``compute_distance_parallel(v, f, threshold, i)`` -- adjacency.pyx:83-106:
  ``[[i, j, distance], ...]`` for j > i with distance < threshold.
* ``distance_lists(v, f, threshold)`` -- every source at once: (pairs [N, 2]
  int32, distances [N] float64), what misc_scripts/
  fwhm_compute_distances_parallel.py:104-110 assembles from V calls of
  compute_distance_parallel (it stores the distances as float32).
* ``GeodesicMesh`` -- the mesh handle for repeated queries.

The reference prints a line per pair found; these do not.  There is no CPU
fallback: without the CUDA library or a GPU these raise.
"""
from __future__ import annotations

import ctypes
import hashlib

import numpy as np

from . import _lib


class GeodesicMesh:
    """A triangle mesh on the device (geodesic_mesh_create): vertices [V, 3]
    (float32, as the reference takes them) and faces [F, 3] (int32)."""

    def __init__(self, v, f):
        self._lib = _lib.load()
        v = np.ascontiguousarray(v, np.float32)
        f = np.ascontiguousarray(f, np.int32)
        if v.ndim != 2 or v.shape[1] != 3 or f.ndim != 2 or f.shape[1] != 3:
            raise ValueError(f"vertices [V, 3] and faces [F, 3] expected, got {v.shape} and {f.shape}")
        h = ctypes.c_void_p()
        _lib.check(self._lib.geodesic_mesh_create(_lib.ptr(v, _lib.c_f32p), v.shape[0], _lib.ptr(f, _lib.c_i32p),
                                                  f.shape[0], ctypes.byref(h)))
        self._h = h
        self.n_vertices = int(v.shape[0])
        self.n_faces = int(f.shape[0])

    @property
    def n_saddle(self) -> int:
        """Pseudo-source vertices: total angle above 2 pi - 1e-5, or on the boundary."""
        n = ctypes.c_int32()
        _lib.check(self._lib.geodesic_mesh_saddles(self._h, ctypes.byref(n)))
        return int(n.value)

    def lists(self, threshold, only_greater=True, src_lo=0, src_hi=None):
        """(i, j, d) for sources i in [src_lo, src_hi) and vertices j != i at
        geodesic distance d < threshold (j > i only when only_greater), sorted
        by i then j; d is float64."""
        src_hi = self.n_vertices if src_hi is None else int(src_hi)
        n = ctypes.c_int64()
        _lib.check(self._lib.geodesic_distance_lists(self._h, float(threshold), int(bool(only_greater)),
                                                     int(src_lo), src_hi, ctypes.byref(n)))
        k = int(n.value)
        i = np.empty(k, np.int32)
        j = np.empty(k, np.int32)
        d = np.empty(k, np.float64)
        _lib.check(self._lib.geodesic_take_lists(self._h, _lib.ptr(i, _lib.c_i32p), _lib.ptr(j, _lib.c_i32p),
                                                 _lib.ptr(d, _lib.c_f64p), k))
        return i, j, d

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._lib.geodesic_mesh_destroy(h)
            self._h = None


_CACHE = {"key": None, "mesh": None}


def _mesh(v, f):
    """The device mesh of (v, f), kept for the next call with the same arrays
    (compute_distance_parallel is called once per source vertex)."""
    v = np.ascontiguousarray(v, np.float32)
    f = np.ascontiguousarray(f, np.int32)
    key = (v.shape, f.shape, hashlib.blake2b(v.tobytes(), digest_size=16).hexdigest(),
           hashlib.blake2b(f.tobytes(), digest_size=16).hexdigest())
    if _CACHE["key"] != key:
        _CACHE["mesh"] = None
        _CACHE["mesh"] = GeodesicMesh(v, f)
        _CACHE["key"] = key
    return _CACHE["mesh"]


def distance_lists(v, f, threshold, only_greater=True):
    """Every source's list at once: (pairs [N, 2] int32 of (i, j), distances
    [N] float64), sorted by i then j, with j > i when only_greater."""
    i, j, d = _mesh(v, f).lists(threshold, only_greater)
    return np.ascontiguousarray(np.stack([i, j], axis=1)), d


def compute_distance_parallel(v, f, threshold, i):
    """adjacency.pyx:83-106: [[i, j, distance], ...] for every vertex j > i at
    geodesic distance below threshold, in j order."""
    i = int(i)
    src, dst, d = _mesh(v, f).lists(float(threshold), True, i, i + 1)
    return [[i, int(b), float(c)] for b, c in zip(dst.tolist(), d.tolist())]


def lists_from_pairs(i, j, d, thresholds, n_vertices):
    """The reference's per-threshold lists from the (i < j) pairs and their
    distances: adjacency.pyx:66-72 appends i to j's list and j to i's list for
    every pair below thresholds[k], sources i ascending and j ascending within
    a source, so each list comes out ascending.  thresholds are float32 values
    compared as doubles (adjacency.pyx:70)."""
    out = []
    for t in np.asarray(thresholds, np.float32).tolist():
        keep = np.asarray(d) < t
        a = np.asarray(i)[keep].astype(np.int64)
        b = np.asarray(j)[keep].astype(np.int64)
        rows = np.concatenate([b, a])
        cols = np.concatenate([a, b])
        order = np.lexsort((cols, rows))
        rows, cols = rows[order], cols[order]
        cuts = np.searchsorted(rows, np.arange(n_vertices + 1))
        flat = cols.tolist()
        out.append([flat[cuts[x]:cuts[x + 1]] for x in range(n_vertices)])
    return out


def compute(v, f, thresholds):
    """adjacency.pyx:44-80: adjacency[k][x] lists every vertex within
    thresholds[k] of vertex x, ascending."""
    thresholds = np.asarray(thresholds, np.float32)
    m = _mesh(v, f)
    i, j, d = m.lists(float(np.max(thresholds)), True)
    return lists_from_pairs(i, j, d, thresholds, m.n_vertices)
