"""Drop-in for ``tfce_mediation.tfce`` (tfce_mediation/tfce.pyx:24-45).

``CreateAdjSet(H, E, pyAdjacency)`` copies the adjacency to the GPU once;
``run(image, enhn)`` sweeps ``image`` and accumulates into ``enhn`` exactly as
the reference's C++ sweep does (tfce_mediation/lib/fast_tfce.hpp:11-95), on the
device.  Argument checks follow the Cython buffer declarations
(``numpy.ndarray[float, ndim=1, mode="c"]``): a non-array raises TypeError, a
wrong dtype / rank / layout raises ValueError.  Unlike the reference, an array
whose length differs from the adjacency's vertex count raises ValueError
instead of reading out of bounds.
"""
from __future__ import annotations

import numpy as np

from .adjacency import AdjacencySet


def _check_buffer(name, a):
    if not isinstance(a, np.ndarray):
        raise TypeError(f"Argument '{name}' has incorrect type (expected numpy.ndarray, got "
                        f"{type(a).__name__})")
    if a.dtype != np.float32:
        raise ValueError(f"Buffer dtype mismatch, expected 'float' but got '{a.dtype}'")
    if a.ndim != 1:
        raise ValueError(f"Buffer has wrong number of dimensions (expected 1, got {a.ndim})")
    if not a.flags.c_contiguous:
        raise ValueError("ndarray is not C-contiguous")


class CreateAdjSet:
    """TFCE operator bound to one adjacency set and one (H, E) pair."""

    def __init__(self, H, E, pyAdjacency):
        # the reference stores H and E as C floats (tfce.pyx:27-28)
        self.H = float(np.float32(H))
        self.E = float(np.float32(E))
        self._adj = AdjacencySet(pyAdjacency, self.H, self.E)

    @property
    def adjacency(self) -> AdjacencySet:
        return self._adj

    @property
    def n_vertices(self) -> int:
        return self._adj.n_vertices

    def run(self, image, enhn):
        _check_buffer("image", image)
        _check_buffer("enhn", enhn)
        if enhn.flags.writeable is False:
            raise ValueError("buffer source array is read-only")
        V = self._adj.n_vertices
        if image.shape[0] != V or enhn.shape[0] != V:
            raise ValueError(f"array length {image.shape[0]}/{enhn.shape[0]} differs from the "
                             f"adjacency set's {V} vertices")
        self._adj.run(image, enhn)
        return None
