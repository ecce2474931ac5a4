"""Generate tests/golden/geodesic_vectors.npz by running the reference's own
exact geodesic neighbour lists (tfce_mediation/adjacency.pyx:44-106 over the
header-only library tfce_mediation/lib/geodesic).

Run on a machine that holds a reference checkout (``$TFCE_REFERENCE_ROOT``,
else ``reference`` beside the repository directory) after
``python oracle/build_ref.py`` (which compiles ``adjacency.pyx`` into
oracle/_ref/tfce_mediation/):

    python tests/golden/make_geodesic_golden.py

Meshes (seeded): a radius-10 icosphere of level 3 with 5% radial noise (saddle
vertices), an open cap cut from it (boundary vertices) and a radius-12
icosphere of level 4 with 8% noise.  For each, every source's
``compute_distance_parallel`` list is recorded (sources 0-299 on the level-4
mesh), and for the first mesh also ``compute`` at three thresholds.
"""
from __future__ import annotations

import contextlib
import io
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from tfce_mediation_gb300 import synth  # noqa: E402


def meshes():
    v, f = synth.icosphere(3)
    rng = np.random.default_rng(1)
    sphere = (v * 10.0 * (1.0 + 0.05 * rng.standard_normal((v.shape[0], 1)))).astype(np.float32)
    keep = (v[f][:, :, 2] * 10.0 > -2.0).all(axis=1)
    fc = f[keep]
    used = np.unique(fc)
    remap = -np.ones(v.shape[0], np.int64)
    remap[used] = np.arange(used.shape[0])
    cap_v = sphere[used]
    cap_f = remap[fc].astype(np.int32)
    v4, f4 = synth.icosphere(4)
    rng = np.random.default_rng(2)
    bumpy = (v4 * 12.0 * (1.0 + 0.08 * rng.standard_normal((v4.shape[0], 1)))).astype(np.float32)
    return [("sphere", sphere, f.astype(np.int32), 3.0, None),
            ("cap", cap_v.astype(np.float32), cap_f, 4.0, None),
            ("bumpy", bumpy, f4.astype(np.int32), 2.5, 300)]


def main():
    sys.path.insert(0, os.path.join(ROOT, "oracle", "_ref"))
    from tfce_mediation import adjacency  # the reference's own module, built into oracle/_ref
    out = {}
    for name, v, f, thr, n_src in meshes():
        v = np.ascontiguousarray(v, np.float32)
        f = np.ascontiguousarray(f, np.int32)
        rows = []
        with contextlib.redirect_stdout(io.StringIO()):  # it prints a line per source
            for i in range(v.shape[0] if n_src is None else n_src):
                rows += adjacency.compute_distance_parallel(v, f, thr, i)
        arr = np.asarray(rows, np.float64).reshape(-1, 3)
        out[f"{name}_v"] = v
        out[f"{name}_f"] = f
        out[f"{name}_threshold"] = np.float64(thr)
        out[f"{name}_n_src"] = np.int32(v.shape[0] if n_src is None else n_src)
        out[f"{name}_i"] = arr[:, 0].astype(np.int32)
        out[f"{name}_j"] = arr[:, 1].astype(np.int32)
        out[f"{name}_d"] = arr[:, 2]
        print(name, v.shape[0], "vertices,", arr.shape[0], "pairs below", thr)
    v, f = out["sphere_v"], out["sphere_f"]
    thresholds = np.array([1.5, 2.5, 3.0], np.float32)
    with contextlib.redirect_stdout(io.StringIO()):  # it prints a line per pair
        lists = adjacency.compute(v, f, thresholds)
    out["compute_thresholds"] = thresholds
    for k, lk in enumerate(lists):
        lens = np.array([len(x) for x in lk], np.int64)
        out[f"compute_{k}_off"] = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
        out[f"compute_{k}_idx"] = np.array([y for x in lk for y in x], np.int32)
    np.savez_compressed(os.path.join(HERE, "geodesic_vectors.npz"), **out)


if __name__ == "__main__":
    main()
