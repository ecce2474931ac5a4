"""Seeded synthetic studies with the shapes of the benchmark workloads.

The reference ships no data for this path, so every workload is generated:
icosphere surfaces with triangle-edge adjacency, ellipsoidal voxel masks with
26-neighbour adjacency, Gaussian subject data smoothed over the mesh (or the
volume) and re-standardised per vertex, localised effects, and designs with
an intercept plus group / age / sex / covariate columns.  Data come from
``numpy.random.default_rng(seed)``; permutations from
``RandomState(seed + p).permutation(n)`` (the mmr-lr seed convention,
tfce_mediation/tm_func.py:147-151).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .adjacency import concat_csr, mesh_csr, voxel_csr


# ---------------------------------------------------------------------------
# geometry
# ---------------------------------------------------------------------------
def icosphere(level: int):
    """Unit icosphere subdivided `level` times: 10*4^level + 2 vertices."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = np.array([(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t),
                  (0, -1, -t), (0, 1, -t), (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)],
                 np.float64)
    f = np.array([(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9),
                  (5, 11, 4), (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2),
                  (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10),
                  (8, 6, 7), (9, 8, 1)], np.int64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    for _ in range(level):
        F = f.shape[0]
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
        uniq, inv = np.unique(np.sort(e, axis=1), axis=0, return_inverse=True)
        inv = inv.ravel()
        mid = v[uniq[:, 0]] + v[uniq[:, 1]]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        m = v.shape[0] + np.arange(uniq.shape[0])
        a, b, c = m[inv[:F]], m[inv[F:2 * F]], m[inv[2 * F:]]
        v = np.concatenate([v, mid])
        f = np.concatenate([np.stack([f[:, 0], a, c], 1), np.stack([f[:, 1], b, a], 1),
                            np.stack([f[:, 2], c, b], 1), np.stack([a, b, c], 1)])
    return v, f


def bfs_patch(offsets, indices, seed_vertex: int, size: int) -> np.ndarray:
    """The first `size` vertices reached by breadth-first search on the mesh
    (a geodesic patch around `seed_vertex`)."""
    seen = np.zeros(offsets.shape[0] - 1, bool)
    seen[seed_vertex] = True
    order = [seed_vertex]
    frontier = np.array([seed_vertex])
    while len(order) < size and frontier.size:
        nb = np.concatenate([indices[offsets[u]:offsets[u + 1]] for u in frontier])
        nb = np.unique(nb[~seen[nb]])
        seen[nb] = True
        order.extend(nb.tolist())
        frontier = nb
    return np.asarray(order[:size], np.int64)


def ellipsoid_mask(shape=(91, 109, 91), semi=(36.0, 45.0, 34.0)) -> np.ndarray:
    c = [(s - 1) / 2.0 for s in shape]
    g = np.meshgrid(*[np.arange(s) for s in shape], indexing="ij")
    r = sum(((g[i] - c[i]) / semi[i]) ** 2 for i in range(3))
    return r <= 1.0


def skeleton_mask(shape=(120, 140, 120), n_target=120_000, seed=0) -> np.ndarray:
    """A thin 3-D skeleton: nested one-voxel-thick ellipsoidal shells (a stand-in
    for a white-matter skeleton mask), grown until about n_target voxels."""
    c = [(s - 1) / 2.0 for s in shape]
    g = np.meshgrid(*[np.arange(s) for s in shape], indexing="ij")
    mask = np.zeros(shape, bool)
    scale = 0.95
    while mask.sum() < n_target and scale > 0.1:
        semi = [scale * ci for ci in c]
        r = np.sqrt(sum(((g[i] - c[i]) / semi[i]) ** 2 for i in range(3)))
        mask |= np.abs(r - 1.0) * min(semi) < 0.5
        scale -= 0.08
    return mask


# ---------------------------------------------------------------------------
# data
# ---------------------------------------------------------------------------
def smoothing_matrix(offsets, indices):
    """Row-normalised (self + neighbours) averaging operator, scipy CSR."""
    import scipy.sparse as sp
    V = offsets.shape[0] - 1
    deg = np.diff(offsets)
    rows = np.concatenate([np.arange(V), np.repeat(np.arange(V), deg)])
    cols = np.concatenate([np.arange(V), indices.astype(np.int64)])
    w = (1.0 / (1.0 + deg))[rows]
    return sp.csr_matrix((w.astype(np.float32), (rows, cols)), shape=(V, V))


def standardise(Y):
    Y = Y - Y.mean(axis=0, keepdims=True)
    sd = Y.std(axis=0, keepdims=True)
    sd[sd == 0] = 1.0
    return Y / sd


def surface_data(rng, n, offsets, indices, passes):
    """n x V data: i.i.d. N(0,1), `passes` of neighbour averaging, then
    re-standardised per vertex (float32)."""
    V = offsets.shape[0] - 1
    S = smoothing_matrix(offsets, indices)
    Yt = rng.standard_normal((V, n), dtype=np.float32)
    for _ in range(passes):
        Yt = S @ Yt
    return np.ascontiguousarray(standardise(Yt.T.astype(np.float64)).astype(np.float32))


def volume_data(rng, n, mask, fwhm):
    from scipy.ndimage import gaussian_filter
    sigma = fwhm / (2.0 * np.sqrt(2.0 * np.log(2.0)))
    out = np.empty((n, int(mask.sum())), np.float32)
    for s in range(n):
        vol = rng.standard_normal(mask.shape).astype(np.float32)
        out[s] = gaussian_filter(vol, sigma)[mask]
    return np.ascontiguousarray(standardise(out.astype(np.float64)).astype(np.float32))


def zscore(x):
    x = np.asarray(x, np.float64)
    return (x - x.mean()) / x.std()


def binary_half(rng, n):
    g = np.zeros(n)
    g[: n // 2] = 1.0
    return rng.permutation(g)


def permutation(n, seed, p):
    return np.random.RandomState(seed + p).permutation(n)


# ---------------------------------------------------------------------------
# workloads
# ---------------------------------------------------------------------------
@dataclass
class Study:
    """One synthetic study.  Y: n x V float32 (subjects x vertices, concatenated
    segments); pred_x: n x (k-1) regressors (the design is [1, pred_x]);
    offsets/indices: CSR over V (global indices); segments: vertex offsets;
    H/E per segment; vdensity: per-vertex weight or None."""
    name: str
    Y: np.ndarray
    pred_x: np.ndarray
    offsets: np.ndarray
    indices: np.ndarray
    segments: np.ndarray
    H: np.ndarray
    E: np.ndarray
    vdensity: np.ndarray | None = None
    depend_y: np.ndarray | None = None
    info: dict = field(default_factory=dict)

    @property
    def n(self):
        return self.Y.shape[0]

    @property
    def V(self):
        return self.Y.shape[1]

    def design(self):
        return np.column_stack([np.ones(self.n), self.pred_x])


def vertex_study(seed=1, level=5, n=100, passes=5, hemispheres=1, k=3, patches=((300, 0.5, 1),),
                 H=2.0, E=1.0, name="vertex"):
    """Surface GLM study.  patches: (size, effect SD, regressor column) per patch,
    placed round-robin over the hemispheres around seeded vertices."""
    rng = np.random.default_rng(seed)
    v, f = icosphere(level)
    off1, idx1 = mesh_csr(f, v.shape[0])
    V1 = v.shape[0]
    parts, Ys = [], []
    for _ in range(hemispheres):
        parts.append((off1, idx1))
        Ys.append(surface_data(rng, n, off1, idx1, passes))
    off, idx, seg = concat_csr(parts)
    Y = np.ascontiguousarray(np.concatenate(Ys, axis=1))
    cols = [binary_half(rng, n), zscore(rng.uniform(20, 60, n))]
    if k >= 4:
        cols.append(rng.integers(0, 2, n).astype(np.float64))
    if k >= 5:
        cols.append(rng.standard_normal(n))
    pred_x = np.column_stack(cols[: k - 1])
    for i, (size, eff, col) in enumerate(patches):
        h = i % hemispheres
        centre = int(rng.integers(0, V1))
        patch = bfs_patch(off1, idx1, centre, size) + h * V1
        Y[:, patch] += (eff * pred_x[:, col - 1])[:, None].astype(np.float32)
    return Study(name, Y, pred_x, off, idx, seg, np.full(hemispheres, H, np.float32),
                 np.full(hemispheres, E, np.float32), None, None,
                 {"level": level, "passes": passes, "hemispheres": hemispheres})


def config1(seed=1):
    """Icosphere L5 (10,242 vertices), n=100, k=3, one 300-vertex +0.5 SD patch."""
    return vertex_study(seed, level=5, n=100, passes=5, hemispheres=1, k=3,
                        patches=((300, 0.5, 1),), name="config1")


def config2(seed=2, n=350, level=7):
    """Two icospheres L7 (2 x 163,842), n=350, k=5, three 2,000-vertex +0.3 SD patches."""
    return vertex_study(seed, level=level, n=n, passes=5, hemispheres=2, k=5,
                        patches=((2000, 0.3, 1), (2000, 0.3, 1), (2000, 0.3, 2)), name="config2")


def config3(seed=3, n=200, shape=(91, 109, 91), semi=(36.0, 45.0, 34.0), fwhm=3.0):
    """Ellipsoidal voxel mask (~230k voxels), 26-neighbour adjacency, n=200,
    k=4, two r=6 spheres +0.4 SD on the continuous predictor; H=2, E=0.5."""
    rng = np.random.default_rng(seed)
    mask = ellipsoid_mask(shape, semi)
    off, idx = voxel_csr(mask, 26, "pyfunc")
    Y = volume_data(rng, n, mask, fwhm)
    pred_x = np.column_stack([rng.standard_normal(n), zscore(rng.uniform(20, 60, n)),
                              rng.integers(0, 2, n).astype(np.float64)])
    coords = np.array(np.where(mask)).T
    c = np.array([(s - 1) / 2.0 for s in shape])
    for centre in (c + np.array([-12, 10, 5]), c + np.array([14, -15, -6])):
        roi = np.sum((coords - centre) ** 2, axis=1) <= 36.0
        Y[:, roi] += (0.4 * pred_x[:, 0])[:, None].astype(np.float32)
    return Study("config3", Y, pred_x, off, idx, np.array([0, Y.shape[1]], np.int64),
                 np.array([2.0], np.float32), np.array([0.5], np.float32), None, None,
                 {"shape": shape, "voxels": int(mask.sum())})


def config4_mediation(seed=4, n=350, level=7):
    """Binary X, mediator M = surface data on two L7 icospheres, outcome
    Y = 0.3 mean(M_patch) + 0.2 X + N(0,1); medtype 'M'."""
    st = vertex_study(seed, level=level, n=n, passes=5, hemispheres=2, k=3,
                      patches=((2000, 0.3, 1),), name="config4a")
    rng = np.random.default_rng(seed + 1000)
    x = st.pred_x[:, 0]
    V1 = st.V // 2
    patch = bfs_patch(st.offsets[: V1 + 1], st.indices[: st.offsets[V1]], 17, 2000)
    dy = 0.3 * st.Y[:, patch].mean(axis=1) + 0.2 * x + rng.standard_normal(n)
    st.pred_x = x[:, None]
    st.depend_y = dy.astype(np.float64)
    return st


def config4_mmr(seed=5, n=350, levels=None, skeleton_voxels=120_000, passes=5):
    """Multimodal multisurface study: icospheres of uneven levels plus a voxel
    skeleton, concatenated with an offset table; per-segment H/E."""
    rng = np.random.default_rng(seed)
    if levels is None:
        levels = [7] * 6 + [6] * 7 + [5] * 7
    parts, Ys, Hs, Es = [], [], [], []
    meshes = {}
    for lv in levels:
        if lv not in meshes:
            v, f = icosphere(lv)
            meshes[lv] = mesh_csr(f, v.shape[0])
        off1, idx1 = meshes[lv]
        parts.append((off1, idx1))
        Ys.append(surface_data(rng, n, off1, idx1, passes))
        Hs.append(2.0)
        Es.append(1.0)
    if skeleton_voxels:
        m = skeleton_mask(n_target=skeleton_voxels)
        offv, idxv = voxel_csr(m, 26, "mmr")
        parts.append((offv, idxv))
        Ys.append(volume_data(rng, n, m, 2.0))
        Hs.append(2.0)
        Es.append(0.5)
    off, idx, seg = concat_csr(parts)
    Y = np.ascontiguousarray(np.concatenate(Ys, axis=1))
    pred_x = np.column_stack([binary_half(rng, n), zscore(rng.uniform(20, 60, n))])
    return Study("config4b", Y, pred_x, off, idx, seg, np.asarray(Hs, np.float32),
                 np.asarray(Es, np.float32), None, None, {"levels": levels})
