"""Training data for the tail surrogate: null studies synthesised on the GPU
(icosphere meshes, Gaussian subject data smoothed by neighbour averaging,
random designs) and their max-TFCE nulls from the permutation engine."""
from __future__ import annotations

import numpy as np

from ..adjacency import mesh_csr
from .. import engine as E
from .. import synth

_MESH = {}


def mesh(level):
    if level not in _MESH:
        v, f = synth.icosphere(level)
        _MESH[level] = mesh_csr(f, v.shape[0])
    return _MESH[level]


def smooth_gpu(off, idx, n, passes, seed):
    """n subjects of i.i.d. N(0,1) on the mesh, `passes` of neighbour
    averaging (torch sparse on the device: data synthesis only), standardised
    per vertex; returns an (n, V) CUDA float32 tensor."""
    import torch
    V = off.shape[0] - 1
    deg = np.diff(off)
    rows = np.concatenate([np.arange(V), np.repeat(np.arange(V), deg)])
    cols = np.concatenate([np.arange(V), idx.astype(np.int64)])
    w = (1.0 / (1.0 + deg))[rows].astype(np.float32)
    order = np.lexsort((cols, rows))
    crow = np.zeros(V + 1, np.int64)
    np.add.at(crow, rows + 1, 1)
    crow = np.cumsum(crow)
    S = torch.sparse_csr_tensor(torch.from_numpy(crow), torch.from_numpy(cols[order]),
                                torch.from_numpy(w[order]), size=(V, V)).cuda()
    g = torch.Generator(device="cuda")
    g.manual_seed(int(seed))
    Y = torch.randn((V, n), generator=g, device="cuda")
    for _ in range(int(passes)):
        Y = S @ Y
    Y = Y - Y.mean(dim=1, keepdim=True)
    Y = Y / Y.std(dim=1, unbiased=False, keepdim=True).clamp_min(1e-12)
    return Y.t().contiguous()


def neighbour_correlation(Y, off, idx, max_edges=200_000, seed=0):
    """Mean across-subject correlation of neighbouring vertices (a
    smoothness measure observable in any study); Y is (n, V) on the device,
    standardised per vertex."""
    import torch
    V = off.shape[0] - 1
    rows = np.repeat(np.arange(V), np.diff(off))
    rng = np.random.default_rng(seed)
    sel = rng.choice(rows.shape[0], size=min(max_edges, rows.shape[0]), replace=False)
    a = torch.from_numpy(rows[sel]).cuda()
    b = torch.from_numpy(np.asarray(idx, np.int64)[sel]).cuda()
    Ys = (Y - Y.mean(dim=0, keepdim=True)) / Y.std(dim=0, unbiased=False, keepdim=True).clamp_min(1e-12)
    return float((Ys[:, a] * Ys[:, b]).mean().item())


def sample_settings(count, seed=0, levels=(5, 6, 7), level_p=(0.5, 0.35, 0.15)):
    """Seeded synthetic settings: icosphere level, n in [50, 400], k in [2, 6],
    1-10 smoothing passes, E in {0.5, 1}."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        out.append(dict(level=int(rng.choice(levels, p=level_p)), n=int(rng.integers(50, 401)),
                        k=int(rng.integers(2, 7)), passes=int(rng.integers(1, 11)),
                        E=float(rng.choice([0.5, 1.0])), hemispheres=int(rng.choice([1, 2], p=[0.6, 0.4])),
                        seed=int(seed * 100_000 + i)))
    return out


def null_for_setting(s, n_perm, batch=128):
    """(null maxima (2 n_perm,), smoothness, V) of one setting: contrast 1,
    both signs, in permutation order (+ then - per permutation); with two
    hemispheres the maximum is taken over both, as the vertex path does."""
    import torch
    from ..adjacency import concat_csr
    off1, idx1 = mesh(s["level"])
    H = s.get("hemispheres", 1)
    Ys = [smooth_gpu(off1, idx1, s["n"], s["passes"], s["seed"] + 1000 * h) for h in range(H)]
    Y = torch.cat(Ys, dim=1).contiguous() if H > 1 else Ys[0]
    off, idx, seg = concat_csr([(off1, idx1)] * H)
    rng = np.random.default_rng(s["seed"] + 7)
    cols = [synth.binary_half(rng, s["n"])] + [rng.standard_normal(s["n"]) for _ in range(s["k"] - 2)]
    pred_x = np.column_stack(cols)
    eng = E.PermutationEngine(Y, pred_x, (off, idx), seg, 2.0, s["E"], contrasts=[1], batch=batch)
    full = n_perm // batch * batch  # whole batches through the captured graphs, the rest as one short batch
    parts = [eng.run_graph(n_perm=full, seed=s["seed"] + 11)] if full else []
    if n_perm > full:
        parts.append(eng.run(start=full, stop=n_perm, seed=s["seed"] + 11))
    mx = np.concatenate(parts)  # (P, 1, 2, H)
    null = mx[:, 0, :, :].max(axis=-1).reshape(-1).astype(np.float64)
    return null, neighbour_correlation(Ys[0], off1, idx1), off.shape[0] - 1
