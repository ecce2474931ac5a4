"""Drop-ins for the reference's permutation drivers (L4 scripts).

Each ``*_run(opts)`` reads the same hand-off files the reference's STEP_1
scripts write, runs the permutations through the batched GPU engines, and
appends the same CSV lines in the same order and format:

* vertex_regress_run   -- tmanalysis/vertex_tfce_multiple_regression_randomise.py:56-118
  (python_temp_<surface>/, output_<surface>/perm_Tstat_<surface>/perm_tstat_con<c>_TFCE_maxVertex.csv, %.4f)
* voxel_regress_run    -- tmanalysis/voxel_tfce_multiple_regression_randomise.py:51-120
  (python_temp/, output/perm_Tstat/perm_tstat_con<c>_TFCE_maxVoxel.csv, %1.4f)
* vertex_mediation_run -- tmanalysis/vertex_tfce_mediation_randomise.py:48-92
  (python_temp_med_<surface>/, perm_Zstat_<m>_TFCE_maxVertex.csv)
* voxel_mediation_run  -- tmanalysis/voxel_tfce_mediation_randomise.py:42-77
* mmr_lr_run           -- tm_multisurface/tm_mmr_rand_low_ram_parallel.py:166-207
  (tmi_temp/<s>_*_temp.npy, <path>/perm_maxTFCE_surf<s>_tcon<c>.csv, %f)
* mmr_lr_tmi_run       -- mmr-lr from the TMI file itself (tm_mmr_rand_low_ram.py:140-201 builds the
  tmi_temp/ hand-off the per-surface jobs read): every surface in one launch per batch
* mmr_run              -- tm_multisurface/tm_multimodality_multisurface_regression.py:404-640
  (the in-memory multisurface driver: reads the TMI file; with -p the
  permutation loop of calculate_tfce / calc_mixed_tfce / calculate_mediation_tfce,
  many permutations per launch, output_<name>/output_[med_]stats_<name>.tmi/
  perm_maxTFCE_surf<s>_tcon<c>.csv (or _<m>_zstat.csv), %f; without -p the
  observed maps in stats_<name>.tmi)
* tm_models_glm_run    -- tmanalysis/tm_models_randomise.py:76-92,193-274 (the GLM branch:
  tmtemp_GLM_<surface|volume>/, output_GLM_<..>/perm_GLM/perm_Fstat_<var>_TFCE_max*.csv
  and perm_Tstat_con<c>_TFCE_max*.csv)
* tm_models_cosinor_run, tm_models_rmancova_run, tm_models_mediation_run,
  tm_models_cosinor_mediation_run -- the other tm_models_randomise.py branches;
  tm_models_randomise_run dispatches on the reference's own flags
  (python -m tfce_mediation_gb300.randomise -r 0 99 -s area -glm)

Permutations: the reference seeds each iteration from the clock
(``np.random.seed(int(iter_perm*1000+time()))``); that stays the default.
``opts.seed`` (an added, optional argument) selects the host-seeded stream
``RandomState(seed + iter_perm).permutation(n)`` instead, which makes runs
reproducible and shardable.
"""
from __future__ import annotations

import argparse
import os
from time import time

import numpy as np

from . import engine as E
from .adjacency import induced_csr, concat_csr, to_csr


def _load(path):
    return np.load(path, allow_pickle=True)


def _saved_none(a):
    """Whether a loaded .npy holds a saved None (the reference tests
    `np.all(x) is None`, which numpy >= 2 no longer answers with None for a
    0-d object array)."""
    if a is None:
        return True
    a = np.asarray(a)
    return a.dtype == object and a.ndim == 0 and a.item() is None


def _perm_rows(n, start, stop, seed):
    rows = []
    for it in range(start, stop):
        if seed is None:
            np.random.seed(int(it * 1000 + time()))
            rows.append(np.random.permutation(list(range(n))))
        else:
            rows.append(np.random.RandomState(seed + it).permutation(n))
    return np.asarray(rows)


def _append(path, lines):
    with open(path, "a") as fh:
        fh.write("".join(l + "\n" for l in lines))


def _vd(v, mask):
    if np.isscalar(v) or np.ndim(v) == 0:
        return np.full(int(np.sum(mask)), float(v), np.float32)
    return np.asarray(v, np.float32)[np.asarray(mask, bool)]


def _hemispheres(adj_lh, adj_rh, mask_lh, mask_rh):
    o1, i1 = induced_csr(adj_lh, mask_lh)
    o2, i2 = induced_csr(adj_rh, mask_rh)
    return concat_csr([(o1, i1), (o2, i2)])


def parser_common(ap, surface=True):
    ap.add_argument("-r", "--range", nargs=2, type=int, required=True, metavar=("INT", "INT"))
    if surface:
        ap.add_argument("-s", "--surface", nargs=1, required=True, metavar=("STR",))
    ap.add_argument("--seed", nargs=1, type=int, default=None,
                    help="host-seeded permutation stream RandomState(seed + i) (default: clock seeding)")
    ap.add_argument("--batch", type=int, default=64)
    return ap


def vertex_regress_parser(ap=None):
    ap = parser_common(ap or argparse.ArgumentParser(description="Vertex-wise GLM + TFCE permutations (GPU)"))
    ap.add_argument("-v", "--specifyvars", nargs=2, type=int, metavar=("INT", "INT"))
    ap.add_argument("-e", "--exchangeblock", nargs=1, metavar=("*.csv",))
    return ap


def _designs_for(X, n, start, stop, opts, seed, equal_blocks_only=False):
    """Permuted designs of the reference loop (randomise :90-105), including the
    in-place cumulative -v column permutation and exchange blocks.  The
    vertex/voxel loops always shuffle the blocks' order; the tm-models loops
    (rand_blocks, pyfunc.py:2733-2757, with check_blocks) shuffle it only when
    every block has the same size: pass equal_blocks_only=True for those."""
    out = []
    X = X.copy()
    block_list = None
    if getattr(opts, "exchangeblock", None):
        block_list = np.genfromtxt(opts.exchangeblock[0], dtype=str)
        indexer = np.array(range(len(block_list)))
        sizes = [int(np.sum(block_list == b)) for b in np.unique(block_list)]
        shuffle_blocks = not equal_blocks_only or all(z == sizes[0] for z in sizes)
    for it in range(start, stop):
        if seed is None:
            np.random.seed(int(it * 1000 + time()))
            rng = np.random
        else:
            rng = np.random.RandomState(seed + it)
        if getattr(opts, "specifyvars", None):
            a, b = opts.specifyvars[0], opts.specifyvars[1] + 1
            X[:, a:b] = X[:, a:b][rng.permutation(list(range(n)))]
            out.append(X.copy())
        elif block_list is not None:
            order = rng.permutation(list(np.unique(block_list))) if shuffle_blocks else np.unique(block_list)
            randindex = [rng.permutation(indexer[block_list == blk]) for blk in order]
            out.append(X[np.concatenate(randindex)])
        else:
            out.append(X[rng.permutation(list(range(n)))])
    return np.stack(out)


def _run_designs(eng, designs, batch):
    from .glm import DesignBatch
    res = []
    for b in range(0, designs.shape[0], batch):
        db = DesignBatch(designs[b:b + batch])
        tm = eng.tmaps(db)
        mx = eng.sweep_max(tm, db.G * eng.C)
        res.append(mx.cpu().numpy().reshape(db.G, eng.C, eng.signs, eng.n_seg))
        eng.status()
    return np.concatenate(res)


def vertex_regress_run(opts):
    start, stop = int(opts.range[0]), int(opts.range[1]) + 1
    surface = str(opts.surface[0])
    seed = opts.seed[0] if getattr(opts, "seed", None) else None
    d = "python_temp_%s" % surface
    ny = _load(f"{d}/merge_y.npy")
    num_vertex_lh = int(_load(f"{d}/num_vertex_lh.npy"))
    mask_lh, mask_rh = _load(f"{d}/bin_mask_lh.npy"), _load(f"{d}/bin_mask_rh.npy")
    n = int(_load(f"{d}/num_subjects.npy"))
    pred_x = _load(f"{d}/pred_x.npy")
    adj_lh, adj_rh = _load(f"{d}/adjac_lh.npy"), _load(f"{d}/adjac_rh.npy")
    optstfce = _load(f"{d}/optstfce.npy")
    vd_lh, vd_rh = _load(f"{d}/vdensity_lh.npy"), _load(f"{d}/vdensity_rh.npy")
    off, idx, seg = _hemispheres(adj_lh, adj_rh, mask_lh, mask_rh)
    vd = np.concatenate([_vd(vd_lh, mask_lh), _vd(vd_rh, mask_rh)])
    X = np.column_stack([np.ones(n), pred_x])
    k = X.shape[1]
    if getattr(opts, "specifyvars", None):
        ncon = opts.specifyvars[1] + 1 - opts.specifyvars[0]
    else:
        ncon = k - 1
    eng = E.PermutationEngine(ny, pred_x, (off, idx), seg, float(optstfce[0]), float(optstfce[1]),
                              vdensity=vd, contrasts=list(range(1, ncon + 1)), floor_zero=True,
                              batch=getattr(opts, "batch", 64))
    designs = _designs_for(X, n, start, stop, opts, seed)
    maxima = _run_designs(eng, designs, eng.batch).max(axis=-1)  # (P, C, 2)
    out = "output_%s/perm_Tstat_%s" % (surface, surface)
    os.makedirs(out, exist_ok=True)
    for c in range(ncon):
        lines = []
        for p in range(maxima.shape[0]):
            lines += ["%.4f" % maxima[p, c, 0], "%.4f" % maxima[p, c, 1]]
        _append(os.path.join(out, "perm_tstat_con%d_TFCE_maxVertex.csv" % (c + 1)), lines)
    return maxima


def voxel_regress_run(opts):
    start, stop = int(opts.range[0]), int(opts.range[1]) + 1
    seed = opts.seed[0] if getattr(opts, "seed", None) else None
    n = int(_load("python_temp/num_subjects.npy"))
    ny = _load("python_temp/raw_nonzero_corr.npy").T
    pred_x = _load("python_temp/pred_x.npy")
    adjac = _load("python_temp/adjac.npy")
    ancova = int(_load("python_temp/ancova.npy"))
    optstfce = _load("python_temp/optstfce.npy")
    off, idx = to_csr(adjac)
    X = np.column_stack([np.ones(n), pred_x])
    k = X.shape[1]
    out = "output/perm_Tstat"
    os.makedirs(out, exist_ok=True)
    if ancova == 1:
        return voxel_ftest_run(ny, X, (off, idx), optstfce, start, stop, seed, out)
    if getattr(opts, "specifyvars", None):
        ncon = opts.specifyvars[1] + 1 - opts.specifyvars[0]
    else:
        ncon = k - 1
    eng = E.PermutationEngine(np.ascontiguousarray(ny, np.float32), pred_x, (off, idx), None,
                              float(optstfce[0]), float(optstfce[1]), contrasts=list(range(1, ncon + 1)),
                              batch=getattr(opts, "batch", 64))
    designs = _designs_for(X, n, start, stop, opts, seed)
    maxima = _run_designs(eng, designs, eng.batch)[..., 0]  # (P, C, 2)
    for c in range(ncon):
        lines = []
        for p in range(maxima.shape[0]):
            lines += ["%1.4f" % maxima[p, c, 0], "%1.4f" % maxima[p, c, 1]]
        _append(os.path.join(out, "perm_tstat_con%d_TFCE_maxVoxel.csv" % (c + 1)), lines)
    return maxima


def voxel_ftest_run(ny, X, adjacency, optstfce, start, stop, seed, out):
    """The voxel --ftest (ancova) branch (voxel_…randomise.py:79-89): twice the
    permutations, sqrt(max(F,0)) swept with one sign."""
    import torch

    from .adjacency import AdjacencySet
    from .device import ptr, stream_handle
    from .glm import DesignBatch, glm_fstat
    n = X.shape[0]
    adj = AdjacencySet(adjacency, float(optstfce[0]), float(optstfce[1]))
    adj.set_accumulation("component")
    Yd = torch.from_numpy(np.ascontiguousarray(ny, np.float32)).cuda()
    centre = float(np.mean(ny))
    lines = []
    perms = _perm_rows(n, start, int((stop - 1) * 2 + 1), seed)
    for b in range(0, perms.shape[0], 64):
        db = DesignBatch(X[perms[b:b + 64]])
        F = glm_fstat(Yd, db, centre=centre)
        F = torch.sqrt(torch.clamp(F, min=0.0)).contiguous()
        mx = torch.empty(db.G, device="cuda")
        adj.sweep_batch(ptr(F), F.shape[1], db.G, 1, None, 0, ptr(mx), None, 0, stream_handle())
        adj.status()
        lines += ["%1.4f" % v for v in mx.cpu().numpy()]
    _append(os.path.join(out, "perm_fstat_TFCE_maxVoxel.csv"), lines)
    return np.asarray([float(l) for l in lines])


def mediation_parser(ap=None, surface=True):
    ap = parser_common(ap or argparse.ArgumentParser(description="Mediation + TFCE permutations (GPU)"),
                       surface=surface)
    ap.add_argument("-m", "--medtype", nargs=1, choices=["M", "Y", "I"], required=True)
    return ap


def vertex_mediation_run(opts):
    start, stop = int(opts.range[0]), int(opts.range[1]) + 1
    medtype, surface = str(opts.medtype[0]), str(opts.surface[0])
    seed = opts.seed[0] if getattr(opts, "seed", None) else None
    d = "python_temp_med_%s" % surface
    y = _load(f"{d}/merge_y.npy")
    mask_lh, mask_rh = _load(f"{d}/bin_mask_lh.npy"), _load(f"{d}/bin_mask_rh.npy")
    n = int(_load(f"{d}/num_subjects.npy"))
    pred_x, depend_y = _load(f"{d}/pred_x.npy"), _load(f"{d}/depend_y.npy")
    adj_lh, adj_rh = _load(f"{d}/adjac_lh.npy"), _load(f"{d}/adjac_rh.npy")
    optstfce = _load(f"{d}/optstfce.npy")
    vd_lh, vd_rh = _load(f"{d}/vdensity_lh.npy"), _load(f"{d}/vdensity_rh.npy")
    off, idx, seg = _hemispheres(adj_lh, adj_rh, mask_lh, mask_rh)
    vd = np.concatenate([_vd(vd_lh, mask_lh), _vd(vd_rh, mask_rh)])
    eng = E.MediationEngine(y, pred_x, depend_y, medtype, (off, idx), seg, float(optstfce[0]),
                            float(optstfce[1]), vdensity=vd, floor_zero=True, batch=getattr(opts, "batch", 64))
    maxima = eng.run(perms=_perm_rows(n, start, stop, seed))[:, 0, 0, :].max(axis=-1)
    out = "output_med_%s/perm_SobelZ_%s" % (surface, medtype)
    os.makedirs(out, exist_ok=True)
    _append(os.path.join(out, "perm_Zstat_%s_TFCE_maxVertex.csv" % medtype), ["%.4f" % m for m in maxima])
    return maxima


def voxel_mediation_run(opts):
    start, stop = int(opts.range[0]), int(opts.range[1]) + 1
    medtype = str(opts.medtype[0])
    seed = opts.seed[0] if getattr(opts, "seed", None) else None
    n = int(_load("python_temp/num_subjects.npy"))
    ny = _load("python_temp/raw_nonzero_corr.npy").T
    pred_x, depend_y = _load("python_temp/pred_x.npy"), _load("python_temp/depend_y.npy")
    adjac = _load("python_temp/adjac.npy")
    optstfce = _load("python_temp/optstfce.npy")
    eng = E.MediationEngine(np.ascontiguousarray(ny, np.float32), pred_x, depend_y, medtype, to_csr(adjac), None,
                            float(optstfce[0]), float(optstfce[1]), batch=getattr(opts, "batch", 64))
    maxima = eng.run(perms=_perm_rows(n, start, stop, seed))[:, 0, 0, 0]
    out = "output/perm_SobelZ"
    os.makedirs(out, exist_ok=True)
    _append(os.path.join(out, "perm_Zstat_%s_TFCE_maxVoxel.csv" % medtype), ["%1.4f" % m for m in maxima])
    return maxima


def mmr_lr_run(surf_num, perm_range, seed, path, H, E_, pred_x=None, mediation=None, batch=64):
    """One surface of mmr-lr (tm_mmr_rand_low_ram_parallel.py:166-207): reads
    tmi_temp/<s>_{adjacency,mask,data,vdensity}_temp.npy; the permutation of
    iteration p is RandomState(p + seed) (tm_func.py:147-151) for every surface,
    so the study-wide maxima line up across surfaces."""
    adjacency = _load("tmi_temp/%d_adjacency_temp.npy" % surf_num)
    mask = _load("tmi_temp/%d_mask_temp.npy" % surf_num)
    data = _load("tmi_temp/%d_data_temp.npy" % surf_num)
    vdensity = _load("tmi_temp/%d_vdensity_temp.npy" % surf_num)
    n = data.shape[0]
    m = np.asarray(mask).ravel() == 1
    off, idx = induced_csr(adjacency, m) if m.shape[0] == len(adjacency) and not m.all() else to_csr(adjacency)
    # --noweight saves a one-element array (tm_mmr_rand_low_ram.py:160-163); it broadcasts
    vdensity = np.asarray(vdensity, np.float32)
    if vdensity.size == 1:
        vd = None if float(vdensity.ravel()[0]) == 1.0 else np.full(data.shape[1], vdensity.ravel()[0], np.float32)
    else:
        vd = _vd(vdensity, np.ones(data.shape[1], bool))
    perms = _perm_rows(n, perm_range[0], perm_range[1] + 1, seed)
    floor = not m.all()
    if mediation is None:
        eng = E.PermutationEngine(np.ascontiguousarray(data, np.float32), pred_x, (off, idx), None, H, E_,
                                  vdensity=vd, floor_zero=floor, batch=batch)
        maxima = eng.run(perms=perms)[..., 0]  # (P, C, 2)
        for c in range(maxima.shape[1]):
            lines = []
            for p in range(maxima.shape[0]):
                lines += ["%f" % maxima[p, c, 0], "%f" % maxima[p, c, 1]]
            _append(os.path.join(path, "perm_maxTFCE_surf%d_tcon%d.csv" % (surf_num, c + 1)), lines)
        return maxima
    medtype, mx, dy = mediation
    eng = E.MediationEngine(np.ascontiguousarray(data, np.float32), mx, dy, medtype, (off, idx), None, H, E_,
                            vdensity=vd, floor_zero=floor, batch=batch)
    maxima = eng.run(perms=perms)[:, 0, 0, 0]
    _append(os.path.join(path, "perm_maxTFCE_surf%d_%s_zstat.csv" % (surf_num, medtype)), ["%f" % v for v in maxima])
    return maxima


def mmr_lr_tmi_run(tmifile, perm_range, seed, path, tfce=(2.0, 1.0), pred_x=None, mediation=None,
                   covariates=None, subset=None, setadjacencyobjs=None, assigntfcesettings=None, noweight=False,
                   batch=64):
    """mmr-lr straight from the TMI file, every surface in one launch per
    batch: the data, masks, adjacency sets and density weights that
    tm_mmr_rand_low_ram.py:140-201 writes to tmi_temp/ for its per-surface
    jobs (tm_mmr_rand_low_ram_parallel.py:166-207) are built in memory, and
    each surface keeps its own threshold table and (H, E) (tfce: one pair, or
    one pair per setting with assigntfcesettings), as the per-surface jobs
    sweep them.  Writes <path>/perm_maxTFCE_surf<s>_tcon<c>.csv (or
    _<m>_zstat.csv) for every surface, '%f'; permutation p of every surface is
    RandomState(p + seed) (tm_func.py:147-151).  The zero-filled maximum of
    the low-RAM scaling applies to every surface when any surface mask leaves
    vertices out (it changes only the sign of a zero maximum of a surface
    whose values are all negative).  Returns the maxima (P, C, signs, S)."""
    from . import cynumstats
    from .tmi import read_tm_filetype
    _, image_array, masking_array, _, _, _, _, _, adjacency_array, _, _ = read_tm_filetype(tmifile, verbose=False)
    n_surf = len(masking_array)
    adjacent_range = list(setadjacencyobjs) if setadjacencyobjs else list(range(len(adjacency_array)))
    tf = [float(v) for v in tfce]
    if assigntfcesettings is not None:
        assign = [int(a) for a in assigntfcesettings]
        H = np.array([tf[2 * a] for a in assign], np.float32)
        Es = np.array([tf[2 * a + 1] for a in assign], np.float32)
    else:
        H, Es = np.full(n_surf, tf[0], np.float32), np.full(n_surf, tf[1], np.float32)
    off, idx, seg, vd = _mmr_layout(masking_array, adjacency_array, adjacent_range, noweight)
    data = np.asarray(image_array[0])
    if subset is not None:
        data = data[:, np.isfinite(np.genfromtxt(str(subset), delimiter=","))]
    if covariates is not None:
        covars = np.genfromtxt(covariates, delimiter=",")
        merge_y = cynumstats.resid_covars(np.column_stack([np.ones(len(covars)), covars]), data)
    else:
        merge_y = data.T
    merge_y = np.ascontiguousarray(merge_y, np.float32)
    n = merge_y.shape[0]
    floor = any(np.asarray(m).shape[2] == 1 and not np.asarray(m).all() for m in masking_array)
    perms = _perm_rows(n, perm_range[0], perm_range[1] + 1, seed)
    os.makedirs(path, exist_ok=True)
    if mediation is None:
        eng = E.PermutationEngine(merge_y, pred_x, (off, idx), seg, H, Es, vdensity=vd, floor_zero=floor,
                                  batch=batch)
        maxima = eng.run(perms=perms)  # (P, C, 2, S)
        for s_ in range(n_surf):
            for c in range(maxima.shape[1]):
                lines = []
                for p in range(maxima.shape[0]):
                    lines += ["%f" % maxima[p, c, 0, s_], "%f" % maxima[p, c, 1, s_]]
                _append(os.path.join(path, "perm_maxTFCE_surf%d_tcon%d.csv" % (s_, c + 1)), lines)
        return maxima
    medtype, mx, dy = mediation
    eng = E.MediationEngine(merge_y, mx, dy, medtype, (off, idx), seg, H, Es, vdensity=vd, floor_zero=floor,
                            batch=batch)
    maxima = eng.run(perms=perms)
    for s_ in range(n_surf):
        _append(os.path.join(path, "perm_maxTFCE_surf%d_%s_zstat.csv" % (s_, medtype)),
                ["%f" % v for v in maxima[:, 0, 0, s_]])
    return maxima


def mmr_parser(ap=None):
    """The arguments of tm_multimodality_multisurface_regression.py:33-130
    that the statistics use, plus --seed and --batch."""
    ap = ap or argparse.ArgumentParser(description="Multimodal multisurface regression / mediation (GPU)")
    ap.add_argument("-i_tmi", "--tmifile", nargs=1, required=True, metavar=("*.tmi",))
    group = ap.add_mutually_exclusive_group(required=True)
    group.add_argument("-i", "--input", nargs="+", metavar=("*.csv",))
    group.add_argument("-im", "--inputmediation", nargs=3, metavar=("{I,M,Y}", "*.csv", "*.csv"))
    group.add_argument("-r", "--regressors", nargs=1, metavar=("*.csv",))
    ap.add_argument("-c", "--covariates", nargs=1, metavar=("*.csv",))
    ap.add_argument("-p", "--randomise", nargs=2, type=int, metavar=("INT", "INT"))
    ap.add_argument("-i_name", "--analysisname", nargs=1)
    ap.add_argument("--tfce", nargs="+", default=[2.0, 1.0], type=float)
    ap.add_argument("-sa", "--setadjacencyobjs", nargs="+", type=int)
    ap.add_argument("-st", "--assigntfcesettings", nargs="+", type=int)
    ap.add_argument("--noweight", action="store_true")
    ap.add_argument("--subset", nargs=1)
    ap.add_argument("--seed", nargs=1, type=int, default=None,
                    help="host-seeded permutation stream RandomState(seed + i) (default: clock seeding)")
    ap.add_argument("--batch", type=int, default=64)
    return ap


def _mmr_layout(masking_array, adjacency_array, adjacent_range, noweight):
    """Segments of the in-memory multisurface study: per surface the lists of
    its masked vertices (surfaces: [V,1,1] masks; volumes: the lists are over
    the mask's voxels already), concatenated in position order, and the
    vertex-density weights of the driver
    (tm_multimodality_multisurface_regression.py:449-462)."""
    parts, vd = [], []
    for i, m in enumerate(masking_array):
        m = np.asarray(m)
        adj = adjacency_array[adjacent_range[i]]
        if m.shape[2] == 1:
            parts.append(induced_csr(list(adj), m[:, 0, 0]))
        else:
            parts.append(to_csr(list(adj)))
        if not noweight:
            deg = np.array([len(a) for a in adj], np.float64)
            if m.shape[2] == 1:
                deg = deg[m[:, 0, 0] == True]  # noqa: E712
            vd.append(np.array(1 - deg / deg.max() + deg.mean() / deg.max(), np.float32))
    off, idx, seg = concat_csr(parts)
    return off, idx, seg, (np.concatenate(vd) if vd else None)


def mmr_run(opts):
    """The randomise and observed branches of the in-memory multisurface
    driver on one GPU.  Each launch covers P permutations x contrasts x signs
    x surfaces; with -st every TFCE setting is a threshold group with its own
    (H, E) (calc_mixed_tfce), otherwise all surfaces share one group
    (calculate_tfce's merged adjacency); mediation sweeps the indirect-effect z
    (calculate_mediation_tfce).  Returns the maxima (P, C, signs, surfaces)
    with -p, else the observed maps."""
    from . import cynumstats
    from .tmi import read_tm_filetype, write_tm_filetype
    _, image_array, masking_array, maskname, affine_array, vertex_array, face_array, surfname, adjacency_array, _, _ = \
        read_tm_filetype(opts.tmifile[0], verbose=False)
    n_surf = len(masking_array)
    adjacent_range = (list(opts.setadjacencyobjs) if getattr(opts, "setadjacencyobjs", None)
                      else list(range(len(adjacency_array))))
    if len(adjacent_range) < n_surf:
        raise ValueError("every masking array needs an adjacency set")
    tfce_opts = [float(v) for v in opts.tfce]
    if getattr(opts, "assigntfcesettings", None):
        assign = np.asarray(opts.assigntfcesettings, np.int32)
        if assign.shape[0] != n_surf:
            raise ValueError(f"# of masking arrays ({n_surf}) and of tfce setting assignments ({assign.shape[0]}) "
                             f"must be equal")
        if len(tfce_opts) % 2:
            raise ValueError("--tfce needs H E pairs")
        settings = np.unique(assign)
        groups = np.searchsorted(settings, assign).astype(np.int32)
        H = np.array([tfce_opts[2 * int(a)] for a in assign], np.float32)
        Es = np.array([tfce_opts[2 * int(a) + 1] for a in assign], np.float32)
    else:
        groups = np.zeros(n_surf, np.int32)
        H = np.full(n_surf, tfce_opts[0], np.float32)
        Es = np.full(n_surf, tfce_opts[1], np.float32)
    off, idx, seg, vd = _mmr_layout(masking_array, adjacency_array, adjacent_range, opts.noweight)
    data = np.asarray(image_array[0])
    sub = None
    if getattr(opts, "subset", None):
        sub = np.isfinite(np.genfromtxt(str(opts.subset[0]), delimiter=","))
    medtype = None
    if getattr(opts, "inputmediation", None):
        medtype = opts.inputmediation[0]
        pred_x = np.genfromtxt(opts.inputmediation[1], delimiter=",")
        depend_y = np.genfromtxt(opts.inputmediation[2], delimiter=",")
    elif getattr(opts, "regressors", None):
        pred_x = np.genfromtxt(opts.regressors[0], delimiter=",")
    else:
        cols = [np.genfromtxt(a, delimiter=",") for a in opts.input]
        pred_x = cols[0] if len(cols) == 1 else np.column_stack(cols)
    if sub is not None:
        data = data[:, sub]
    if getattr(opts, "covariates", None) and not getattr(opts, "regressors", None):
        covars = np.genfromtxt(opts.covariates[0], delimiter=",")
        merge_y = cynumstats.resid_covars(np.column_stack([np.ones(len(covars)), covars]), data)
    else:
        merge_y = data.T
    merge_y = np.ascontiguousarray(merge_y, np.float32)
    n = merge_y.shape[0]
    outname = opts.analysisname[0] if getattr(opts, "analysisname", None) else opts.tmifile[0][:-4]
    base = "output_%s" % outname
    os.makedirs(base, exist_ok=True)
    tag = ("med_stats_" if medtype else "stats_") + (outname if outname.endswith("tmi") else outname + ".tmi")
    kw = dict(vdensity=vd, threshold_groups=groups, batch=getattr(opts, "batch", 64))
    if medtype:
        eng = E.MediationEngine(merge_y, pred_x, depend_y, medtype, (off, idx), seg, H, Es, **kw)
    else:
        eng = E.PermutationEngine(merge_y, pred_x, (off, idx), seg, H, Es, **kw)
    if not getattr(opts, "randomise", None):
        if medtype:
            z, tz, _ = eng.observed()
            outdata = np.column_stack((z, tz))
            names = ["SobelZ", "SobelZ_tfce"]
        else:
            tv, maps, _ = eng.observed()
            C = tv.shape[0]
            outdata = np.column_stack((tv.T, maps[:, 0].T, maps[:, 1].T))
            names = (["tstat_con%d" % (i + 1) for i in range(C)] + ["tstat_tfce_con%d" % (i + 1) for i in range(C)]
                     + ["negtstat_tfce_con%d" % (i + 1) for i in range(C)])
        write_tm_filetype(os.path.join(base, tag), image_array=outdata, masking_array=masking_array,
                          maskname=maskname, affine_array=affine_array, vertex_array=vertex_array,
                          face_array=face_array, surfname=surfname, checkname=False, columnids=np.array(names),
                          tmi_history=[])
        return outdata
    start, stop = int(opts.randomise[0]), int(opts.randomise[1]) + 1
    seed = opts.seed[0] if getattr(opts, "seed", None) else None
    perms = _perm_rows(n, start, stop, seed)
    maxima = eng.run(perms=perms)  # (P, C, signs, n_surf)
    out = os.path.join(base, "output_%s" % tag)
    os.makedirs(out, exist_ok=True)
    for s_ in range(n_surf):
        if medtype:
            _append(os.path.join(out, "perm_maxTFCE_surf%d_%s_zstat.csv" % (s_, medtype)),
                    ["%f" % v for v in maxima[:, 0, 0, s_]])
            continue
        for c in range(maxima.shape[1]):
            lines = []
            for p in range(maxima.shape[0]):
                lines += ["%f" % maxima[p, c, 0, s_], "%f" % maxima[p, c, 1, s_]]
            _append(os.path.join(out, "perm_maxTFCE_surf%d_tcon%d.csv" % (s_, c + 1)), lines)
    return maxima


def _tm_models_space(tempdir, surface):
    """Adjacency and sweep settings of a tm-models temp directory
    (tm_models_randomise.py:155-170): surface -> both masked hemispheres as two
    segments with density weights and the zero-fill floor of
    write_perm_maxTFCE_vertex; volume -> one voxel adjacency."""
    if surface:
        mask_lh, mask_rh = _load(f"{tempdir}/mask_lh.npy"), _load(f"{tempdir}/mask_rh.npy")
        adj_lh, adj_rh = _load(f"{tempdir}/adjac_lh.npy"), _load(f"{tempdir}/adjac_rh.npy")
        vd_lh, vd_rh = _load(f"{tempdir}/vdensity_lh.npy"), _load(f"{tempdir}/vdensity_rh.npy")
        off, idx, seg = _hemispheres(adj_lh, adj_rh, mask_lh, mask_rh)
        vd = np.concatenate([_vd(vd_lh, mask_lh), _vd(vd_rh, mask_rh)])
        return off, idx, dict(segments=seg, vdensity=vd, floor_zero=True), "%.4f", "maxVertex"
    off, idx = to_csr(_load(f"{tempdir}/adjac.npy"))
    return off, idx, dict(segments=None), "%1.4f", "maxVoxel"


def tm_models_glm_parser(ap=None):
    ap = ap or argparse.ArgumentParser(description="tm-models GLM permutations (GPU)")
    ap.add_argument("-r", "--range", nargs=2, type=int, required=True, metavar=("INT", "INT"))
    ap.add_argument("-s", "--surface", nargs=1, default=None, metavar=("STR",))
    ap.add_argument("-e", "--exchangeblock", nargs=1, metavar=("*.csv",))
    ap.add_argument("--seed", nargs=1, type=int, default=None,
                    help="host-seeded permutation stream RandomState(seed + i) (default: clock seeding)")
    ap.add_argument("--batch", type=int, default=64)
    return ap


def tm_models_glm_run(opts):
    """The GLM branch of tm_models_randomise.py (:76-92, :193-274): per
    permutation of the design rows, glm_typeI's drop-one F of every exog
    variable (gstat 'f') and/or t of every exog column with both signs
    (gstat 't'), TFCE maxima appended to the reference's CSVs.  F maps run on
    the engine's partial-F mode (one sign, as the reference TFCEs F)."""
    start, stop = int(opts.range[0]), int(opts.range[1]) + 1
    seed = opts.seed[0] if getattr(opts, "seed", None) else None
    surface = str(opts.surface[0]) if getattr(opts, "surface", None) else None
    tempdir = "tmtemp_GLM_%s" % surface if surface else "tmtemp_GLM_volume"
    outdir = "output_GLM_%s/perm_GLM" % surface if surface else "output_GLM_volume/perm_GLM"
    exog_flat = _load(f"{tempdir}/exog_flat.npy")
    exog_shape = [int(c) for c in _load(f"{tempdir}/exog_shape.npy")]
    varnames = _load(f"{tempdir}/varnames.npy")
    gstat = str(_load(f"{tempdir}/gstat.npy"))
    data = _load(f"{tempdir}/data.npy")
    optstfce = _load(f"{tempdir}/optstfce.npy")
    cov = _load(f"{tempdir}/dmy_covariates.npy")
    cov = None if _saved_none(cov) else np.asarray(cov, np.float64)
    n = data.shape[0]
    pred_x = exog_flat if cov is None else np.column_stack([exog_flat, cov])
    X = np.column_stack([np.ones(n), pred_x])
    groups, s0 = [], 1
    for w in exog_shape:
        groups.append((s0, w))
        s0 += w
    numcon = sum(exog_shape)
    H, E_ = float(optstfce[0]), float(optstfce[1])
    off, idx, kw, fmt, suffix = _tm_models_space(tempdir, surface)
    Y = np.ascontiguousarray(data, np.float32)
    batch = getattr(opts, "batch", 64)
    designs = _designs_for(X, n, start, stop, opts, seed, equal_blocks_only=True)
    os.makedirs(outdir, exist_ok=True)
    out = {}

    def reduce(m):
        return m.max(axis=-1) if surface else m[..., 0]

    if gstat != "f":
        eng = E.PermutationEngine(Y, pred_x, (off, idx), H=H, E=E_, contrasts=list(range(1, numcon + 1)),
                                  batch=batch, **kw)
        mt = reduce(_run_designs(eng, designs, eng.batch))  # (P, numcon, 2)
        for c in range(numcon):
            lines = []
            for p in range(mt.shape[0]):
                lines += [fmt % mt[p, c, 0], fmt % mt[p, c, 1]]
            _append(os.path.join(outdir, "perm_Tstat_con%d_TFCE_%s.csv" % (c + 1, suffix)), lines)
        out["t"] = mt
    if gstat != "t":
        eng = E.PermutationEngine(Y, pred_x, (off, idx), H=H, E=E_, f_groups=groups, batch=batch, **kw)
        mf = reduce(_run_designs(eng, designs, eng.batch))  # (P, n_var, 1)
        for j in range(len(groups)):
            _append(os.path.join(outdir, "perm_Fstat_%s_TFCE_%s.csv" % (varnames[j], suffix)),
                    [fmt % mf[p, j, 0] for p in range(mf.shape[0])])
        out["f"] = mf
    return out


def tm_models_cosinor_parser(ap=None):
    return tm_models_glm_parser(ap or argparse.ArgumentParser(description="tm-models cosinor permutations (GPU)"))


def cosinor_outputs(n_period, n_exog, n_cov=0):
    """Output program of the cosinor permutation statistics
    (tm_models_randomise.py:274-372, glm_cosinor with calc_MESOR=False): model F
    (the partial F of every column after the intercept), per period the
    amplitude and acrophase t, then t and -t of every exogenous column; the
    design is [1, (cos, sin) per period, exog columns, covariates]."""
    k = 1 + 2 * n_period + n_exog + n_cov
    outs = [("f", 1, k - 1)]
    for i in range(n_period):
        outs += [("amp", 1 + 2 * i), ("acro", 1 + 2 * i)]
    c0 = 1 + 2 * n_period
    for j in range(n_exog):
        outs += [("t", c0 + j), ("-t", c0 + j)]
    return outs


def tm_models_cosinor_run(opts):
    """The cosinor branch of tm_models_randomise.py (:102-118, :274-372): per
    permutation of the design rows (exchange blocks as rand_blocks), the model
    F, the amplitude and acrophase t of every period and +/- t of every
    exogenous column, each TFCE'd with one sign (the reference sweeps -t as its
    own map into the same CSV); maxima appended to the reference's CSVs
    (perm_Fstat_model, perm_Tstat_amplitude_%2.2f, perm_Tstat_acrophase_%2.2f,
    perm_Tstat_<name> or perm_Tstat_con%d)."""
    from .pyfunc import cosinor_design
    start, stop = int(opts.range[0]), int(opts.range[1]) + 1
    seed = opts.seed[0] if getattr(opts, "seed", None) else None
    surface = str(opts.surface[0]) if getattr(opts, "surface", None) else None
    tempdir = "tmtemp_cosinor_%s" % surface if surface else "tmtemp_cosinor_volume"
    outdir = "output_cosinor_%s/perm_cosinor" % surface if surface else "output_cosinor_volume/perm_cosinor"
    time_var = np.asarray(_load(f"{tempdir}/time_var.npy"), np.float64)
    period = [float(p) for p in np.atleast_1d(_load(f"{tempdir}/period.npy"))]
    exog_flat = _load(f"{tempdir}/exog_flat.npy")
    if _saved_none(exog_flat):
        exog, varnames, numcon = None, [], 0
    else:
        exog_flat = np.asarray(exog_flat, np.float64)
        exog_flat = exog_flat.reshape(exog_flat.shape[0], -1)
        exog = [exog_flat]
        numcon = exog_flat.shape[1]
        varnames = list(_load(f"{tempdir}/varnames.npy"))
    data = _load(f"{tempdir}/data.npy")
    optstfce = _load(f"{tempdir}/optstfce.npy")
    cov = _load(f"{tempdir}/dmy_covariates.npy")
    cov = None if _saved_none(cov) else np.asarray(cov, np.float64).reshape(data.shape[0], -1)
    n = data.shape[0]
    X = cosinor_design(time_var, period, exog, cov)
    outs = cosinor_outputs(len(period), numcon, 0 if cov is None else cov.shape[1])
    H, E_ = float(optstfce[0]), float(optstfce[1])
    off, idx, kw, fmt, suffix = _tm_models_space(tempdir, surface)
    Y = np.ascontiguousarray(data, np.float32)
    batch = getattr(opts, "batch", 64)
    designs = _designs_for(X, n, start, stop, opts, seed, equal_blocks_only=True)
    os.makedirs(outdir, exist_ok=True)
    eng = E.PermutationEngine(Y, X[:, 1:], (off, idx), H=H, E=E_, outputs=outs, batch=batch, **kw)
    m = _run_designs(eng, designs, eng.batch)  # (P, C, 1, S)
    m = (m.max(axis=-1) if surface else m[..., 0])[:, :, 0]  # (P, C)

    def csv(name):
        return os.path.join(outdir, "perm_%s_TFCE_%s.csv" % (name, suffix))

    _append(csv("Fstat_model"), [fmt % v for v in m[:, 0]])
    for i, per in enumerate(period):
        _append(csv("Tstat_amplitude_%2.2f" % per), [fmt % v for v in m[:, 1 + 2 * i]])
        _append(csv("Tstat_acrophase_%2.2f" % per), [fmt % v for v in m[:, 2 + 2 * i]])
    c0 = 1 + 2 * len(period)
    for j in range(numcon):
        name = "Tstat_%s" % varnames[j] if len(varnames) == numcon else "Tstat_con%d" % (j + 1)
        lines = []
        for p in range(m.shape[0]):
            lines += [fmt % m[p, c0 + 2 * j], fmt % m[p, c0 + 2 * j + 1]]
        _append(csv(name), lines)
    return m


def tm_models_rmancova_parser(ap=None):
    ap = tm_models_glm_parser(ap or argparse.ArgumentParser(description="tm-models RM-ANCOVA permutations (GPU)"))
    ap.add_argument("-tfa", "--twobetweenssubjectfactor", action="store_true",
                    help="two between-subject factors (default: one)")
    return ap


def rm_permutations(n, N, start, stop, seed, block_list=None):
    """Subject permutations and cumulative long-row shuffles of the reference's
    RM-ANCOVA loop (tm_models_randomise.py:522-530, 577-585 with
    pyfunc.py:2139 / 1833): per iteration rand_array (np.random.permutation(n),
    or rand_blocks when exchange blocks are given: blocks shuffled only when of
    equal size), then np.random.shuffle of the n*s data rows -- which the
    reference applies to its one data array, so the shuffles compose.
    Returns (ras (P, n), cums (P, N)), cums[i] the long-row order of the data
    seen by iteration i."""
    ras, cums = [], []
    c = np.arange(N)
    if block_list is not None:
        block_list = np.asarray(block_list)
        uniq = np.unique(block_list)
        sizes = [int(np.sum(block_list == b)) for b in uniq]
        equal = all(z == sizes[0] for z in sizes)
        indexer = np.arange(len(block_list))
    for it in range(start, stop):
        if seed is None:
            np.random.seed(int(it * 1000 + time()))
            rng = np.random
        else:
            rng = np.random.RandomState(seed + it)
        if block_list is None:
            ra = rng.permutation(list(range(n)))
        else:
            order = rng.permutation(list(uniq)) if equal else uniq
            ra = np.concatenate([rng.permutation(indexer[block_list == b]) for b in order])
        c = c[rng.permutation(N)]
        ras.append(np.asarray(ra))
        cums.append(c.copy())
    return np.asarray(ras), np.asarray(cums)


def tm_models_rmancova_run(opts):
    """The RM-ANCOVA branches of tm_models_randomise.py (-ofa :135-145, :522-571;
    -tfa :146-156, :574-684): per permutation the F maps of
    reg_rm_ancova_one_bs_factor (F_a, F_s, F_sa) or reg_rm_ancova_two_bs_factor
    (F_a, F_b, F_ab, F_s, F_sa, F_sb, F_sab), each TFCE'd with one sign, maxima
    appended to the reference's CSVs (perm_Fstat_<factor>, perm_Fstat_time,
    perm_Fstat_<factor>.X.time, ...)."""
    from .rm_anova import RMAncovaEngine, RMModel, long_data
    two = bool(getattr(opts, "twobetweenssubjectfactor", False))
    start, stop = int(opts.range[0]), int(opts.range[1]) + 1
    seed = opts.seed[0] if getattr(opts, "seed", None) else None
    surface = str(opts.surface[0]) if getattr(opts, "surface", None) else None
    tag = "rmANCOVA2BS" if two else "rmANCOVA1BS"
    tempdir = "tmtemp_%s_%s" % (tag, surface if surface else "volume")
    outdir = "output_%s_%s/perm_%s" % (tag, surface if surface else "volume", tag)
    f1 = _load(f"{tempdir}/dmy_factor1.npy")
    f2 = _load(f"{tempdir}/dmy_factor2.npy") if two else None
    factors = [str(x) for x in np.atleast_1d(_load(f"{tempdir}/factors.npy"))]
    subj = _load(f"{tempdir}/dmy_subjects.npy")
    dformat = str(np.atleast_1d(_load(f"{tempdir}/dformat.npy"))[0])
    data = _load(f"{tempdir}/data.npy")
    optstfce = _load(f"{tempdir}/optstfce.npy")
    cov = _load(f"{tempdir}/dmy_covariates.npy")
    cov = None if _saved_none(cov) else np.asarray(cov, np.float64)
    n = len(f1)
    endog, n, s = long_data(data, dformat, n)
    model = RMModel(n, s, f1, subj, dmy_factor2=f2, dmy_covariates=cov)
    H, E_ = float(optstfce[0]), float(optstfce[1])
    off, idx, kw, fmt, suffix = _tm_models_space(tempdir, surface)
    block_list = None
    if getattr(opts, "exchangeblock", None):
        block_list = np.genfromtxt(opts.exchangeblock[0], dtype=str)
    ras, cums = rm_permutations(n, n * s, start, stop, seed, block_list)
    os.makedirs(outdir, exist_ok=True)
    eng = RMAncovaEngine(np.ascontiguousarray(endog, np.float32), model, (off, idx), H=H, E=E_,
                         batch=getattr(opts, "batch", 64), **kw)
    m = eng.maxima(list(ras), cums)  # (P, n_f, S)
    m = m.max(axis=-1) if surface else m[..., 0]
    if two:
        names = [factors[0], factors[2], "%s.X.%s" % (factors[0], factors[2]), "time", "%s.X.time" % factors[0],
                 "%s.X.time" % factors[2], "%s.X.%s.X.time" % (factors[0], factors[2])]
    else:
        names = [factors[0], "time", "%s.X.time" % factors[0]]
    for j, nm in enumerate(names):
        _append(os.path.join(outdir, "perm_Fstat_%s_TFCE_%s.csv" % (nm, suffix)), [fmt % v for v in m[:, j]])
    return m


def _subject_perms(n, start, stop, seed, opts):
    """Index rows of the tm-models loops' rand_array: np.random.permutation(n)
    per iteration, or rand_blocks with the equal-size rule when exchange blocks
    are given (seeded RandomState(seed + i), or clock seeding)."""
    ident = np.arange(n, dtype=np.float64)[:, None]
    return _designs_for(ident, n, start, stop, opts, seed, equal_blocks_only=True)[:, :, 0].astype(np.int64)


def tm_models_mediation_run(opts):
    """The mediation branch of tm_models_randomise.py (:93-101, :430-520): per
    permutation dmy_leftvar (and for medtype 'Y' also dmy_rightvar) is
    permuted, path a = t of column 1 of glm_typeI on [1, left, covariates]
    (for 'Y': of dmy_rightvar on it, a scalar), path b = t of column 1 of
    [1, left, right, covariates] ('I') or [1, right, left, covariates] ('M',
    'Y'); Aroian z, TFCE'd with one sign, appended to perm_Zstat_<medtype>.
    The reference reassigns dmy_leftvar = dmy_leftvar[rand_array] inside its
    loop, so the permutations compose: iteration i sees the rows c_i =
    c_{i-1}[rand_array_i]."""
    start, stop = int(opts.range[0]), int(opts.range[1]) + 1
    seed = opts.seed[0] if getattr(opts, "seed", None) else None
    surface = str(opts.surface[0]) if getattr(opts, "surface", None) else None
    tempdir = "tmtemp_mediation_%s" % surface if surface else "tmtemp_mediation_volume"
    outdir = "output_mediation_%s/perm_mediation" % surface if surface else "output_mediation_volume/perm_mediation"
    left = np.asarray(_load(f"{tempdir}/dmy_leftvar.npy"), np.float64)
    right = np.asarray(_load(f"{tempdir}/dmy_rightvar.npy"), np.float64)
    medtype = str(np.atleast_1d(_load(f"{tempdir}/medtype.npy"))[0])
    data = _load(f"{tempdir}/data.npy")
    optstfce = _load(f"{tempdir}/optstfce.npy")
    cov = _load(f"{tempdir}/dmy_covariates.npy")
    cov = None if _saved_none(cov) else np.asarray(cov, np.float64)
    n = left.shape[0]
    H, E_ = float(optstfce[0]), float(optstfce[1])
    off, idx, kw, fmt, suffix = _tm_models_space(tempdir, surface)
    perms = _subject_perms(n, start, stop, seed, opts)
    c = np.arange(n)
    for i in range(perms.shape[0]):
        c = c[perms[i]]
        perms[i] = c
    os.makedirs(outdir, exist_ok=True)
    eng = E.MediationEngine(np.ascontiguousarray(data, np.float32), left, right, medtype, (off, idx), H=H, E=E_,
                            batch=getattr(opts, "batch", 64), covariates=cov, **kw)
    m = eng.run(perms=perms)[:, 0, 0, :]
    m = m.max(axis=-1) if surface else m[:, 0]
    _append(os.path.join(outdir, "perm_Zstat_%s_TFCE_%s.csv" % (medtype, suffix)), [fmt % v for v in m])
    return m


def tm_models_cosinor_mediation_run(opts):
    """The cosinor-mediation branch of tm_models_randomise.py (:119-133,
    :374-428): path a = the unpermuted amplitude t of the mediator's own
    cosinor fit (glm_cosinor of dmy_mediator, first period), path b = t of the
    mediator column in the permuted cosinor design [1, (cos, sin) per period,
    mediator] (the tensor-core GLM's programmed epilogue); Aroian z, TFCE'd with
    one sign, appended to perm_Zstat_<medtype>."""
    from .glm import DesignBatch
    from .pyfunc import ALG, cosinor_design, glm_cosinor
    start, stop = int(opts.range[0]), int(opts.range[1]) + 1
    seed = opts.seed[0] if getattr(opts, "seed", None) else None
    surface = str(opts.surface[0]) if getattr(opts, "surface", None) else None
    tempdir = "tmtemp_medcosinor_%s" % surface if surface else "tmtemp_medcosinor_volume"
    outdir = "output_medcosinor_%s/perm_cosinor" % surface if surface else "output_medcosinor_volume/perm_cosinor"
    time_var = np.asarray(_load(f"{tempdir}/time_var.npy"), np.float64)
    period = [float(p) for p in np.atleast_1d(_load(f"{tempdir}/period.npy"))]
    mediator = np.asarray(_load(f"{tempdir}/dmy_mediator.npy"), np.float64)
    medtype = str(np.atleast_1d(_load(f"{tempdir}/medtype.npy"))[0])
    data = _load(f"{tempdir}/data.npy")
    optstfce = _load(f"{tempdir}/optstfce.npy")
    n = data.shape[0]
    H, E_ = float(optstfce[0]), float(optstfce[1])
    off, idx, kw, fmt, suffix = _tm_models_space(tempdir, surface)
    t_amp_a = float(np.ravel(glm_cosinor(mediator, time_var, period=period)[9][0])[0])
    X = cosinor_design(time_var, period, [mediator])
    c0 = 1 + 2 * len(period)
    perms = _subject_perms(n, start, stop, seed, opts)
    os.makedirs(outdir, exist_ok=True)
    eng = E.PermutationEngine(np.ascontiguousarray(data, np.float32), X[:, 1:], (off, idx), H=H, E=E_,
                              outputs=[("t", c0)], batch=getattr(opts, "batch", 64), **kw)
    from . import _lib
    from .device import dev, ptr, stream_handle
    t = eng.t
    res = []
    for b in range(0, perms.shape[0], eng.batch):
        rows = perms[b:b + eng.batch]
        P = rows.shape[0]
        tb = eng.tmaps(DesignBatch(X[rows]))  # (P, 1, V)
        z = t.empty((P, eng.V), device="cuda", dtype=t.float32)
        tas = dev(np.full(P, t_amp_a, np.float32))
        _lib.check(eng.lib.sobel_combine(None, eng.V, ptr(tas), ptr(tb), eng.V, P, eng.V, ALG["aroian"], ptr(z),
                                         eng.V, stream_handle()))
        mx = eng.sweep_max(z, P)
        res.append(mx.cpu().numpy().reshape(P, 1, eng.n_seg))
        eng.status()
    m = np.concatenate(res)[:, 0, :]
    m = m.max(axis=-1) if surface else m[:, 0]
    _append(os.path.join(outdir, "perm_Zstat_%s_TFCE_%s.csv" % (medtype, suffix)), [fmt % v for v in m])
    return m


def tm_models_randomise_parser(ap=None):
    """The argument parser of tmanalysis/tm_models_randomise.py:30-68 (same
    flags), plus --seed (host-seeded stream) and --batch (permutations per
    launch)."""
    ap = ap or argparse.ArgumentParser(description="tm-models permutations on the GPU")
    ap.add_argument("-r", "--range", nargs=2, type=int, required=True, metavar=("INT", "INT"))
    modality = ap.add_mutually_exclusive_group(required=True)
    modality.add_argument("-s", "--surface", nargs=1, metavar=("STR",))
    modality.add_argument("-v", "--voxel", action="store_true")
    modality.add_argument("-t", "--tmi", action="store_true")
    stat = ap.add_mutually_exclusive_group(required=False)
    for short, long_ in (("-glm", "--generalizedlinearmodel"), ("-med", "--mediation"),
                         ("-ofa", "--onebetweenssubjectfactor"), ("-tfa", "--twobetweenssubjectfactor"),
                         ("-cos", "--cosinor"), ("-mcos", "--cosinormediation")):
        stat.add_argument(short, long_, action="store_true")
    ap.add_argument("-e", "--exchangeblock", nargs=1, metavar=("*.csv",))
    ap.add_argument("--seed", nargs=1, type=int, default=None,
                    help="host-seeded permutation stream RandomState(seed + i) (default: clock seeding)")
    ap.add_argument("--batch", type=int, default=64)
    return ap


def tm_models_randomise_run(opts):
    """tm_models_randomise.run (tmanalysis/tm_models_randomise.py:70-684): the
    branch its statistic flag selects, on the GPU.  The reference has no
    branch for -t (TMI) input; it is refused here."""
    if getattr(opts, "tmi", False):
        raise ValueError("tm_models_randomise has no TMI (-t) branch; use -s SURFACE or -v")
    if getattr(opts, "voxel", False):
        opts.surface = None
    if getattr(opts, "generalizedlinearmodel", False):
        return tm_models_glm_run(opts)
    if getattr(opts, "mediation", False):
        return tm_models_mediation_run(opts)
    if getattr(opts, "onebetweenssubjectfactor", False) or getattr(opts, "twobetweenssubjectfactor", False):
        return tm_models_rmancova_run(opts)
    if getattr(opts, "cosinor", False):
        return tm_models_cosinor_run(opts)
    if getattr(opts, "cosinormediation", False):
        return tm_models_cosinor_mediation_run(opts)
    return None  # no statistic flag: the reference's loop does nothing either


if __name__ == "__main__":  # python -m tfce_mediation_gb300.randomise -r 0 99 -s area -glm
    tm_models_randomise_run(tm_models_randomise_parser().parse_args())
