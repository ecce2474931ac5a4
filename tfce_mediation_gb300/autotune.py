"""Choice of P (permutations per launch), of the sweep's CTA shape and of the
tensor-core GLM's designs per tile for a permutation engine.

Each candidate (P, CTAs per SM) is timed on the device (CUDA events, after a
warm-up launch) for the GLM + sweep of one batch; the one with the highest
permutations per second wins.  The sweep runs 3 CTAs of 512 threads per SM
(40 registers, the most items in flight) or 2 (64 registers, no spills);
which is faster depends on the segments' sizes and list lengths.  The GLM
runs as the quadratic form (t from the cross products of the centred
designs with the data, where it applies) or with the residual epilogue, whose
tile holds 32 designs (N = 256 MMA columns) or 16 (N = 128); the forms are
timed first, on the largest candidate batch.  Good
values of P fill the persistent sweep grid evenly: one launch has P x
contrasts x signs x segments sweep items spread over the resident CTAs
(tfce_sweep_resident_slots), so P where that count is a multiple of the CTA
count avoids a ragged last wave.  Results are cached per (GPU, n, k, V,
entries, segments, contrasts, signs, precision) in
~/.cache/tfce_mediation_gb300/autotune.json.
"""
from __future__ import annotations

import json
import os

import numpy as np

CACHE = os.path.join(os.path.expanduser("~"), ".cache", "tfce_mediation_gb300", "autotune.json")


def _key(eng):
    import torch
    name = torch.cuda.get_device_name()
    return "|".join(str(x) for x in (name, eng.n, eng.k, eng.V, eng.adj.n_entries, eng.n_seg, eng.C, eng.signs,
                                     getattr(eng, "precision", "fp32")))


def _load():
    try:
        with open(CACHE) as fh:
            return json.load(fh)
    except Exception:
        return {}


def _save(d):
    try:
        os.makedirs(os.path.dirname(CACHE), exist_ok=True)
        tmp = CACHE + f".{os.getpid()}"
        with open(tmp, "w") as fh:
            json.dump(d, fh, indent=1)
        os.replace(tmp, CACHE)
    except OSError:
        pass


def candidates(eng, max_p=256):
    """Batch sizes whose sweep items fill whole waves of the resident CTAs,
    plus the powers of two."""
    try:
        ctas = eng.adj.resident_slots()
    except Exception:  # a tuning hint only: fall back to two CTAs per SM
        import torch
        ctas = 2 * torch.cuda.get_device_properties(0).multi_processor_count
    per_perm = eng.C * eng.signs * eng.n_seg
    out = {16, 32, 64, 128, 256}
    for waves in range(1, 64):
        items = waves * ctas
        if items % per_perm == 0:
            out.add(items // per_perm)
    return sorted(p for p in out if 4 <= p <= max_p)


def time_batch(eng, P, seed=12345, repeats=3):
    """Milliseconds per batch of P permutations (GLM + sweep), device time."""
    import torch
    from .engine import permutations
    from .glm import DesignBatch
    perms = permutations(eng.n, seed, 0, P)
    ops = DesignBatch(eng.X[perms])
    t = torch.empty((P, eng.C, eng.V), device="cuda", dtype=torch.float32)
    mx = torch.empty(P * eng.C * eng.signs * eng.n_seg, device="cuda", dtype=torch.float32)
    eng.tmaps(ops, out=t)
    eng.sweep_max(t, P * eng.C, out=mx)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(repeats):
        eng.tmaps(ops, out=t)
        eng.sweep_max(t, P * eng.C, out=mx)
    b.record()
    torch.cuda.synchronize()
    eng.status()
    return a.elapsed_time(b) / repeats


def time_glm(eng, P, seed=12345, repeats=3):
    """Milliseconds of the GLM of one batch of P permutations (device time)."""
    import torch
    from .engine import permutations
    from .glm import DesignBatch
    ops = DesignBatch(eng.X[permutations(eng.n, seed, 0, P)])
    t = torch.empty((P, eng.C, eng.V), device="cuda", dtype=torch.float32)
    eng.tmaps(ops, out=t)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(repeats):
        eng.tmaps(ops, out=t)
    b.record()
    torch.cuda.synchronize()
    eng.status()
    return a.elapsed_time(b) / repeats


def choose_design_block(eng, P):
    """The tensor-core GLM's form, timed on one batch and set on the engine's
    operands: the quadratic form where the engine's GLM allows it, or the
    residual epilogue with 32 or 16 designs per tile (only 16 exists for more
    than 5 columns).  Returns (design_block, quadratic_form); the timings
    (ms per batch) are kept as the operands' glm_timings."""
    tc = getattr(eng, "_tc", None)
    if tc is None:
        return None, False
    ms = {}
    tc.quadratic_form = True
    if eng._graph_qf():
        ms["qf"] = time_glm(eng, P)
    tc.quadratic_form = False
    res = {}
    for db in ((32, 16) if eng.k <= 5 else (16,)):
        tc.design_block = db
        res[db] = ms[f"res{db}"] = time_glm(eng, P)
    tc.glm_timings = ms
    tc.design_block = min(res, key=res.get)
    tc.quadratic_form = "qf" in ms and ms["qf"] <= res[tc.design_block]
    return tc.design_block, tc.quadratic_form


def choose_batch(eng, max_p=256, use_cache=True, shapes=(3, 2)):
    """Best P and sweep CTA shape for this engine's problem, and the GLM's
    form and designs per tile (cached); the shape is set on the engine's
    adjacency handle and the GLM's choice on its operands, P is returned."""
    key = _key(eng)
    cache = _load() if use_cache else {}
    if key in cache and "ctas_per_sm" in cache[key]:
        eng.adj.set_sweep_shape(int(cache[key]["ctas_per_sm"]))
        if getattr(eng, "_tc", None) is not None:
            if cache[key].get("design_block"):
                eng._tc.design_block = int(cache[key]["design_block"])
            eng._tc.quadratic_form = bool(cache[key].get("quadratic_form", True))
            eng._tc.glm_timings = cache[key].get("glm_ms")
        return int(cache[key]["P"])
    design_block, quadratic_form = choose_design_block(eng, max(candidates(eng, max_p)))
    results = {}
    for shape in shapes:
        eng.adj.set_sweep_shape(shape)
        for P in candidates(eng, max_p):
            try:
                ms = time_batch(eng, P)
            except RuntimeError:
                continue
            results[(shape, P)] = P / ms * 1000.0
    shape, best = max(results, key=results.get)
    eng.adj.set_sweep_shape(shape)
    cache[key] = {"P": best, "ctas_per_sm": shape, "design_block": design_block, "quadratic_form": quadratic_form,
                  "glm_ms": getattr(getattr(eng, "_tc", None), "glm_timings", None),
                  "perm_per_s": {f"{s}x{p}": v for (s, p), v in results.items()}}
    if use_cache:
        _save(cache)
    return best
