"""Benchmark: permutations per second of the GLM + TFCE null-distribution path.

Workload (the headline configuration): two icosphere-L7 hemispheres
(2 x 163,842 = 327,684 vertices, triangle-edge adjacency), n = 350 subjects,
k = 5 regressors (intercept, group, age, sex, covariate), 4 contrasts x (+,-)
x 2 hemispheres = 16 TFCE sweeps per permutation, H = 2, E = 1.  A step is one
batch of P permutations: the tiling of the batch's centred design columns, one
tensor-core GLM launch (glm_tstat_tc_qf, or the form the autotuner keeps) and
one tfce_sweep_batch launch.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--batch P]
  python bench.py --impl reference ...   # the reference's CPU algorithm (oracle port)

Prints one JSON line.  Under torchrun each rank takes a disjoint permutation
range (no data-path collective) and rank 0 reports the whole-job rate.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import shutil
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "perm/s at 327,684 vertices x 350 subj"
WORKLOAD = "config2: 2 x icosphere-L7 (327,684 vertices), n=350, k=5, 4 contrasts x +/- x 2 hemispheres, H=2 E=1"
SEED = 2


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), d.get("bf16_tflops", 1900.0), "measured"
    return 6800.0, 1900.0, "fallback"


def profile_traffic(kernel):
    """DRAM bytes per sweep recorded from an ncu capture in
    profiles/<kernel>*.md (line 'dram_bytes_per_sweep: <number> (<note>)'),
    or (None, None)."""
    d = os.path.join(ROOT, "profiles")
    if not os.path.isdir(d):
        return None, None
    for f in sorted(os.listdir(d)):
        if f.startswith(kernel) and f.endswith(".md"):
            m = re.search(r"dram_bytes_per_sweep:\s*([0-9.eE+]+)\s*\(([^)]*)\)", open(os.path.join(d, f)).read())
            if m:
                return float(m.group(1)), f"{m.group(2)} [profiles/{f}]"
    return None, None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thr = threading.Thread(target=self._read, daemon=True)
            self.thr.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            parts = [p.strip() for p in l.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


# ---------------------------------------------------------------------------
# CPU side: the reference's algorithm (oracle port), one permutation per task
# ---------------------------------------------------------------------------
_W = {}


def _cpu_init(study_args, stash=None):
    from tfce_mediation_gb300 import synth
    st = _unstash_study(stash) if stash else synth.config2(**study_args)
    _W["st"] = st
    from oracle import oracle
    oracle.lib()


def _cpu_perm(p):
    """One permutation as the reference computes it: FP64 tval_int
    (cynumstats.pyx:59-64, chunked over vertices) then, per contrast and sign,
    the sweep of each hemisphere scaled by max/100 and reduced
    (pyfunc.py:107-119)."""
    from oracle import oracle
    st = _W["st"]
    X = st.design()[np.random.RandomState(SEED + p).permutation(st.n)]
    n, k = X.shape
    invXX = np.linalg.inv(X.T @ X)
    t = np.empty((k, st.V), np.float32)
    for v0 in range(0, st.V, 32768):
        y = st.Y[:, v0:v0 + 32768]
        t[:, v0:v0 + 32768] = oracle.tval_int_ref(X, invXX, y, n, k)
    out = []
    for c in range(1, k):
        for s in (1.0, -1.0):
            best = -np.inf
            for h in range(2):
                a, b = st.segments[h], st.segments[h + 1]
                off = st.offsets[a:b + 1] - st.offsets[a]
                idx = st.indices[st.offsets[a]:st.offsets[b]] - a
                best = max(best, oracle.tfce_max_batch(off, idx, t[c, a:b], 2.0, 1.0, sign=s,
                                                       floor_zero=True)[0])
            out.append(best)
    return out


# ---------------------------------------------------------------------------
# The next rows' workloads (--workload cosinor | rmancova | gd_fwhm): the
# tm-models cosinor and RM-ANCOVA permutation statistics on the config-2
# surfaces, and geodesic FWHM smoothing of subject images on one L7 hemisphere
# ---------------------------------------------------------------------------
NEXT = {
    "cosinor": "tm-models cosinor on config-2 surfaces (327,684 vertices), n=350, period 24 h, 1 exog + 1 "
               "covariate: model F, amplitude t, acrophase t, +/-t exog = 5 maps x 2 hemispheres",
    "rmancova": "tm-models RM-ANCOVA (one between-subject factor + covariate) on config-2 surfaces (327,684 "
                "vertices), 120 subjects x 3 intervals: F_a, F_s, F_sa = 3 maps x 2 hemispheres",
    "gd_fwhm": "geodesic FWHM smoothing, one icosphere-L7 hemisphere (163,842 vertices), vertex pairs within "
               "chord 0.038 (~60 per vertex), batches of 64 images",
    "geodesic": "exact geodesic distance lists (adjacency.compute_distance_parallel for every source), one "
                "icosphere-L7 hemisphere (163,842 vertices) scaled to a 0.9 mm mean edge with 0.15 mm radial "
                "noise (saddle vertices), radius 9 mm",
}


def _next_study(kind):
    """Seeded inputs of a next-row workload (deterministic, rebuilt in every process)."""
    from tfce_mediation_gb300 import synth
    rng = np.random.default_rng(7)
    if kind == "cosinor":
        st = synth.config2()
        tv = rng.uniform(0.0, 24.0, st.n)
        from tfce_mediation_gb300.pyfunc import cosinor_design
        X = cosinor_design(tv, [24.0], [st.pred_x[:, 1]], st.pred_x[:, 2])
        return dict(st=st, X=X, tv=tv)
    if kind == "rmancova":
        n, s = 120, 3
        st = synth.config2(n=n * s)
        g = rng.integers(0, 2, n)
        from tfce_mediation_gb300.rm_anova import dummy_code
        Y = st.Y.reshape(s, n, -1) + (0.6 * rng.standard_normal(n))[None, :, None].astype(np.float32)
        return dict(st=st, Y=np.ascontiguousarray(Y.reshape(s * n, -1), np.float32), n=n, s=s,
                    f1=dummy_code(g), subj=dummy_code(np.arange(n), demean=False),
                    cov=rng.standard_normal((n, 1)))
    if kind == "gd_fwhm":
        from scipy.spatial import cKDTree
        v, _ = synth.icosphere(7)
        qp = cKDTree(v).query_pairs(0.038, output_type="ndarray")
        pairs = np.ascontiguousarray(qp[np.lexsort((qp[:, 1], qp[:, 0]))], np.int32)
        dist = np.linalg.norm(v[pairs[:, 0]] - v[pairs[:, 1]], axis=1).astype(np.float32)
        imgs = rng.standard_normal((64, v.shape[0])).astype(np.float32)
        return dict(pairs=pairs, dist=dist, imgs=imgs, V=v.shape[0], sigma=4e-4)
    if kind == "geodesic":
        v, f = synth.icosphere(7)
        e = np.linalg.norm(v[f[:, 0]] - v[f[:, 1]], axis=1).mean()
        r = 0.9 / e
        v = v * r * (1.0 + (0.15 / r) * rng.standard_normal((v.shape[0], 1)))
        return dict(v=np.ascontiguousarray(v, np.float32), f=np.ascontiguousarray(f, np.int32), radius=9.0)
    raise ValueError(kind)


def _next_cpu_init(kind):
    _W["next"] = (kind, _next_study(kind))
    from oracle import oracle
    oracle.lib()


def _segment_max(st, img, s=1.0):
    from oracle import oracle
    best = -np.inf
    for h in range(2):
        a, b = st.segments[h], st.segments[h + 1]
        off = st.offsets[a:b + 1] - st.offsets[a]
        idx = st.indices[st.offsets[a]:st.offsets[b]] - a
        best = max(best, oracle.tfce_max_batch(off, idx, img[a:b], 2.0, 1.0, sign=s, floor_zero=True)[0])
    return best


def _next_cpu_perm(p):
    """One permutation (or, for gd_fwhm, a bounded slice of one image's pair
    scatter) as the reference computes it, with the oracle."""
    from oracle import oracle
    kind, d = _W["next"]
    if kind == "cosinor":
        st = d["st"]
        perm = np.random.RandomState(SEED + p).permutation(st.n)
        r = oracle.glm_cosinor(st.Y, d["tv"], exog=[st.pred_x[:, 1]], dmy_covariates=st.pred_x[:, 2],
                               rand_array=perm, period=[24.0], calc_MESOR=False)
        maps = [r[7], r[9][0], r[10][0], r[11][0], -r[11][0]]
        return [_segment_max(st, np.asarray(m, np.float32)) for m in maps]
    if kind == "rmancova":
        st, n, s = d["st"], d["n"], d["s"]
        rng = np.random.RandomState(SEED + p)
        ra, sh = rng.permutation(n), rng.permutation(n * s)
        F = oracle.rm_ancova_one(d["Y"].reshape(s, n, -1), d["f1"], d["subj"], dmy_covariates=d["cov"],
                                 rand_array=ra, shuffle=sh)
        return [_segment_max(st, np.asarray(m, np.float32)) for m in F]
    if kind == "geodesic":
        oracle.geodesic_lists(d["v"], d["f"], d["radius"], True, p * 100, (p + 1) * 100)
        return []
    sl = slice(p * 20_000, (p + 1) * 20_000)
    oracle.calc_gd_fwhm(d["pairs"][sl], d["dist"][sl], d["imgs"][0], d["sigma"])
    return []


def run_next(args):
    """One JSON line for a next-row workload: whole-job rate through the public
    API with the data resident (the engines' own batched loops), the device
    kernels timed with CUDA events, and the oracle on one core for a bounded
    sample."""
    import multiprocessing as mp
    kind = args.workload
    cpu = None
    if not args.no_cpu_baseline or args.impl == "reference":  # before the first GPU call (spawned pool)
        _one_thread_per_process()
        ctx = mp.get_context("spawn")
        n_cpu = 3 if kind == "gd_fwhm" else 2
        with ctx.Pool(1, initializer=_next_cpu_init, initargs=(kind,)) as pool:
            t0 = time.perf_counter()
            pool.map(_next_cpu_perm, range(n_cpu))
            dt = time.perf_counter() - t0
        if kind == "gd_fwhm":
            M = len(_next_study(kind)["pairs"])
            per_img = dt / (n_cpu * 20_000) * M
            cpu = {"value": 1.0 / per_img, "unit": "images/s", "cores": 1, "kind": "port",
                   "sample": f"{n_cpu} x 20,000 of {M:,} pairs of one image, extrapolated per pair"}
        elif kind == "geodesic":
            cpu = {"value": n_cpu * 100 / dt, "unit": "sources/s", "cores": 1, "kind": "port",
                   "sample": f"{n_cpu} x 100 sources of the same mesh and radius, {dt:.1f} s (the oracle's "
                             "window propagation; the reference's own library runs this propagation and then "
                             "queries every vertex j > i)"}
        else:
            cpu = {"value": n_cpu / dt, "unit": "perm/s", "cores": 1, "kind": "port",
                   "sample": f"{n_cpu} permutations of the same workload, {dt:.1f} s"}
    if args.impl == "reference":  # the oracle port alone, on the line's own metric
        print(json.dumps({"impl": "reference", "metric": cpu["unit"], "value": cpu["value"], "unit": cpu["unit"],
                          "workload": kind, "config": {"workload": NEXT[kind]}, "higher_is_better": True,
                          "cpu_baseline": cpu, "data": "synthetic",
                          "e2e": {"value": cpu["value"], "unit": cpu["unit"], "h2d_bytes_per_step": 0,
                                  "d2h_bytes_per_step": 0}}), flush=True)
        return
    import torch
    from tfce_mediation_gb300 import engine as E
    d = _next_study(kind)
    torch.cuda.set_device(0)
    K = args.steps
    if kind == "gd_fwhm":
        from tfce_mediation_gb300.gd_fwhm import GeodesicSmoother
        from tfce_mediation_gb300.device import ptr
        sm = GeodesicSmoother(d["pairs"], d["dist"], d["sigma"], d["V"])
        x = torch.from_numpy(d["imgs"]).cuda()
        out = torch.empty_like(x)
        B, V, M = x.shape[0], d["V"], sm.M
        st_ = torch.cuda.current_stream().cuda_stream

        def launch():
            sm.lib.gd_fwhm_smooth(ptr(sm.off), ptr(sm.src), ptr(sm.pidx), ptr(sm.w), M, ptr(x), V, B, V,
                                  ptr(out), V, ptr(sm.err), st_)
        for _ in range(args.warmup):
            launch()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(K):
            launch()
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / K
        assert int(sm.err.item()) == 0
        # per image: the gather list (src + pidx, 8 B per entry, 2M entries) and the weights it
        # indexes (4 B per entry), the image gather (4 B per entry) and the output (4V)
        alg_bytes = B * (2 * M * 16 + 4 * V)
        hbm, _, peak_kind = measured_peaks()
        achieved = alg_bytes / (ms / 1e3) / 1e9
        line = {"metric": "images/s", "value": B / (ms / 1e3), "unit": "images/s", "workload": kind,
                "config": {"workload": NEXT[kind], "pairs": int(M), "images_per_launch": B},
                "ms_per_launch": ms, "steps": K, "warmup": args.warmup, "higher_is_better": True,
                "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                             "frac": achieved / hbm, "peak_source": peak_kind + " hbm_gbs",
                             "note": "16 B per gather entry (index, pair, weight, value; every image re-reads "
                                     "the list)"},
                "cpu_baseline": cpu, "gpu_launches": K, "data": "synthetic"}
        print(json.dumps(line), flush=True)
        return
    if kind == "geodesic":
        from tfce_mediation_gb300.geodesic import GeodesicMesh
        t0 = time.perf_counter()
        m = GeodesicMesh(d["v"], d["f"])
        setup_s = time.perf_counter() - t0
        V = d["v"].shape[0]
        for _ in range(args.warmup):
            m.lists(3.0, True, 0, min(V, 4096))
        times, n_pairs = [], 0
        for _ in range(K):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            i, j, dist = m.lists(d["radius"], True)
            times.append(time.perf_counter() - t0)
            n_pairs = int(i.shape[0])
        dt = float(np.median(times))
        t0 = time.perf_counter()
        n3 = int(m.lists(3.0, True)[0].shape[0])
        dt3 = time.perf_counter() - t0
        line = {"metric": "sources/s", "value": V / dt, "unit": "sources/s", "workload": kind,
                "config": {"workload": NEXT[kind], "sources": V, "saddle_vertices": m.n_saddle,
                           "pairs_below_radius": n_pairs},
                "seconds_per_mesh": dt, "mesh_setup_s": setup_s, "steps": K, "warmup": args.warmup,
                "higher_is_better": True,
                "radius_3mm": {"seconds_per_mesh": dt3, "pairs": n3},
                "note": "whole call through GeodesicMesh.lists (propagation of every source on the GPU, lists "
                        "copied back and ordered by (i, j) on the host); one warp per source; bound by the FP64 "
                        "pipe (76% active, profiles/geodesic_warp_lists.md)",
                "cpu_baseline": cpu, "gpu_launches": K, "data": "synthetic"}
        print(json.dumps(line), flush=True)
        return
    st = d["st"]
    if kind == "cosinor":
        from tfce_mediation_gb300.randomise import cosinor_outputs
        eng = E.PermutationEngine(st.Y, d["X"][:, 1:], (st.offsets, st.indices), st.segments, 2.0, 1.0,
                                  batch=args.batch or 256, floor_zero=True, outputs=cosinor_outputs(1, 1, 1))
        P = eng.batch
        eng.run_graph(perms=E.permutations(st.n, SEED, 0, P))  # capture
        torch.cuda.synchronize()
        perms = E.permutations(st.n, SEED, P, P + K * P)
        t0 = time.perf_counter()
        eng.run_graph(perms=perms)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        maps = 5 * 2
    else:
        from tfce_mediation_gb300 import randomise
        from tfce_mediation_gb300.rm_anova import RMAncovaEngine, RMModel
        model = RMModel(d["n"], d["s"], d["f1"], d["subj"], dmy_covariates=d["cov"])
        P = args.batch or 128
        eng = RMAncovaEngine(d["Y"], model, (st.offsets, st.indices), st.segments, 2.0, 1.0, floor_zero=True,
                             batch=P)
        ras, cums = randomise.rm_permutations(d["n"], d["n"] * d["s"], 0, P + K * P, SEED)
        eng.maxima(list(ras[:P]), cums[:P])
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        eng.maxima(list(ras[P:]), cums[P:])
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        maps = 3 * 2
    line = {"metric": "perm/s", "value": K * P / dt, "unit": "perm/s", "workload": kind,
            "config": {"workload": NEXT[kind], "perms_per_step": P, "sweeps_per_perm": maps},
            "ms_per_step": dt / K * 1e3, "steps": K, "warmup": 1, "higher_is_better": True,
            "note": "whole job through the engine's public loop, data resident, host design work included",
            "cpu_baseline": cpu, "data": "synthetic"}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# The other synthetic configurations (sub-lines of the default run): the
# small vertex study, the voxel study, mediation and the multimodal study
# ---------------------------------------------------------------------------
CONFIGS = {
    "config1": "icosphere-L5 (10,242 vertices), n=100, k=3, 2 contrasts x +/-, H=2 E=1",
    "config3": "91x109x91 ellipsoid mask (~230k voxels, 26-neighbour), n=200, k=4, 3 contrasts x +/-, H=2 E=0.5",
    "config4a": "mediation 'M' (Aroian z) on 2 x icosphere-L7 (327,684 vertices), n=350, one sign x 2 hemispheres",
    "config4b": "multimodal: 20 icospheres (levels 5-7) + ~120k-voxel skeleton (~1.4M elements), n=350, k=3, "
                "2 contrasts x +/- x 21 surfaces; icospheres one threshold group (H=2 E=1), skeleton (H=2 E=0.5)",
}
CONFIG_BATCH = {"config1": 512, "config3": 128, "config4a": 128, "config4b": 32}
CONFIG_CPU_PERMS = {"config1": 200, "config3": 4, "config4a": 3, "config4b": 2}


def _config_study(kind):
    from tfce_mediation_gb300 import synth
    if kind == "config1":
        return synth.config1()
    if kind == "config3":
        return synth.config3()
    if kind == "config4a":
        return synth.config4_mediation()
    return synth.config4_mmr()


def _config_groups(st):
    S = len(st.segments) - 1
    return np.array([0] * (S - 1) + [1], np.int32)


def _stash_study(st, d):
    """Write a study where the CPU-baseline worker can map it instead of
    generating it again (the data as .npy, the rest pickled)."""
    import pickle
    os.makedirs(d, exist_ok=True)
    np.save(os.path.join(d, "Y.npy"), st.Y)
    rest = dict(st.__dict__)
    rest.pop("Y")
    with open(os.path.join(d, "study.pkl"), "wb") as fh:
        pickle.dump(rest, fh)


def _unstash_study(d):
    import pickle
    from tfce_mediation_gb300 import synth
    with open(os.path.join(d, "study.pkl"), "rb") as fh:
        rest = pickle.load(fh)
    return synth.Study(Y=np.load(os.path.join(d, "Y.npy"), mmap_mode="r"), **rest)


def _config_cpu_init(kind, stash=None):
    _W["cfg"] = (kind, _unstash_study(stash) if stash else _config_study(kind))
    from oracle import oracle
    oracle.lib()


def _config_cpu_perm(p):
    """One permutation of a configuration as the reference's CPU path
    computes it (the oracle port: FP64 t or Sobel z, C sweeps)."""
    from oracle import oracle
    kind, st = _W["cfg"]
    perm = np.random.RandomState(SEED + p).permutation(st.n)
    segs = [(int(st.segments[h]), int(st.segments[h + 1])) for h in range(len(st.segments) - 1)]

    def sub(a, b):
        return st.offsets[a:b + 1] - st.offsets[a], st.indices[st.offsets[a]:st.offsets[b]] - a

    if kind == "config4a":
        with np.errstate(all="ignore"):
            z = oracle.calc_sobelz("M", st.pred_x[perm, 0], st.depend_y, st.Y.astype(np.float64), st.n)
        z = z.astype(np.float32)
        return [max(oracle.tfce_max_batch(*sub(a, b), z[a:b], 2.0, 1.0, floor_zero=True)[0] for a, b in segs)]
    X = st.design()[perm]
    n, k = X.shape
    invXX = np.linalg.inv(X.T @ X)
    t = np.empty((k, st.V), np.float32)
    for v0 in range(0, st.V, 32768):
        t[:, v0:v0 + 32768] = oracle.tval_int_ref(X, invXX, st.Y[:, v0:v0 + 32768], n, k)
    out = []
    if kind == "config4b":
        groups = _config_groups(st)
        for c in range(1, k):
            for sgn in (1.0, -1.0):
                for g in (0, 1):
                    ss = np.flatnonzero(groups == g)
                    a, b = st.segments[ss[0]], st.segments[ss[-1] + 1]
                    im = (t[c, a:b] * np.float32(sgn)).astype(np.float32)
                    e = oracle.tfce(*sub(a, b), im, float(st.H[ss[0]]), float(st.E[ss[0]]))
                    for s_ in ss:
                        lo, hi = st.segments[s_] - a, st.segments[s_ + 1] - a
                        out.append(float(np.max(e[lo:hi] * (im[lo:hi].max() / np.float32(100)))))
        return out
    E_ = 0.5 if kind == "config3" else 1.0
    for c in range(1, k):
        for sgn in (1.0, -1.0):
            out.append(max(oracle.tfce_max_batch(*sub(a, b), t[c, a:b], 2.0, E_, sign=sgn,
                                                 floor_zero=(kind != "config3"))[0] for a, b in segs))
    return out


def config_cpu_baseline(kind, stash=None):
    import multiprocessing as mp
    _one_thread_per_process()
    ctx = mp.get_context("spawn")
    n_cpu = CONFIG_CPU_PERMS[kind]
    with ctx.Pool(1, initializer=_config_cpu_init, initargs=(kind, stash)) as pool:
        pool.map(_config_cpu_perm, [10_000])  # warm: libraries loaded, caches filled
        t0 = time.perf_counter()
        pool.map(_config_cpu_perm, range(n_cpu))
        dt = time.perf_counter() - t0
    return {"value": n_cpu / dt, "unit": "perm/s", "cores": 1, "kind": "port",
            "sample": f"{n_cpu} permutation(s) of the same workload, {dt:.1f} s, single process"}


def _sweep_bytes(st):
    """Algorithmic bytes of one sweep of every segment: statistic 4V +
    offsets 4(V+1) + entries 4D per segment, summed over the segments."""
    tot = 0
    for h in range(len(st.segments) - 1):
        a, b = int(st.segments[h]), int(st.segments[h + 1])
        tot += 4 * (b - a) + 4 * (b - a + 1) + 4 * int(st.offsets[b] - st.offsets[a])
    return tot


def run_config(kind, args, stash=None):
    """Sub-line of one configuration: whole-job rate through the engine's
    public loop with the data resident, the same through the pipelined entry
    with the data copied from pinned host memory every step (e2e), and the
    sweep kernel's CUDA-event time against its algorithmic bytes."""
    import torch
    from tfce_mediation_gb300 import engine as E
    from tfce_mediation_gb300.device import ptr
    from tfce_mediation_gb300.glm import DesignBatch
    st = _config_study(kind)
    if stash:
        _stash_study(st, stash)
    P = CONFIG_BATCH[kind]
    K = max(2, min(args.steps, 12))
    signs = 1 if kind == "config4a" else 2
    if kind == "config4a":
        eng = E.MediationEngine(st.Y, st.pred_x[:, 0], st.depend_y, "M", (st.offsets, st.indices), st.segments,
                                2.0, 1.0, floor_zero=True, batch=P)
        C, adj = 1, eng.inner.adj
    else:
        kw = dict(threshold_groups=_config_groups(st)) if kind == "config4b" else {}
        seg = None if kind == "config3" else st.segments
        eng = E.PermutationEngine(st.Y, st.pred_x, (st.offsets, st.indices), seg, st.H, st.E,
                                  floor_zero=(kind != "config3"), batch=P, **kw)
        C, adj = eng.C, eng.adj
    S = adj.n_seg
    perms = E.permutations(st.n, SEED, 0, (2 * K + 2) * P)
    run = eng.run if kind == "config4a" else eng.run_graph
    run(perms=perms[:P])  # warm (graph capture)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    run(perms=perms[P:(K + 1) * P])
    torch.cuda.synchronize()
    job_s = time.perf_counter() - t0
    # e2e: new data from pinned host memory every step
    Yh = torch.from_numpy(st.Y).pin_memory()
    # (both engines: run_stream, the pipelined public entry)
    eng.run_stream([(Yh, perms[:P])])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    eng.run_stream((Yh, perms[(K + 1 + s_) * P:(K + 2 + s_) * P]) for s_ in range(K))
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    h2d = st.Y.nbytes
    # the sweep kernel alone: P x C maps (x signs x segments items)
    if kind == "config4a":
        maps = eng.zmaps(perms[:P])
    else:
        maps = eng.tmaps(DesignBatch(eng.X[perms[:P]]))
    out = torch.empty((P * C, signs, S), device="cuda")
    stream = torch.cuda.current_stream()

    def sweep():
        adj.sweep_batch(ptr(maps), eng.V, P * C, signs, None, int(kind != "config3"), ptr(out), None, 0,
                        stream.cuda_stream)
    for _ in range(2):
        sweep()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(3):
        sweep()
    e1.record(stream)
    torch.cuda.synchronize()
    adj.status()
    ms = e0.elapsed_time(e1) / 3
    hbm, _, peak_kind = measured_peaks()
    alg = _sweep_bytes(st) * P * C * signs
    achieved = alg / (ms / 1e3) / 1e9
    line = {"workload": CONFIGS[kind], "metric": "perm/s", "value": K * P / job_s, "unit": "perm/s",
            "perms_per_step": P, "steps": K, "ms_per_step": job_s / K * 1e3,
            "note": "whole job through the engine's public loop (%s), data resident" %
                    ("MediationEngine.run" if kind == "config4a" else "PermutationEngine.run_graph"),
            "e2e": {"value": K * P / e2e_s, "unit": "perm/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(P * C * signs * S * 4),
                    "note": "new data from pinned host memory every step (%s.run_stream)" %
                            ("MediationEngine" if kind == "config4a" else "PermutationEngine")},
            "roofline": {"bound": "hbm", "kernel": "tfce_sweep_kernel", "achieved": achieved, "peak": hbm,
                         "unit": "GB/s", "frac": achieved / hbm, "peak_source": f"{peak_kind} hbm_gbs",
                         "traffic": None, "algorithmic_bytes_per_launch": alg, "ms_per_launch": ms,
                         "sweeps_per_launch": P * C * signs * S}}
    del eng, maps, out
    torch.cuda.empty_cache()
    return line


def dropin_rate(st, P, n_perm=2048):
    """The reference-facing drop-in, timed as a user of the reference's CLI
    would run it: randomise.vertex_regress_run (the
    vertex_tfce_multiple_regression_randomise.py replacement) reading the
    python_temp_<surface> hand-off files of the headline study (Y, masks,
    adjacency lists, per-vertex density weights) and appending the
    per-permutation maxima to the CSVs.  Wall clock of one call over n_perm
    permutations, files, engine set-up and CSV writing included."""
    from types import SimpleNamespace

    from tfce_mediation_gb300 import adjacency as A
    from tfce_mediation_gb300 import randomise
    Vh = st.segments[1] - st.segments[0]
    off, idx = st.offsets[:Vh + 1], st.indices[:st.offsets[Vh]]
    adj = np.empty(Vh, dtype=object)
    for v, l in enumerate(A.from_csr(off, idx)):
        adj[v] = l
    vd = A.vertex_density((off, idx))
    cwd = os.getcwd()
    with tempfile.TemporaryDirectory() as root:
        d = os.path.join(root, "python_temp_area")
        os.makedirs(d)
        mask = np.ones(Vh, bool)
        for name, val in (("merge_y", st.Y), ("num_vertex", st.Y.shape[1]), ("num_vertex_lh", Vh),
                          ("all_vertex", Vh), ("bin_mask_lh", mask), ("bin_mask_rh", mask), ("num_subjects", st.n),
                          ("pred_x", st.pred_x), ("adjac_lh", adj), ("adjac_rh", adj),
                          ("optstfce", np.array([2.0, 1.0])), ("vdensity_lh", vd), ("vdensity_rh", vd)):
            np.save(os.path.join(d, f"{name}.npy"), val, allow_pickle=True)
        os.chdir(root)
        try:
            opts = SimpleNamespace(range=[0, n_perm - 1], surface=["area"], seed=[SEED], specifyvars=None,
                                   exchangeblock=None, batch=P)
            t0 = time.perf_counter()
            randomise.vertex_regress_run(opts)
            dt = time.perf_counter() - t0
            lines = sum(1 for _ in open("output_area/perm_Tstat_area/perm_tstat_con1_TFCE_maxVertex.csv"))
        finally:
            os.chdir(cwd)
    return {"value": n_perm / dt, "unit": "perm/s", "perms": n_perm, "seconds": dt, "csv_lines_per_contrast": lines,
            "note": "randomise.vertex_regress_run (drop-in for vertex_tfce_multiple_regression_randomise.py): "
                    "hand-off files read, engine built, maxima appended to the CSVs, all inside the timed call; "
                    "per-vertex density weights on, so the sweep keeps its potential form"}


def geodesic_sub_line():
    """The exact geodesic neighbour lists (adjacency.compute_distance_parallel
    for every source of one L7 hemisphere, the "geodesic" workload) at the
    3 mm and 9 mm radii the reference's scripts use, through GeodesicMesh.lists;
    wall clock of each whole call.  The one-core rate of the oracle's window
    propagation on this mesh and radius is in bench.py --workload geodesic."""
    from tfce_mediation_gb300.geodesic import GeodesicMesh
    d = _next_study("geodesic")
    m = GeodesicMesh(d["v"], d["f"])
    V = d["v"].shape[0]
    m.lists(3.0, True, 0, min(V, 4096))  # warm-up
    out = {"workload": NEXT["geodesic"], "sources": V, "saddle_vertices": m.n_saddle}
    for r in (3.0, 9.0):
        t0 = time.perf_counter()
        n = int(m.lists(r, True)[0].shape[0])
        dt = time.perf_counter() - t0
        out[f"radius_{r:g}mm"] = {"seconds": dt, "sources_per_s": V / dt, "pairs": n}
    return out


def time_to_fwer(eng, st, n_perm=10_000, seed=99):
    """Wall time from the resident data to the 1-p(FWER) maps of every
    contrast and sign: the plain path (n_perm permutations) and the learned
    tail (300 permutations + the margin fallback), and how far apart the
    two maps are where the plain p <= 0.05."""
    import torch
    from tfce_mediation_gb300 import fwer
    from tfce_mediation_gb300.tail import data
    from tfce_mediation_gb300.tail.surrogate import TailSurrogate, learned_fwer_maps
    _, maps, _ = eng.observed()
    V1 = int(st.segments[1])
    rho = data.neighbour_correlation(torch.from_numpy(st.Y[:, :V1]).cuda(), st.offsets[:V1 + 1],
                                     st.indices[:st.offsets[V1]])
    sur = TailSurrogate()
    images = {c: [maps[c, 0], maps[c, 1]] for c in range(eng.C)}
    learned_fwer_maps(eng, images, rho, 1.0, seed=seed, surrogate=sur)  # warm
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    mx = eng.run_graph(n_perm=n_perm, seed=seed).max(axis=-1)
    # the plain GPU path's own 1-p maps: one device sort of each contrast's null, device lookups
    srt = {c: fwer.sorted_null(mx[:, c, :].reshape(-1)) for c in range(eng.C)}
    plain = {c: [fwer.fwep_presorted(srt[c], maps[c, s_]) for s_ in range(2)] for c in range(eng.C)}
    torch.cuda.synchronize()
    plain_s = time.perf_counter() - t0
    m, info = learned_fwer_maps(eng, images, rho, 1.0, seed=seed, surrogate=sur)
    worst, nsig = 0.0, 0
    for c in range(eng.C):
        for s_ in range(2):
            sig = (1.0 - plain[c][s_]) <= 0.05
            nsig += int(sig.sum())
            if sig.any():
                worst = max(worst, float(np.abs(m[c][s_] - plain[c][s_])[sig].max()))
    return {"plain": {"perms": n_perm, "seconds": plain_s, "maps": 2 * eng.C},
            "learned_tail": {"perms": info["perms"], "seconds": info["seconds"],
                             "fraction_of_plain": info["seconds"] / plain_s, "near_alpha_vertices": info["near_alpha"],
                             "max_abs_dp_where_p_le_0.05": worst, "vertices_p_le_0.05": nsig},
            "note": "1-p(FWER) maps of 4 contrasts x (+,-) of the observed study (calculate_fweP formula); "
                    "learned tail: MLP GPD tail from 300 permutations; vertices whose surrogate or small-sample p lies within "
                    "0.02 of alpha get at least 1,200 more permutations (rounded up to whole batches)"}


def _one_thread_per_process():
    """BLAS / OpenMP thread counts of 1 for the worker processes (spawned
    children read these when their numpy loads), so `cores` processes use
    exactly `cores` host cores, as independent single-threaded jobs do."""
    for var in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS", "NUMEXPR_NUM_THREADS"):
        os.environ[var] = "1"


def cpu_rate(n_perm, cores, study_args, stash=None):
    """perm/s of the oracle port over n_perm permutations on `cores` processes."""
    import multiprocessing as mp
    _one_thread_per_process()
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores, initializer=_cpu_init, initargs=(study_args, stash)) as pool:
        pool.map(_cpu_perm, range(10_000, 10_000 + cores))  # warm: data built, libs loaded
        t0 = time.perf_counter()
        pool.map(_cpu_perm, range(n_perm))
        dt = time.perf_counter() - t0
    return n_perm / dt, dt


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    study_args = {"n": args.n, "level": args.level}
    import multiprocessing as mp
    _one_thread_per_process()
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores, initializer=_cpu_init, initargs=(study_args,)) as pool:
        for w in range(args.warmup):
            pool.map(_cpu_perm, range(10_000 + w * cores, 10_000 + (w + 1) * cores))
        times = []
        for s in range(args.steps):
            t0 = time.perf_counter()
            pool.map(_cpu_perm, range(s * cores, (s + 1) * cores))
            times.append(time.perf_counter() - t0)
    total = sum(times)
    value = args.steps * cores / total
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "perm/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * total / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64/f32",
            "data": "synthetic",
            "config": {"workload": WORKLOAD, "perms_per_step": cores,
                       "note": "oracle port of the reference CPU path (FP64 tval_int + C restatement of "
                               "fast_tfce.hpp), one single-threaded process per host core"},
            "cpu_baseline": {"value": value, "unit": "perm/s", "cores": cores, "kind": "port",
                             "sample": f"{args.steps} steps x {cores} permutations (one per process)"},
            "e2e": {"value": value, "unit": "perm/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GPU side
# ---------------------------------------------------------------------------
def run_gpu(args):
    import torch
    import torch.distributed as dist

    from tfce_mediation_gb300 import engine as E
    from tfce_mediation_gb300 import shard, synth
    from tfce_mediation_gb300.glm import DesignBatch

    t_wall = time.perf_counter()
    ws, rank, local = dist_env()
    if ws > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    t_gen = time.perf_counter()
    st = synth.config2(n=args.n, level=args.level)
    gen_s = time.perf_counter() - t_gen
    eng = E.PermutationEngine(st.Y, st.pred_x, (st.offsets, st.indices), st.segments, 2.0, 1.0,
                              batch="auto" if args.batch == 0 else args.batch, floor_zero=True,
                              precision=args.precision)
    P = eng.batch
    if ws > 1:
        # every rank runs rank 0's batch, so the whole-job count is P x steps x ranks
        pt = torch.tensor([P], device="cuda", dtype=torch.int64)
        dist.broadcast(pt, 0)
        if int(pt.item()) != P:
            P = eng.batch = int(pt.item())
            eng._alloc_buffers()
    C, S, V, n = eng.C, eng.n_seg, eng.V, eng.n
    total_steps = args.warmup + args.steps
    # disjoint permutation ranges per rank
    base = shard.shard_range(ws * total_steps * P, ws, rank)[0]
    perms = [E.permutations(n, SEED, base + s * P, base + (s + 1) * P) for s in range(total_steps)]
    # device-resident design operators (inputs resident before the timed region)
    tc = eng._tc
    qf = eng._graph_qf()
    from tfce_mediation_gb300.device import dev
    if qf:
        ops = []
        for p in perms:
            db = DesignBatch(eng.X[p])
            XR, GI = tc.host_operands_qf(db)
            ops.append((dev(XR), dev(GI), dev(db.invdiag64.astype(np.float32)), dev(db.dof.astype(np.float32))))
        xt_buf = tc.tile_designs_qf(ops[0][0], P, eng.k)
    elif tc is not None:
        ops = []
        for p in perms:
            db = DesignBatch(eng.X[p])
            P8, U, Xt = tc.host_operands(db, centred=eng._centred)
            ops.append((dev(P8), dev(U), dev(Xt), dev(db.invdiag64.astype(np.float32)),
                        dev(db.dof.astype(np.float32))))
        pt_buf = tc.tile_designs(ops[0][0], P, eng.k)
    else:
        ops = [DesignBatch(eng.X[p]).to_device() for p in perms]
    out_max = torch.empty((total_steps, P, C, 2, S), device="cuda")
    stream = torch.cuda.current_stream()
    lib = eng.lib
    from tfce_mediation_gb300 import _lib
    from tfce_mediation_gb300.device import ptr

    def step(s, ev=None):
        if ev is not None:
            ev[0].record(stream)
        if qf:
            XRd, GId, invd, dof = ops[s]
            tc.tile_designs_qf(XRd, P, eng.k, out=xt_buf)
            tc.tstat_qf(xt_buf, GId, invd, dof, P, eng.k, eng._coef, C, eng._tbuf, V)
        elif tc is not None:
            P8d, Ud, Xtd, invd, dof = ops[s]
            tc.tile_designs(P8d, P, eng.k, out=pt_buf)
            tc.stat(0, pt_buf, Ud, Xtd, invd, dof, P, eng.k, eng._coef, C, eng._tbuf, V, centred=eng._centred)
        else:
            pinv, Xp, invd, dof = ops[s]
            _lib.check(lib.glm_tstat(ptr(eng.Yd), V, n, V, ptr(pinv), ptr(Xp), ptr(invd), ptr(dof), P, eng.k,
                                     ptr(eng._coef), C, ptr(eng._tbuf), V, stream.cuda_stream))
        if ev is not None:
            ev[1].record(stream)
        eng.adj.sweep_batch(ptr(eng._tbuf), V, P * C, 2, None, 1, ptr(out_max[s]), None, 0,
                            stream.cuda_stream)
        if ev is not None:
            ev[2].record(stream)

    for s in range(args.warmup):
        step(s)
    torch.cuda.synchronize()
    eng.status()
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    if ws > 1:
        dist.barrier()
    torch.cuda.synchronize()
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        start.record(stream)
        for s in range(args.steps):
            step(args.warmup + s, evs[s])
        stop.record(stream)
        torch.cuda.synchronize()
    eng.status()
    ms = start.elapsed_time(stop)
    glm_ms = [e[0].elapsed_time(e[1]) for e in evs]
    sweep_ms = [e[1].elapsed_time(e[2]) for e in evs]
    ms = shard.max_over_ranks(ms)  # the slowest rank's time
    perms_total = args.steps * P * ws
    value = perms_total / (ms / 1000.0)

    # e2e through the public API from host buffers: Y (pinned) up, permutations
    # generated and design operators formed on the host, maxima down
    Yh = torch.from_numpy(st.Y).pin_memory()
    torch.cuda.synchronize()
    if ws > 1:
        dist.barrier()
    # public API, pipelined: each step hands the engine new pinned host data
    # and its permutations (PermutationEngine.run_stream: captured batch
    # graphs, host preparation of a batch overlapped with the previous one)
    e2e_steps = max(2, min(args.steps, 30))
    pr_all = E.permutations(n, SEED, 10 ** 6 + base, 10 ** 6 + base + e2e_steps * P)
    eng.run_stream([(Yh, pr_all[:P])])  # capture outside the timed region
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    res = eng.run_stream((Yh, pr_all[s * P:(s + 1) * P]) for s in range(e2e_steps))
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0)
    assert sum(r.shape[0] for r in res) == e2e_steps * P
    e2e_value = e2e_steps * P * ws / e2e_s
    # whole job through the public API with Y resident: the engine's own loop
    job_perms = E.permutations(n, SEED, 2 * 10 ** 6 + base, 2 * 10 ** 6 + base + 8 * P)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    eng.run_graph(perms=job_perms)
    torch.cuda.synchronize()
    job_value = job_perms.shape[0] * ws / (time.perf_counter() - t0)
    slot = eng._slots[0]
    h2d = st.Y.nbytes + sum(v.numel() * v.element_size() for k_, v in slot.items()
                            if k_.startswith("h_") and k_ != "h_max")
    d2h = P * C * 2 * S * 4
    dropin = dropin_rate(st, P) if (rank == 0 and not args.no_configs) else None

    if rank != 0:
        dist.destroy_process_group() if ws > 1 else None
        return
    hbm, bf16, peak_kind = measured_peaks()
    bf16_sus = bf16
    try:
        bf16_sus = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))).get("bf16_tflops_sustained", bf16)
    except (OSError, ValueError):
        pass
    # dominant kernel: the sweep.  Algorithmic bytes per sweep: statistic 4V +
    # CSR offsets 4(V+1) + CSR entries 4D (per hemisphere).
    Vh = int(st.segments[1] - st.segments[0])
    Dh = int(st.offsets[st.segments[1]] - st.offsets[st.segments[0]])
    bytes_per_sweep = 4 * Vh + 4 * (Vh + 1) + 4 * Dh
    sweeps_per_launch = P * C * 2 * S
    sweep_avg = float(np.mean(sweep_ms))
    glm_avg = float(np.mean(glm_ms))
    achieved = bytes_per_sweep * sweeps_per_launch / (sweep_avg / 1000) / 1e9
    # work rate of the reference algorithm: sum over thresholds of the active
    # vertices (its per-threshold pass over every active vertex), from a host
    # sample of this step's t maps and the same float threshold recurrence
    upd = []
    tsample = eng._tbuf[: min(P, 4)].reshape(-1, V).cpu().numpy()
    for m in tsample:
        for sgn in (1.0, -1.0):
            for h in range(S):
                a_, b_ = int(st.segments[h]), int(st.segments[h + 1])
                xs = (sgn * m[a_:b_]).astype(np.float32)
                mx = max(float(xs.max()), 0.0)
                if mx <= 0.0:
                    upd.append(0)
                    continue
                T = [np.float32(mx)]
                dT = np.float32(mx) / np.float32(100.0)
                while True:
                    nxt = np.float32(T[-1] - dT)
                    if nxt < 0:
                        break
                    T.append(nxt)
                T = np.asarray(T, np.float32)
                upd.append(int(sum(int(np.count_nonzero(xs > t_)) for t_ in T)))
    updates_per_sweep = float(np.mean(upd))
    per_sweep, traffic_note = profile_traffic("tfce_sweep")
    traffic = None if per_sweep is None else per_sweep * sweeps_per_launch
    clocks = clk.summary()
    if qf:
        # split-BF16 GEMM: 3 MMAs of M=V, N=R rows per design (the k-1 centred
        # columns padded to 4 or 8), K=n_pad; epilogue O(k^2) per vertex and design
        R = tc.qf_rows(eng.k)
        mma_flop = 2.0 * 3 * V * R * tc.qf_padded(P, eng.k) * tc.n_pad
        glm_info = {"precision": "bf16x3", "kernels": "tile_split_kernel + glm_tc_qf_kernel<%d>" % (eng.k - 1),
                    "form": "quadratic (RSS = yy - c'inv(Xc'Xc)c)",
                    "ms_per_launch": glm_avg,
                    "tensor_tflops_issued": mma_flop / (glm_avg / 1000) / 1e12,
                    "tensor_peak_tflops": bf16_sus,
                    "tensor_frac": mma_flop / (glm_avg / 1000) / 1e12 / bf16_sus,
                    "peak_source": f"{peak_kind} bf16_tflops_sustained (kernel timed inside a long step)",
                    "glm_ms_by_form": getattr(tc, "glm_timings", None),
                    "note": "tensor FLOPs count the three split-BF16 products on %d rows per design" % R}
        launches = 3 * args.steps
    elif tc is not None:
        # split-BF16 GEMM: 3 MMAs of M=V, N=8 rows per design, K=n_pad; residual
        # epilogue: (k+1) FP32 FMAs per vertex, design and subject (k with the
        # centred form)
        mma_flop = 2.0 * 3 * V * 8 * tc.padded(P, eng.k) * tc.n_pad
        epi_flop = 2.0 * (eng.k + (0 if eng._centred else 1)) * n * V * P
        glm_info = {"precision": "bf16x3", "kernels": "tile_split_kernel + glm_tc_kernel<%d>" % eng.k,
                    "ms_per_launch": glm_avg,
                    "tensor_tflops_issued": mma_flop / (glm_avg / 1000) / 1e12,
                    "tensor_peak_tflops": bf16_sus,
                    "tensor_frac": mma_flop / (glm_avg / 1000) / 1e12 / bf16_sus,
                    "peak_source": f"{peak_kind} bf16_tflops_sustained (kernel timed inside a long step)",
                    "epilogue_fp32_tflops": epi_flop / (glm_avg / 1000) / 1e12,
                    "glm_ms_by_form": getattr(tc, "glm_timings", None),
                    "note": "tensor FLOPs count the three split-BF16 products on 8 padded rows per design"}
        launches = 3 * args.steps
    else:
        glm_flop = 4.0 * n * eng.k * V * P  # beta + residual passes, FP32 CUDA cores
        glm_info = {"precision": "fp32", "kernels": "glm_tstat_kernel", "ms_per_launch": glm_avg,
                    "achieved_tflops_fp32": glm_flop / (glm_avg / 1000) / 1e12}
        launches = 2 * args.steps
    line = {
        "metric": METRIC, "value": value, "unit": "perm/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32" if tc is None else "f32+bf16x3",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "perms_per_step": P, "sweeps_per_step": sweeps_per_launch,
                   "l2": "inputs larger than L2 (Y 459 MB, t maps %d MB per step)" % (P * C * V * 4 // 2 ** 20),
                   "parallelism": f"replicas over permutation ranges x{ws}",
                   "sweep_ctas_per_sm": getattr(eng.adj, "ctas_per_sm", None),
                   "glm_designs_per_tile": (int(tc.lib.glm_qf_design_block(eng.k)) if qf else
                                            getattr(tc, "design_block", None) if tc is not None else None),
                   "glm_form": "quadratic" if qf else "residual" if tc is not None else "fp32",
                   "data_gen_s": round(gen_s, 1)},
        "e2e": {"value": e2e_value, "unit": "perm/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "steps": e2e_steps,
                "note": "PermutationEngine.run_stream; per step: Y (pinned host) -> HBM and re-tiled, host "
                        "FP64 design inverses (overlapped with the previous step), captured GLM + sweep, "
                        "maxima -> host"},
        "dropin": dropin,
        "job_api": {"value": job_value, "unit": "perm/s",
                    "note": "PermutationEngine.run_graph over %d permutations, Y resident" % (8 * P)},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "kernel": "tfce_sweep_kernel", "achieved": achieved, "peak": hbm,
                     "unit": "GB/s", "frac": achieved / hbm, "peak_source": f"{peak_kind} hbm_gbs",
                     "traffic": traffic, "traffic_note": traffic_note,
                     "algorithmic_bytes_per_launch": bytes_per_sweep * sweeps_per_launch,
                     "ms_per_launch": sweep_avg,
                     "vertex_sweeps_per_s": sweeps_per_launch * Vh / (sweep_avg / 1000),
                     "vertex_threshold_updates_per_sweep": updates_per_sweep,
                     "vertex_threshold_updates_per_s": updates_per_sweep * sweeps_per_launch / (sweep_avg / 1000)},
        "kernels_ms_per_step": {"glm": glm_avg, "tfce_sweep": sweep_avg},
        "glm": glm_info,
        "clocks": clocks,
    }
    stash_root = tempfile.mkdtemp(prefix="tfgb_bench_")
    if not args.no_configs:
        line["time_to_fwer"] = time_to_fwer(eng, st)
        del eng
        torch.cuda.empty_cache()
        line["configs"] = {}
        for kind in CONFIGS:
            line["configs"][kind] = run_config(kind, args, None if args.no_cpu_baseline else
                                               os.path.join(stash_root, kind))
        line["geodesic_lists"] = geodesic_sub_line()
    if not args.no_cpu_baseline:
        cores = 1
        _stash_study(st, os.path.join(stash_root, "config2"))
        v, dt = cpu_rate(args.cpu_perms, cores, {"n": args.n, "level": args.level}, os.path.join(stash_root, "config2"))
        line["cpu_baseline"] = {"value": v, "unit": "perm/s", "cores": cores, "kind": "port",
                                "sample": f"{args.cpu_perms} permutations of the same workload, "
                                          f"{dt:.1f} s, single process"}
        for kind in line.get("configs", {}):
            line["configs"][kind]["cpu_baseline"] = config_cpu_baseline(kind, os.path.join(stash_root, kind))
    shutil.rmtree(stash_root, ignore_errors=True)
    line["bench_wall_s"] = round(time.perf_counter() - t_wall, 1)
    print(json.dumps(line), flush=True)
    if ws > 1:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=60)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--batch", type=int, default=0, help="permutations per step (0: autotuned)")
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=350)
    ap.add_argument("--level", type=int, default=7)
    ap.add_argument("--cpu-perms", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the other configurations' sub-lines and the time-to-FWER block")
    ap.add_argument("--precision", default="bf16x3", choices=["bf16x3", "fp32"],
                    help="GLM arithmetic: tensor-core split BF16 or FP32 CUDA cores")
    ap.add_argument("--workload", default="config2", choices=["config2"] + sorted(NEXT),
                    help="config2: the headline; others: the next rows' workloads (one JSON line each)")
    args = ap.parse_args()
    if args.workload != "config2":
        if args.steps == 60:
            args.steps = 8
        run_next(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
