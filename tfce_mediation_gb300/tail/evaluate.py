"""Evaluate the learned-tail FWER map on the headline study (two
icosphere-L7 hemispheres, n=350, k=5) against the plain GPU path.

    python -m tfce_mediation_gb300.tail.evaluate --full 10000 --out report.json

The plain path runs --full permutations and maps the observed TFCE image with
the reference's calculate_fweP formula; the learned path runs 300 (+ the
margin fallback).  Reported: max |delta p| over vertices with plain p <= 0.05,
wall time of each path, and the same for the classical GPD fit and for the
plain 300-permutation map (what the network gains).
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from .. import engine as E
from .. import synth
from . import data, gpd
from .surrogate import TailSurrogate, learned_fwer


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--full", type=int, default=10000)
    ap.add_argument("--contrast", type=int, default=0)
    ap.add_argument("--weights", default=None)
    ap.add_argument("--out", default=None)
    ap.add_argument("--level", type=int, default=7)
    ap.add_argument("--n", type=int, default=350)
    a = ap.parse_args(argv)
    import torch
    st = synth.config2(n=a.n, level=a.level)
    eng = E.PermutationEngine(st.Y, st.pred_x, (st.offsets, st.indices), st.segments, 2.0, 1.0, batch="auto",
                              floor_zero=True)
    _, tfce_maps, _ = eng.observed()
    obs = tfce_maps[a.contrast, 0]
    V1 = int(st.segments[1])
    rho = data.neighbour_correlation(torch.from_numpy(st.Y[:, :V1]).cuda(), st.offsets[:V1 + 1],
                                     st.indices[:st.offsets[V1]])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    mx = eng.run_graph(n_perm=a.full, seed=99)
    torch.cuda.synchronize()
    plain_s = time.perf_counter() - t0
    null_full = mx[:, a.contrast, :, :].max(axis=-1).reshape(-1)
    plain = gpd.one_minus_p(obs, null_full)
    sig = (1.0 - plain) <= 0.05
    sur = TailSurrogate(a.weights) if a.weights else TailSurrogate()
    rep = {"plain": {"perms": a.full, "seconds": plain_s, "significant_vertices": int(sig.sum())},
           "smoothness": rho}
    for method in ("mlp", "gpd", "empirical"):
        learned_fwer(eng, obs, a.contrast, rho, 1.0, seed=99, method=method, surrogate=sur)  # warm
        m, info = learned_fwer(eng, obs, a.contrast, rho, 1.0, seed=99, method=method, surrogate=sur)
        info["max_abs_dp_where_p_le_0.05"] = float(np.abs(m - plain)[sig].max()) if sig.any() else 0.0
        info["time_fraction_of_plain"] = info["seconds"] / plain_s
        rep[method] = info
    print(json.dumps(rep))
    if a.out:
        with open(a.out, "w") as fh:
            json.dump(rep, fh, indent=1)
    return rep


if __name__ == "__main__":
    main()
