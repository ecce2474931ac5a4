"""The learned-tail FWER path on the headline study at its full size (two
icosphere-L7 hemispheres, 327,684 vertices, n = 350, k = 5): for three seeds
and all four contrasts x (+, -), the 1-p(FWER) maps from 300 permutations
plus the margin fallback (vertices whose surrogate or small-sample p lies
within 0.02 of alpha get at least 1,200 more permutations, rounded up to
whole batches) reproduce the plain 10,000-permutation maps within
0.01 wherever the plain p <= 0.05, in at most a fifth of the plain path's
wall time (the bar stated for the learned path)."""
import time

import numpy as np
import pytest

from tfce_mediation_gb300 import engine as E
from tfce_mediation_gb300 import synth

pytestmark = pytest.mark.gpu


def test_learned_tail_reproduces_plain_fwer_maps():
    import torch
    from tfce_mediation_gb300 import fwer
    from tfce_mediation_gb300.tail import data
    from tfce_mediation_gb300.tail.surrogate import TailSurrogate, learned_fwer_maps
    st = synth.config2()
    eng = E.PermutationEngine(st.Y, st.pred_x, (st.offsets, st.indices), st.segments, 2.0, 1.0, batch=256,
                              floor_zero=True)
    _, maps, _ = eng.observed()
    V1 = int(st.segments[1])
    rho = data.neighbour_correlation(torch.from_numpy(st.Y[:, :V1]).cuda(), st.offsets[:V1 + 1],
                                     st.indices[:st.offsets[V1]])
    sur = TailSurrogate()
    images = {c: [maps[c, 0], maps[c, 1]] for c in range(eng.C)}
    learned_fwer_maps(eng, images, rho, 1.0, seed=1, surrogate=sur)  # graph capture, warm caches
    for seed in (99, 123, 31):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        mx = eng.run_graph(n_perm=10_000, seed=seed).max(axis=-1)
        srt = {c: fwer.sorted_null(mx[:, c, :].reshape(-1)) for c in range(eng.C)}
        plain = {c: [fwer.fwep_presorted(srt[c], maps[c, s]) for s in range(2)] for c in range(eng.C)}
        torch.cuda.synchronize()
        plain_s = time.perf_counter() - t0
        m, info = learned_fwer_maps(eng, images, rho, 1.0, seed=seed, surrogate=sur)
        worst, nsig = 0.0, 0
        for c in range(eng.C):
            for s in range(2):
                sig = (1.0 - plain[c][s]) <= 0.05
                nsig += int(sig.sum())
                if sig.any():
                    worst = max(worst, float(np.abs(m[c][s] - plain[c][s])[sig].max()))
        frac = info["seconds"] / plain_s
        print(f"seed {seed}: max |dp| {worst:.4f} over {nsig} vertices with p <= 0.05; "
              f"{info['perms']} permutations, {info['seconds']:.2f} s = {frac:.3f} of plain {plain_s:.2f} s")
        assert nsig > 0
        assert worst <= 0.01, worst
        assert frac <= 0.2, frac
