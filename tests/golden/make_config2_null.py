"""Generate tests/golden/config2_null.npz: the FP64 oracle's permutation null of
the headline study (two icosphere-L7 hemispheres, 327,684 vertices, n = 350,
k = 5; synth.config2(seed=2)) for permutations 0..999 of the stream
RandomState(2026 + p).permutation(n).

Per permutation and contrast (design columns 1..4) the + and - maxima of
TFCE * (hemisphere max / 100) over both zero-floored hemispheres, rounded as
the vertex CSV writes them ('%.4f', pyfunc.py:119).  The GPU test rebuilds the
study, runs the same permutations through the engine and compares the two
1-p(FWER) maps.  Run once on any machine (the oracle is plain numpy + C):

    python tests/golden/make_config2_null.py [--perms 1000] [--workers N]
"""
from __future__ import annotations

import argparse
import multiprocessing as mp
import os
import sys
import time
from concurrent.futures import ProcessPoolExecutor

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
SEED = 2026
STUDY_SEED = 2


def _chunk(args):
    lo, hi = args
    sys.path.insert(0, ROOT)
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    from oracle import oracle
    from tfce_mediation_gb300 import synth
    st = synth.config2(seed=STUDY_SEED)
    X = st.design()
    segs = []
    for h in range(2):
        v0, v1 = int(st.segments[h]), int(st.segments[h + 1])
        segs.append((st.offsets[v0:v1 + 1] - st.offsets[v0], st.indices[st.offsets[v0]:st.offsets[v1]] - v0, v0, v1))
    out = np.zeros((hi - lo, 4, 2))
    for i, p in enumerate(range(lo, hi)):
        perm = np.random.RandomState(SEED + p).permutation(st.n)
        t = oracle.tval_fp64(X[perm], st.Y)
        for ci, c in enumerate((1, 2, 3, 4)):
            img = t[c].astype(np.float32)
            for si, s in enumerate((1.0, -1.0)):
                m = max(float(oracle.tfce_max_batch(off, idx, img[v0:v1], 2.0, 1.0, sign=s, floor_zero=True)[0])
                        for off, idx, v0, v1 in segs)
                out[i, ci, si] = float("%.4f" % m)
    return lo, out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--perms", type=int, default=1000)
    ap.add_argument("--workers", type=int, default=os.cpu_count())
    a = ap.parse_args()
    step = max(1, a.perms // (a.workers * 4))
    chunks = [(lo, min(lo + step, a.perms)) for lo in range(0, a.perms, step)]
    t0 = time.time()
    null = np.zeros((a.perms, 4, 2))
    with ProcessPoolExecutor(a.workers, mp_context=mp.get_context("spawn")) as ex:
        for lo, out in ex.map(_chunk, chunks):
            null[lo:lo + out.shape[0]] = out
            print(f"{lo + out.shape[0]} / {a.perms}  ({time.time() - t0:.0f} s)", flush=True)
    path = os.path.join(HERE, "config2_null.npz")
    np.savez_compressed(path, null=null, seed=SEED, study_seed=STUDY_SEED)
    print(f"wrote {path}: {a.perms} permutations in {time.time() - t0:.0f} s")


if __name__ == "__main__":
    main()
