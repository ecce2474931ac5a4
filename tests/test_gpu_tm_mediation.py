"""tm-models mediation drivers on the GPU (tm_models_randomise.py -med and
-mcos branches): CSV lines against the oracle pipeline (FP64 path t values,
Aroian z, C sweep) on the same host-seeded permutations -- composed over the
loop for -med, as the reference reassigns the permuted variable.

Bar: per-permutation max-TFCE within 1e-3 relative (+1e-3)."""
import argparse

import numpy as np
import pytest

from oracle import oracle
from tfce_mediation_gb300 import adjacency as A
from tfce_mediation_gb300 import randomise

pytestmark = pytest.mark.gpu


def _volume(tmp_path, name, rng, n):
    mask = np.zeros((9, 8, 7), bool)
    mask[1:8, 1:7, 1:6] = True
    off, idx = A.voxel_csr(mask, 26, "pyfunc")
    V = int(mask.sum())
    d = tmp_path / name
    d.mkdir()
    adj = np.empty(V, dtype=object)
    for v in range(V):
        adj[v] = np.asarray(idx[off[v]:off[v + 1]], np.int64)
    np.save(d / "adjac.npy", adj, allow_pickle=True)
    np.save(d / "optstfce.npy", np.array([2.0, 0.5]))
    return d, off, idx, V


@pytest.mark.parametrize("medtype", ["I", "M", "Y"])
def test_tm_models_mediation_driver(tmp_path, monkeypatch, medtype):
    rng = np.random.default_rng(50 + ord(medtype))
    n = 40
    d, off, idx, V = _volume(tmp_path, "tmtemp_mediation_volume", rng, n)
    left = rng.standard_normal(n)
    right = 0.6 * left + rng.standard_normal(n)
    cov = rng.standard_normal((n, 1))
    data = rng.standard_normal((n, V)).astype(np.float32)
    data[:, :70] += (0.8 * right)[:, None].astype(np.float32)
    np.save(d / "dmy_leftvar.npy", left)
    np.save(d / "dmy_rightvar.npy", right)
    np.save(d / "medtype.npy", np.array([medtype]))
    np.save(d / "data.npy", data)
    np.save(d / "dmy_covariates.npy", cov)
    monkeypatch.chdir(tmp_path)
    opts = argparse.Namespace(range=[0, 5], surface=None, exchangeblock=None, seed=[13], batch=4)
    randomise.tm_models_mediation_run(opts)
    csv = np.loadtxt(tmp_path / "output_mediation_volume" / "perm_mediation" / f"perm_Zstat_{medtype}_TFCE_maxVoxel.csv")
    c = np.arange(n)
    one = np.ones((n, 1))
    for p in range(6):
        c = c[np.random.RandomState(13 + p).permutation(n)]
        x = left[c]
        y = right[c] if medtype == "Y" else right
        if medtype == "Y":
            ta = oracle.tval_fp64(np.column_stack([one, x, cov]), y[:, None])[1, 0]
        else:
            ta = oracle.tval_fp64(np.column_stack([one, x, cov]), data)[1]
        Xb = np.column_stack([one, x, y, cov]) if medtype == "I" else np.column_stack([one, y, x, cov])
        tb = oracle.tval_fp64(Xb, data)[1]
        z = oracle.indirect(ta, tb).astype(np.float32)
        ref = oracle.tfce_max_batch(off, idx, z, 2.0, 0.5)[0]
        assert abs(csv[p] - ref) <= 1e-3 * abs(ref) + 1e-3, (medtype, p, csv[p], ref)


def test_tm_models_cosinor_mediation_driver(tmp_path, monkeypatch):
    rng = np.random.default_rng(61)
    n = 48
    d, off, idx, V = _volume(tmp_path, "tmtemp_medcosinor_volume", rng, n)
    tv = rng.uniform(0.0, 24.0, n)
    med = 1.5 * np.cos(2 * np.pi * (tv - 4.0) / 24.0) + 0.5 * rng.standard_normal(n)
    data = rng.standard_normal((n, V)).astype(np.float32)
    data[:, :60] += (0.7 * med)[:, None].astype(np.float32)
    np.save(d / "time_var.npy", tv)
    np.save(d / "period.npy", np.array([24.0]))
    np.save(d / "dmy_mediator.npy", med)
    np.save(d / "medtype.npy", np.array(["M"]))
    np.save(d / "data.npy", data)
    monkeypatch.chdir(tmp_path)
    opts = argparse.Namespace(range=[0, 4], surface=None, exchangeblock=None, seed=[17], batch=3)
    randomise.tm_models_cosinor_mediation_run(opts)
    csv = np.loadtxt(tmp_path / "output_medcosinor_volume" / "perm_cosinor" / "perm_Zstat_M_TFCE_maxVoxel.csv")
    ta = oracle.glm_cosinor(med[:, None], tv, period=[24.0])[9][0, 0]
    for p in range(5):
        perm = np.random.RandomState(17 + p).permutation(n)
        tb = oracle.glm_cosinor(data, tv, exog=[med], rand_array=perm, period=[24.0], calc_MESOR=False)[11][0]
        z = oracle.indirect(ta, tb).astype(np.float32)
        ref = oracle.tfce_max_batch(off, idx, z, 2.0, 0.5)[0]
        assert abs(csv[p] - ref) <= 1e-3 * abs(ref) + 1e-3, (p, csv[p], ref)
