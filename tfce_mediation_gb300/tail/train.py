"""Train the tail surrogate on the GPU.

    python -m tfce_mediation_gb300.tail.train --settings 500 --full 1500 --out weights.npz

Each seeded setting (data.sample_settings) gets a full null of --full
permutations from the GPU engine; its tail (u, xi, sigma: the 90% quantile
and a GPD fit of the excess) is the target.  Inputs are the features of
disjoint --small-permutation subsets of the same null (gpd.features), so one
setting gives several training rows.  The MLP is trained by the project's own
kernels (tail/mlp.py, csrc/mlp.cu); the held-out settings report the p-value
error of the network against the classical GPD fit of the same small sample.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import data, gpd
from .mlp import MLP


def build_rows(settings, nulls, small):
    X, Y, meta = [], [], []
    for s, (null, rho, V) in zip(settings, nulls):
        per = 2 * small
        for j in range(null.shape[0] // per - 1):  # keep the last block out of the inputs
            sub = null[j * per:(j + 1) * per]
            f, m = gpd.features(sub, V, rho, s["E"], s["n"], s["k"])
            X.append(f)
            Y.append(gpd.targets(null, m))
            meta.append((len(meta), m))
    return np.asarray(X), np.asarray(Y)


def p_errors(model, norm, settings, nulls, small, alpha_band=(0.002, 0.05)):
    """Max |delta p| over tail values (full-null p in alpha_band) for the
    network tail, the classical GPD fit and the plain small-sample empirical p."""
    errs = {"mlp": [], "gpd": [], "empirical": []}
    for s, (null, rho, V) in zip(settings, nulls):
        sub = null[: 2 * small]
        full_sorted = np.sort(null)
        qs = np.quantile(null, 1 - np.linspace(alpha_band[0], alpha_band[1], 25))
        ref = gpd.one_minus_p(qs, null)
        f, m = gpd.features(sub, V, rho, s["E"], s["n"], s["k"])
        pred = model.predict_bf16(((f - norm[0]) / norm[1])[None])[0] * norm[3] + norm[2]
        u, xi, sg = gpd.decode(pred, m)
        errs["mlp"].append(np.abs(gpd.one_minus_p(qs, sub, u, xi, sg) - ref).max())
        u0, xi0, s0 = gpd.tail_params(sub)
        errs["gpd"].append(np.abs(gpd.one_minus_p(qs, sub, u0, xi0, s0) - ref).max())
        errs["empirical"].append(np.abs(gpd.one_minus_p(qs, sub) - ref).max())
        del full_sorted
    return {k: float(np.mean(v)) for k, v in errs.items()}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--settings", type=int, default=500)
    ap.add_argument("--full", type=int, default=1500)
    ap.add_argument("--small", type=int, default=300)
    ap.add_argument("--epochs", type=int, default=600)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--out", default="weights.npz")
    ap.add_argument("--report", default=None)
    ap.add_argument("--level-p", default="0.5,0.35,0.15",
                    help="probabilities of icosphere levels 5, 6, 7 among the settings")
    a = ap.parse_args(argv)
    t0 = time.time()
    level_p = tuple(float(x) for x in a.level_p.split(","))
    settings = data.sample_settings(a.settings, a.seed, level_p=level_p)
    nulls = []
    for i, s in enumerate(settings):
        nulls.append(data.null_for_setting(s, a.full))
        if i % 50 == 0:
            print(f"setting {i}/{len(settings)}  {time.time() - t0:.0f}s", flush=True)
    gen_s = time.time() - t0
    n_hold = max(1, len(settings) // 10)
    tr_s, ho_s = settings[n_hold:], settings[:n_hold]
    tr_n, ho_n = nulls[n_hold:], nulls[:n_hold]
    X, Y = build_rows(tr_s, tr_n, a.small)
    Xh, Yh = build_rows(ho_s, ho_n, a.small)
    fm, fs = X.mean(axis=0), X.std(axis=0) + 1e-6
    tm, ts = Y.mean(axis=0), Y.std(axis=0) + 1e-6
    model = MLP((X.shape[1], 128, 128, 128, 3), seed=a.seed)
    t1 = time.time()
    curve = model.fit((X - fm) / fs, (Y - tm) / ts, epochs=a.epochs, batch=256, lr=2e-3, verbose=True)
    train_s = time.time() - t1
    norm = (fm, fs, tm, ts)
    pred_h = model.predict((Xh - fm) / fs) * ts + tm
    held_mse = float(np.mean(((pred_h - Yh) / ts) ** 2))
    # the classical estimate of the same targets (GPD fit of the small sample) for comparison
    base_h = Xh[:, 13:16]
    base_mse = float(np.mean(((base_h - Yh) / ts) ** 2))
    perr = p_errors(model, norm, ho_s, ho_n, a.small)
    model.save(a.out, feat_mean=fm, feat_std=fs, targ_mean=tm, targ_std=ts, quant=np.float64(gpd.QUANT),
               small=np.int64(a.small))
    rep = {"settings": len(settings), "level_p": list(level_p), "full_perms": a.full, "small_perms": a.small, "train_rows": int(X.shape[0]),
           "heldout_rows": int(Xh.shape[0]), "gen_s": gen_s, "train_s": train_s, "final_train_loss": float(curve[-1]),
           "heldout_mse_normalised": held_mse, "classical_gpd_mse_normalised": base_mse,
           "heldout_max_abs_dp": perr}
    print(json.dumps(rep))
    if a.report:
        with open(a.report, "w") as fh:
            json.dump(rep, fh, indent=1)
    return rep


if __name__ == "__main__":
    main()
