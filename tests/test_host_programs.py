"""Host logic of the programmed GLM outputs and the tm-models drivers (no GPU):
output rows and per-design weights, the cosinor design and output program,
and the exchange-block rules of the two randomise families."""
import argparse

import numpy as np
import pytest

from oracle import oracle
from tfce_mediation_gb300 import pyfunc, randomise
from tfce_mediation_gb300.glm import (OUT_ACRO, OUT_AMP, OUT_F, OUT_NEG_T, OUT_T, DesignBatch, output_columns,
                                      output_program)


def test_output_program_rows_and_offsets():
    rows, stride = output_program([("f", 1, 3), ("amp", 1), ("acro", 3), ("t", 4), ("-t", 4), ("f", 2, 1)])
    np.testing.assert_array_equal(rows, [[OUT_F, 1, 3, 0], [OUT_AMP, 1, 2, 9], [OUT_ACRO, 3, 2, 12],
                                         [OUT_T, 4, 1, 0], [OUT_NEG_T, 4, 1, 0], [OUT_F, 2, 1, 15]])
    assert stride == 16
    assert output_columns([("amp", 1), ("t", 5)]) == {1, 2, 5}
    with pytest.raises(ValueError):
        output_program([("z", 1)])
    with pytest.raises(ValueError):
        output_program([("f", 1, 0)])


def test_program_weights_match_inverse_blocks():
    rng = np.random.default_rng(3)
    n, G = 40, 5
    X = np.column_stack([np.ones(n), rng.standard_normal((n, 4))])
    perms = np.stack([rng.permutation(n) for _ in range(G)])
    db = DesignBatch(X[perms])
    outs = [("f", 1, 4), ("amp", 1), ("acro", 3), ("t", 2), ("amp", 4)]
    W = db.program_weights(outs)
    rows, stride = output_program(outs)
    assert W.shape == (G, stride) and W.dtype == np.float32
    for g in range(G):
        Xg = X[perms[g]]
        inv = np.linalg.inv(Xg.T @ Xg)
        np.testing.assert_allclose(W[g, :16], np.linalg.inv(inv[1:5, 1:5]).ravel(), rtol=1e-6)
        np.testing.assert_allclose(W[g, 16:19], [inv[1, 1], inv[1, 2], inv[2, 2]], rtol=1e-6)
        np.testing.assert_allclose(W[g, 19:22], [inv[3, 3], inv[3, 4], inv[4, 4]], rtol=1e-6)
        assert np.all(W[g, 22:25] == 0.0)  # ("amp", 4) lies outside the 5 columns: NaN on the device
    np.testing.assert_array_equal(db.group_blocks([(1, 4)]), W[:, :16])
    out = np.full((G, stride), 7.0, np.float32)
    db.program_weights(outs, out=out)
    np.testing.assert_array_equal(out[:, :22], W[:, :22])


def test_cosinor_design_and_outputs():
    rng = np.random.default_rng(4)
    n = 30
    tv = rng.uniform(0, 48, n)
    ex = [rng.standard_normal((n, 2)), rng.standard_normal(n)]
    cov = rng.standard_normal((n, 1))
    X = pyfunc.cosinor_design(tv, [24.0, 8.0], ex, cov)
    np.testing.assert_array_equal(X, oracle.cosinor_design(tv, [24.0, 8.0], ex, cov))
    assert X.shape == (n, 1 + 4 + 3 + 1)
    outs = randomise.cosinor_outputs(2, 3, 1)
    assert outs[0] == ("f", 1, 8)
    assert outs[1:5] == [("amp", 1), ("acro", 1), ("amp", 3), ("acro", 3)]
    assert outs[5:] == [("t", 5), ("-t", 5), ("t", 6), ("-t", 6), ("t", 7), ("-t", 7)]
    assert 0 not in output_columns(outs)  # the centred residual form applies


@pytest.mark.parametrize("sizes", [(4, 4, 4), (3, 5, 4)])
def test_exchange_block_rules(tmp_path, sizes):
    """Vertex/voxel loops shuffle the blocks' order always; the tm-models loops
    (rand_blocks + check_blocks) only when the blocks are equal in size; both
    permute within every block."""
    labels = np.concatenate([np.full(s, "b%d" % i) for i, s in enumerate(sizes)])
    f = tmp_path / "blocks.csv"
    np.savetxt(f, labels, fmt="%s")
    n = labels.shape[0]
    X = np.arange(n, dtype=np.float64)[:, None]
    opts = argparse.Namespace(exchangeblock=[str(f)], specifyvars=None)
    equal = len(set(sizes)) == 1
    for tm in (False, True):
        D = randomise._designs_for(X, n, 0, 6, opts, 9, equal_blocks_only=tm)[:, :, 0].astype(int)
        for p in range(6):
            rng = np.random.RandomState(9 + p)
            uniq = np.unique(labels)
            order = rng.permutation(list(uniq)) if (not tm or equal) else uniq
            idx = np.arange(n)
            want = np.concatenate([rng.permutation(idx[labels == b]) for b in order])
            np.testing.assert_array_equal(D[p], want)
            if tm and not equal:
                # block order kept: every position stays inside its own block
                np.testing.assert_array_equal(labels[D[p]], labels)


def test_saved_none(tmp_path):
    np.save(tmp_path / "a.npy", np.array(None, dtype=object), allow_pickle=True)
    np.save(tmp_path / "b.npy", np.zeros((3, 1)))
    assert randomise._saved_none(np.load(tmp_path / "a.npy", allow_pickle=True))
    assert not randomise._saved_none(np.load(tmp_path / "b.npy"))
    assert randomise._saved_none(None)
