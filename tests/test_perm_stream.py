"""Native permutation index streams (perm_stream, csrc/perm_stream.cu)
against numpy's own RandomState(seed + p).permutation(n), the mmr-lr
convention of tfce_mediation/tm_func.py:147-151: bit-identical rows.  Host
code of the library only, so this runs without a GPU."""
import numpy as np
import pytest

from tfce_mediation_gb300 import engine as E


def _ref(n, seed, start, stop):
    return np.stack([np.random.RandomState(seed + p).permutation(n) for p in range(start, stop)])


@pytest.mark.parametrize("n", [1, 2, 3, 16, 17, 100, 350, 1000, 65537])
def test_rows_equal_numpy(n):
    for seed, start, stop in ((0, 0, 6), (12345, 7, 31), (2 ** 32 - 9, 0, 9)):
        if n > 5000:
            stop = start + 2
        np.testing.assert_array_equal(E.permutations(n, seed, start, stop), _ref(n, seed, start, stop))


def test_many_rows_over_threads():
    """Enough rows that the library splits them over threads."""
    got = E.permutations(350, 5, 1000, 1600)
    np.testing.assert_array_equal(got[::37], _ref(350, 5, 1000, 1600)[::37])
    assert got.dtype == np.int64 and got.shape == (600, 350)


def test_seed_range_is_refused():
    """RandomState accepts seeds in [0, 2^32 - 1] only; so does the stream."""
    with pytest.raises(RuntimeError):
        E.permutations(10, 2 ** 32 - 3, 0, 5)
    with pytest.raises(RuntimeError):
        E.permutations(10, -1, 0, 1)
    assert E.permutations(10, 0, 4, 4).shape == (0, 10)
