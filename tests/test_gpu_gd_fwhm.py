"""Geodesic FWHM smoothing on the GPU (calc_gd_fwhm) against the reference's
own outputs (golden vectors) and the oracle, single images and batches.

Bar: at most 1 ulp from the reference (the device's square and exponential
are correctly rounded; the reference's libm powf / expf differ from that on
~0.06 % of arguments), and at least 95 % of values bit-identical."""
import numpy as np
import pytest

from oracle import oracle
from tfce_mediation_gb300 import cynumstats
from tfce_mediation_gb300.gd_fwhm import GeodesicSmoother

pytestmark = pytest.mark.gpu


def _ulps(a, b):
    a = np.asarray(a, np.float32).view(np.int32).astype(np.int64)
    b = np.asarray(b, np.float32).view(np.int32).astype(np.int64)
    return np.abs(a - b)


@pytest.mark.parametrize("k", [0, 1])
def test_calc_gd_fwhm_vs_reference(golden, k):
    got = cynumstats.calc_gd_fwhm(golden["gd_pairs"], golden["gd_dist"], golden[f"gd_data{k}"],
                                  float(golden[f"gd_sigma{k}"]))
    u = _ulps(got, golden[f"gd_out{k}"])
    print("gd_fwhm", k, "max ulp", u.max(), "exact", np.mean(u == 0))
    assert u.max() <= 1
    assert np.mean(u == 0) >= 0.95


def test_smoother_batch_equals_single_images(golden):
    rng = np.random.default_rng(9)
    pairs, dist = golden["gd_pairs"], golden["gd_dist"]
    V = golden["gd_data0"].shape[0]
    sm = GeodesicSmoother(pairs, dist, 0.01, V)
    imgs = (rng.standard_normal((5, V)) * 3).astype(np.float32)
    batch = sm.smooth(imgs)
    for b in range(5):
        np.testing.assert_array_equal(batch[b], sm.smooth(imgs[b]))
        ref = oracle.calc_gd_fwhm(pairs, dist, imgs[b], 0.01)
        assert _ulps(batch[b], ref).max() <= 1
