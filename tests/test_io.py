"""The MGH and NIfTI-1 writers behind write_vertStat_img / write_voxelStat_img
(tfce_mediation/pyfunc.py:80-103) when nibabel is absent: header fields by the
formats' layouts and data round trips."""
import gzip
import struct

import numpy as np
import pytest

from tfce_mediation_gb300 import io

pytestmark = pytest.mark.skipif(io._nib() is not None, reason="nibabel present: its writers are used")


@pytest.mark.parametrize("name", ["stat.mgh", "stat.mgz"])
def test_mgh_header_and_round_trip(tmp_path, name):
    rng = np.random.default_rng(1)
    data = rng.standard_normal((642, 1, 1)).astype(np.float32)
    aff = np.array([[-1, 0, 0, 10], [0, 0, 1, -20], [0, -1, 0, 30], [0, 0, 0, 1]], np.float64)
    p = str(tmp_path / name)
    io.save_mgh(data, aff, p)
    raw = (gzip.open if name.endswith(".mgz") else open)(p, "rb").read()
    version, w, h, d, f, typ, dof = struct.unpack(">7i", raw[:28])
    assert (version, w, h, d, f, typ) == (1, 642, 1, 1, 1, 3)
    assert struct.unpack(">h", raw[28:30])[0] == 1  # RAS information present
    spacing = struct.unpack(">3f", raw[30:42])
    np.testing.assert_allclose(spacing, [1, 1, 1])
    mdc = np.array(struct.unpack(">9f", raw[42:78])).reshape(3, 3).T  # stored column by column
    np.testing.assert_allclose(mdc, aff[:3, :3])
    c_ras = struct.unpack(">3f", raw[78:90])
    np.testing.assert_allclose(c_ras, aff[:3, :3] @ (np.array([642, 1, 1]) / 2.0) + aff[:3, 3], rtol=1e-6)
    assert len(raw) == 284 + 4 * 642
    np.testing.assert_array_equal(io.load_mgh(p)[:, :, :], data)


@pytest.mark.parametrize("name,dtype", [("stat.nii", np.float32), ("stat.nii.gz", np.float32),
                                        ("stat64.nii", np.float64)])
def test_nifti_header_and_round_trip(tmp_path, name, dtype):
    rng = np.random.default_rng(2)
    data = rng.standard_normal((5, 4, 3)).astype(dtype)
    aff = np.diag([2.0, 2.0, 2.5, 1.0])
    aff[:3, 3] = [-90, -126, -72]
    p = str(tmp_path / name)
    io.save_nifti(data, aff, p)
    raw = (gzip.open if name.endswith(".gz") else open)(p, "rb").read()
    assert struct.unpack("<i", raw[:4])[0] == 348
    dims = struct.unpack("<8h", raw[40:56])
    assert dims[:4] == (3, 5, 4, 3)
    datatype, bitpix = struct.unpack("<2h", raw[70:74])
    assert (datatype, bitpix) == ((16, 32) if dtype == np.float32 else (64, 64))
    pix = struct.unpack("<8f", raw[76:108])
    np.testing.assert_allclose(pix[1:4], [2.0, 2.0, 2.5])
    assert struct.unpack("<f", raw[108:112])[0] == 352.0
    qform, sform = struct.unpack("<2h", raw[252:256])
    assert (qform, sform) == (0, 1)
    srow = np.array(struct.unpack("<12f", raw[280:328])).reshape(3, 4)
    np.testing.assert_allclose(srow, aff[:3, :])
    assert raw[344:348] == b"n+1\x00"
    body = np.frombuffer(raw[352:], "<f4" if dtype == np.float32 else "<f8").reshape(data.shape, order="F")
    np.testing.assert_array_equal(body, data)
