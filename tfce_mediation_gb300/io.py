"""Image writers for the observed-statistic outputs (MGH surfaces, NIfTI
volumes) used by write_vertStat_img / write_voxelStat_img
(tfce_mediation/pyfunc.py:80-103).

nibabel is used when it is installed; otherwise minimal writers of the same
formats are used: FreeSurfer MGH (big-endian 284-byte header, float32 data in
column-major order) and single-file NIfTI-1 (348-byte header, sform from the
affine), gzip-compressed for names ending in .gz.
"""
from __future__ import annotations

import gzip
import struct

import numpy as np


def _nib():
    try:
        import nibabel  # noqa: F401
        return nibabel
    except Exception:
        return None


def save_mgh(data, affine, path):
    nib = _nib()
    data = np.asarray(data)
    affine = np.asarray(affine, np.float64)
    if nib is not None:
        nib.save(nib.freesurfer.mghformat.MGHImage(data.astype(np.float32), affine), path)
        return
    arr = data.astype(">f4")
    shape = list(arr.shape) + [1] * (4 - arr.ndim)
    M = affine[:3, :3]
    spacing = np.sqrt((M ** 2).sum(axis=0))
    spacing[spacing == 0] = 1.0
    mdc = M / spacing
    c_ras = M @ (np.asarray(shape[:3], np.float64) / 2.0) + affine[:3, 3]
    hdr = struct.pack(">7i", 1, shape[0], shape[1], shape[2], shape[3], 3, 0)
    hdr += struct.pack(">h", 1)
    hdr += struct.pack(">3f", *spacing)
    hdr += struct.pack(">9f", *mdc.T.ravel())
    hdr += struct.pack(">3f", *c_ras)
    hdr += b"\x00" * (284 - len(hdr))
    body = arr.reshape(shape).ravel(order="F").astype(">f4").tobytes()
    opener = gzip.open if path.endswith(".mgz") else open
    with opener(path, "wb") as fh:
        fh.write(hdr + body)


def save_nifti(data, affine, path):
    nib = _nib()
    data = np.asarray(data)
    affine = np.asarray(affine, np.float64)
    if nib is not None:
        nib.save(nib.Nifti1Image(data, affine), path)
        return
    code, bitpix, dt = {np.dtype(np.float64): (64, 64, "<f8")}.get(data.dtype, (16, 32, "<f4"))
    dims = [data.ndim] + list(data.shape) + [1] * (7 - data.ndim)
    pix = [1.0] + list(np.sqrt((affine[:3, :3] ** 2).sum(axis=0))) + [1.0] * 4
    h = struct.pack("<i", 348) + b"\x00" * 10 + b"\x00" * 18 + struct.pack("<ihcc", 0, 0, b"r", b"\x00")
    h += struct.pack("<8h", *dims)
    h += struct.pack("<3fhhhh", 0.0, 0.0, 0.0, 0, code, bitpix, 0)
    h += struct.pack("<8f", *pix)
    h += struct.pack("<3fhcc", 352.0, 1.0, 0.0, 0, b"\x00", bytes([10]))
    h += struct.pack("<4f2i", 0.0, 0.0, 0.0, 0.0, 0, 0)
    h += b"\x00" * 80 + b"\x00" * 24
    h += struct.pack("<2h", 0, 1)
    h += struct.pack("<6f", 0, 0, 0, 0, 0, 0)
    h += struct.pack("<12f", *affine[:3, :].ravel())
    h += b"\x00" * 16 + b"n+1\x00"
    assert len(h) == 348
    body = np.asarray(data, dt).ravel(order="F").tobytes()
    opener = gzip.open if path.endswith(".gz") else open
    with opener(path, "wb") as fh:
        fh.write(h + b"\x00" * 4 + body)


def load_mgh(path):
    """Read back an MGH written by save_mgh (data, affine-free)."""
    opener = gzip.open if path.endswith(".mgz") else open
    with opener(path, "rb") as fh:
        raw = fh.read()
    v, w, h, d, f, typ, dof = struct.unpack(">7i", raw[:28])
    arr = np.frombuffer(raw[284:284 + 4 * w * h * d * f], ">f4").reshape((w, h, d, f), order="F")
    return arr[..., 0] if f == 1 else arr
