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


_MGH_TYPES = {0: ">u1", 1: ">i4", 3: ">f4", 4: ">i2"}


def load_mgh(path, with_affine=False):
    """Read an MGH/MGZ volume: data (width, height, depth[, frames]) in its
    stored type (float32 for the files this package writes) and, with
    with_affine, the vox2ras matrix from the header (direction cosines,
    spacing and centre RAS)."""
    nib = _nib()
    if nib is not None:
        img = nib.load(path)
        data = np.asarray(img.dataobj)
        return (data, np.asarray(img.affine, np.float64)) if with_affine else data
    opener = gzip.open if path.endswith(".mgz") else open
    with opener(path, "rb") as fh:
        raw = fh.read()
    v, w, h, d, f, typ, dof = struct.unpack(">7i", raw[:28])
    dt = np.dtype(_MGH_TYPES.get(typ, ">f4"))
    n = w * h * d * f
    arr = np.frombuffer(raw[284:284 + dt.itemsize * n], dt).reshape((w, h, d, f), order="F").astype(dt.newbyteorder("="))
    arr = arr[..., 0] if f == 1 else arr
    if not with_affine:
        return arr
    good = struct.unpack(">h", raw[28:30])[0]
    aff = np.eye(4)
    if good:
        spacing = np.asarray(struct.unpack(">3f", raw[30:42]), np.float64)
        mdc = np.asarray(struct.unpack(">9f", raw[42:78]), np.float64).reshape(3, 3).T
        c_ras = np.asarray(struct.unpack(">3f", raw[78:90]), np.float64)
        M = mdc * spacing
        aff[:3, :3] = M
        aff[:3, 3] = c_ras - M @ (np.asarray([w, h, d], np.float64) / 2.0)
    return arr, aff


def load_nifti(path):
    """Read a single-file NIfTI-1 image (.nii / .nii.gz): (data, affine).
    The affine is the sform when set, else the qform-free pixel-size diagonal."""
    nib = _nib()
    if nib is not None:
        img = nib.load(path)
        return np.asarray(img.dataobj), np.asarray(img.affine, np.float64)
    opener = gzip.open if path.endswith(".gz") else open
    with opener(path, "rb") as fh:
        raw = fh.read()
    end = "<" if struct.unpack("<i", raw[:4])[0] == 348 else ">"
    dims = struct.unpack(end + "8h", raw[40:56])
    datatype, bitpix = struct.unpack(end + "hh", raw[70:74])
    pix = struct.unpack(end + "8f", raw[76:108])
    vox_offset = int(struct.unpack(end + "f", raw[108:112])[0])
    scl = struct.unpack(end + "2f", raw[112:120])
    sform_code = struct.unpack(end + "h", raw[254:256])[0]
    types = {2: "u1", 4: "i2", 8: "i4", 16: "f4", 64: "f8", 256: "i1", 512: "u2", 768: "u4"}
    if datatype not in types:
        raise ValueError(f"NIfTI datatype {datatype} not supported")
    dt = np.dtype(end + types[datatype])
    shape = tuple(int(x) for x in dims[1:1 + dims[0]])
    n = int(np.prod(shape))
    data = np.frombuffer(raw[vox_offset:vox_offset + dt.itemsize * n], dt).reshape(shape, order="F")
    data = data.astype(dt.newbyteorder("="))
    if scl[0] not in (0.0, 1.0) or scl[1] != 0.0:
        data = data * scl[0] + scl[1]
    aff = np.eye(4)
    if sform_code > 0:
        aff[:3, :] = np.asarray(struct.unpack(end + "12f", raw[280:328]), np.float64).reshape(3, 4)
    else:
        aff[0, 0], aff[1, 1], aff[2, 2] = pix[1], pix[2], pix[3]
    return data, aff
