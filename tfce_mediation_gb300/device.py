"""Device plumbing: torch provides device memory and streams; every kernel
comes from the native library (``_lib``).  There is no CPU path: without a
CUDA device these helpers raise."""
from __future__ import annotations

import numpy as np

from . import _lib


class NoDeviceError(RuntimeError):
    pass


def torch():
    import torch as _t
    return _t


def require_cuda():
    t = torch()
    if not t.cuda.is_available():
        raise NoDeviceError("tfce_mediation_gb300 runs on a CUDA GPU (sm_103a); none is visible")
    _lib.load()
    return t


def dev(a, dtype=None):
    """numpy / torch -> contiguous CUDA tensor."""
    t = require_cuda()
    if isinstance(a, t.Tensor):
        out = a.to(device="cuda", dtype=dtype or a.dtype)
    else:
        arr = np.asarray(a)
        if dtype is None:
            dtype = {np.dtype(np.float32): t.float32, np.dtype(np.float64): t.float64,
                     np.dtype(np.int32): t.int32, np.dtype(np.int64): t.int64}.get(arr.dtype, t.float32)
        out = t.from_numpy(np.ascontiguousarray(arr)).to(device="cuda", dtype=dtype)
    return out.contiguous()


def ptr(x):
    """Device pointer of a tensor (or None)."""
    return None if x is None else x.data_ptr()


def stream_handle(stream=None):
    t = torch()
    s = stream if stream is not None else t.cuda.current_stream()
    return s.cuda_stream
