"""Page-locked (pinned) host arrays for the engine's transfers.

The C ABI copies into and out of caller buffers; a page-locked buffer lets
the copy engines move the data directly (on the Grace host about 190 GB/s
device to host, against 36 GB/s through the library's staging threads into
pageable memory).  ``empty`` returns a numpy array backed by cudaHostAlloc
memory, freed when the array is garbage-collected.
"""
from __future__ import annotations

import ctypes as C
import glob
import weakref

import numpy as np

_rt = None


def _cudart():
    global _rt
    if _rt is None:
        for c in sorted(glob.glob("/usr/local/cuda/lib64/libcudart.so*")) + ["libcudart.so"]:
            try:
                _rt = C.CDLL(c)
                break
            except OSError:
                continue
        if _rt is None:
            raise RuntimeError("libcudart not found")
        _rt.cudaHostAlloc.argtypes = [C.POINTER(C.c_void_p), C.c_size_t, C.c_uint]
        _rt.cudaFreeHost.argtypes = [C.c_void_p]
    return _rt


def empty(shape, dtype) -> np.ndarray:
    """An uninitialised page-locked numpy array (freed with the last array or
    view that uses it)."""
    dt = np.dtype(dtype)
    n = int(np.prod(shape)) if np.ndim(shape) else int(shape)
    nbytes = max(n * dt.itemsize, 1)
    p = C.c_void_p()
    rc = _cudart().cudaHostAlloc(C.byref(p), nbytes, 0)
    if rc != 0:
        raise MemoryError(f"cudaHostAlloc({nbytes}) failed: {rc}")
    buf = (C.c_char * nbytes).from_address(p.value)
    weakref.finalize(buf, _cudart().cudaFreeHost, C.c_void_p(p.value))
    return np.frombuffer(buf, dtype=dt, count=n).reshape(shape)


def copy(x: np.ndarray) -> np.ndarray:
    """A page-locked copy of x."""
    a = empty(x.shape, x.dtype)
    a[...] = x
    return a
