"""CPU oracle for Vship's SSIMULACRA2 and Butteraugli math (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may import this package;
it is the checker, never the product. See oracle.cpp for the per-function reference citations.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

IN_UINT8, IN_UINT16, IN_HALF, IN_FLOAT = 0, 1, 2, 3
_DT = {np.dtype(np.uint8): IN_UINT8, np.dtype(np.uint16): IN_UINT16, np.dtype(np.float16): IN_HALF,
       np.dtype(np.float32): IN_FLOAT}

_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        P = ctypes.POINTER
        L.oracle_ssimu2.argtypes = [P(ctypes.c_void_p), P(ctypes.c_void_p), ctypes.c_int64, ctypes.c_int64,
                                    ctypes.c_int64, ctypes.c_int64, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                    P(ctypes.c_double), P(ctypes.c_double)]
        L.oracle_butteraugli.argtypes = [P(ctypes.c_void_p), P(ctypes.c_void_p), ctypes.c_int64, ctypes.c_int64,
                                         ctypes.c_int64, ctypes.c_int64, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                         ctypes.c_int, ctypes.c_int, P(ctypes.c_double), ctypes.c_void_p]
        L.oracle_malta_pattern.argtypes = [ctypes.c_int, ctypes.c_int, P(ctypes.c_int)]
        L.oracle_ssimu2_weights.restype = P(ctypes.c_double)
        _lib = L
    return _lib


def _planes(frame):
    """frame: sequence of 3 planes (H x W arrays, same dtype) or a (3, H, W) array.

    Returns (ptr array, stride in bytes, width, height, intype, keepalive)."""
    planes = [np.asarray(p) for p in frame]
    if len(planes) != 3:
        raise ValueError("expected 3 planes")
    dt = planes[0].dtype
    h, w = planes[0].shape
    strides = set()
    for p in planes:
        if p.dtype != dt or p.shape != (h, w) or p.strides[1] != dt.itemsize:
            raise ValueError("planes must share dtype/shape and have contiguous rows")
        strides.add(p.strides[0])
    if len(strides) != 1:
        raise ValueError("planes must share a row stride")
    arr = (ctypes.c_void_p * 3)(*[p.ctypes.data for p in planes])
    return arr, strides.pop(), w, h, _DT[dt], planes


def ssimu2(ref, dist, precision: int = 64, nthreads: int | None = None, measure: bool = False):
    a1, s1, w, h, it, k1 = _planes(ref)
    a2, s2, w2, h2, it2, k2 = _planes(dist)
    if (w, h, it) != (w2, h2, it2):
        raise ValueError("reference and distorted frames differ")
    out = ctypes.c_double()
    m = (ctypes.c_double * 108)()
    nt = nthreads if nthreads is not None else (os.cpu_count() or 1)
    rc = lib().oracle_ssimu2(a1, a2, s1, s2, w, h, it, precision, nt, ctypes.byref(out), m)
    if rc:
        raise RuntimeError("oracle_ssimu2 failed")
    return (out.value, np.array(m[:])) if measure else out.value


def butteraugli(ref, dist, qnorm: int = 2, intensity: float = 203.0, precision: int = 64,
                nthreads: int | None = None, distmap: bool = False):
    a1, s1, w, h, it, k1 = _planes(ref)
    a2, s2, w2, h2, it2, k2 = _planes(dist)
    if (w, h, it) != (w2, h2, it2):
        raise ValueError("reference and distorted frames differ")
    norms = (ctypes.c_double * 3)()
    dm = np.zeros((h, w), np.float32) if distmap else None
    nt = nthreads if nthreads is not None else (os.cpu_count() or 1)
    rc = lib().oracle_butteraugli(a1, a2, s1, s2, w, h, it, qnorm, intensity, precision, nt, norms,
                                  dm.ctypes.data if dm is not None else None)
    if rc:
        raise RuntimeError("oracle_butteraugli failed")
    res = tuple(norms[:])
    return (res, dm) if distmap else res


def malta_pattern(hf_unit: bool, index: int):
    buf = (ctypes.c_int * 18)()
    n = lib().oracle_malta_pattern(1 if hf_unit else 0, index, buf)
    return [(buf[2 * t], buf[2 * t + 1]) for t in range(n)]


def ssimu2_weights():
    p = lib().oracle_ssimu2_weights()
    return [p[i] for i in range(108)]
