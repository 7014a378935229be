"""ctypes binding of the reference's own CUDA library (oracle/_ref/libvship_ref.so, built by
oracle/ref_build.py from pkp24/Vship src/VshipLib.cpp).

Test and benchmark infrastructure only: the differential parity tests, the reference-fixture
script and bench.py's reference_cuda leg use it; the product never does. The calls are the
reference's C ABI (src/VshipAPI.h:32-148), plus VshipRef_ComputeButteraugli (oracle/ref_shim.cu),
which runs the same computing implementation but returns the float norms the ABI's int struct
would truncate.

The library is loaded with RTLD_LOCAL, so its Vship_* symbols never interpose on the product
library's when both are in one process.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import ref_build

_lib = None
_PP = ctypes.POINTER(ctypes.c_void_p)


class _Handler(ctypes.Structure):
    _fields_ = [("id", ctypes.c_int)]


class _ButterScore(ctypes.Structure):
    _fields_ = [("norm2", ctypes.c_int), ("norm3", ctypes.c_int), ("norminf", ctypes.c_int)]


_E = ctypes.c_int
SIGNATURES = {
    "Vship_GetDeviceCount": (_E, [ctypes.POINTER(ctypes.c_int)]),
    "Vship_SetDevice": (_E, [ctypes.c_int]),
    "Vship_GetErrorMessage": (ctypes.c_int, [ctypes.c_int, ctypes.c_char_p, ctypes.c_int]),
    "Vship_SSIMU2Init": (_E, [ctypes.POINTER(_Handler), ctypes.c_int, ctypes.c_int]),
    "Vship_SSIMU2Free": (_E, [_Handler]),
    "Vship_ComputeSSIMU2Float": (_E, [_Handler, ctypes.POINTER(ctypes.c_double), _PP, _PP, ctypes.c_int64]),
    "Vship_ComputeSSIMU2Uint16": (_E, [_Handler, ctypes.POINTER(ctypes.c_double), _PP, _PP, ctypes.c_int64]),
    "Vship_ButteraugliInitv2": (_E, [ctypes.POINTER(_Handler), ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_float]),
    "Vship_ButteraugliFree": (_E, [_Handler]),
    "Vship_ComputeButteraugliUint16": (_E, [_Handler, ctypes.POINTER(_ButterScore), ctypes.c_void_p,
                                            ctypes.c_int64, _PP, _PP, ctypes.c_int64]),
    "Vship_ComputeButteraugliFloat": (_E, [_Handler, ctypes.POINTER(_ButterScore), ctypes.c_void_p,
                                           ctypes.c_int64, _PP, _PP, ctypes.c_int64]),
    "VshipRef_ComputeButteraugli": (_E, [_Handler, ctypes.POINTER(ctypes.c_float), ctypes.c_int, ctypes.c_void_p,
                                         ctypes.c_int64, _PP, _PP, ctypes.c_int64, ctypes.c_int64]),
}


class ReferenceError_(RuntimeError):
    pass


def available() -> bool:
    return ref_build.available()


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not ref_build.available():
            raise ImportError(f"{ref_build.LIB} is missing: stage and build it with `python -m oracle.ref_build`")
        L = ctypes.CDLL(ref_build.LIB, mode=os.RTLD_LOCAL | os.RTLD_NOW)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _check(rc: int, where: str):
    if rc != 0:
        L = lib()
        n = L.Vship_GetErrorMessage(int(rc), None, 0)
        buf = ctypes.create_string_buffer(max(n, 1))
        L.Vship_GetErrorMessage(int(rc), buf, max(n, 1))
        raise ReferenceError_(f"{where}: reference error {rc}: {buf.value.decode(errors='replace')}")


def _planes(frame):
    planes = [np.ascontiguousarray(p) for p in frame]
    if len(planes) != 3 or len({p.shape for p in planes}) != 1 or len({p.dtype for p in planes}) != 1:
        raise ValueError("a frame is three planes of one shape and dtype")
    if planes[0].dtype not in (np.float32, np.uint16):
        raise TypeError("planes must be float32 or uint16")
    return (ctypes.c_void_p * 3)(*[p.ctypes.data for p in planes]), planes[0].strides[0], planes


class SSIMU2:
    """The reference's SSIMULACRA2 handler (Vship_SSIMU2Init / Vship_ComputeSSIMU2* / Free)."""

    def __init__(self, width: int, height: int):
        self.width, self.height = int(width), int(height)
        h = _Handler()
        _check(lib().Vship_SSIMU2Init(ctypes.byref(h), self.width, self.height), "Vship_SSIMU2Init")
        self._h = h

    def compute(self, reference, distorted) -> float:
        a, s, ka = _planes(reference)
        b, s2, kb = _planes(distorted)
        if s != s2 or ka[0].dtype != kb[0].dtype or ka[0].shape != (self.height, self.width):
            raise ValueError("frames must match the handler's size and each other's layout")
        out = ctypes.c_double()
        f = lib().Vship_ComputeSSIMU2Uint16 if ka[0].dtype == np.uint16 else lib().Vship_ComputeSSIMU2Float
        _check(f(self._h, ctypes.byref(out), ctypes.cast(a, _PP), ctypes.cast(b, _PP), s), "Vship_ComputeSSIMU2")
        return out.value

    def free(self):
        if self._h is not None:
            _check(lib().Vship_SSIMU2Free(self._h), "Vship_SSIMU2Free")
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.free()


def butteraugli_size_safe(width: int, height: int) -> bool:
    """Whether the reference's Butteraugli stays inside its own allocations at this frame size.

    Its window-8 tiled blur (src/butter/gaussianblur.hpp:95-185; 32x32 outputs per 16x16-thread
    CTA, two 16-column and two 16-row halves per thread) renormalises at the border with
    gaussiankernel_integral[min(width, c + 9) - (c - 8)] for every output column (and row) c of
    the tile, including columns past the image edge. For the last tile of a dimension d that
    index reaches d - (32 * ((d - 1) // 32) + 23), below -17 when d mod 32 is 1 to 5; the sigma
    1.2 kernel's integral starts 17 floats into the handler's table allocation
    (src/butter/gaussianblur.hpp:18-56, indices[0] = 0), so those sizes read before the start of
    that allocation. The blur runs at full and half resolution (src/butter/main.hpp:116-139)."""
    for d in (width, height, (width - 1) // 2 + 1, (height - 1) // 2 + 1):
        if 1 <= d % 32 <= 5:
            return False
    return True


class Butteraugli:
    """The reference's Butteraugli handler (Vship_ButteraugliInitv2 / VshipRef_ComputeButteraugli /
    Free): float norms (Qnorm, 3-norm, inf-norm) and, on request, the float32 distortion map.
    Sizes at which the reference reads outside its allocations (butteraugli_size_safe) are
    refused before anything reaches the GPU."""

    def __init__(self, width: int, height: int, qnorm: int = 2, intensity_multiplier: float = 203.0):
        if not butteraugli_size_safe(width, height):
            raise ValueError(f"{width}x{height}: the reference's Butteraugli reads outside its own allocations "
                             "at this size (butteraugli_size_safe)")
        self.width, self.height = int(width), int(height)
        h = _Handler()
        _check(lib().Vship_ButteraugliInitv2(ctypes.byref(h), self.width, self.height, int(qnorm),
                                             ctypes.c_float(intensity_multiplier)), "Vship_ButteraugliInitv2")
        self._h = h

    def compute(self, reference, distorted, distmap: bool = False):
        a, s, ka = _planes(reference)
        b, s2, kb = _planes(distorted)
        if ka[0].dtype != kb[0].dtype or ka[0].shape != (self.height, self.width):
            raise ValueError("frames must match the handler's size and each other's type")
        norms = (ctypes.c_float * 3)()
        dm = np.empty((self.height, self.width), np.float32) if distmap else None
        _check(lib().VshipRef_ComputeButteraugli(self._h, norms, 1 if ka[0].dtype == np.uint16 else 0,
                                                 dm.ctypes.data if dm is not None else None, self.width * 4,
                                                 ctypes.cast(a, _PP), ctypes.cast(b, _PP), s, s2),
               "VshipRef_ComputeButteraugli")
        res = (float(norms[0]), float(norms[1]), float(norms[2]))
        return (res, dm) if distmap else res

    def free(self):
        if self._h is not None:
            _check(lib().Vship_ButteraugliFree(self._h), "Vship_ButteraugliFree")
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.free()
