"""vship_gb300: GB300-native SSIMULACRA2 and Butteraugli scoring behind Vship's C ABI.

The product is ``libvship.so`` (hand-written sm_103a CUDA kernels plus the C ABI declared in
``include/VshipAPI.h``). This module binds it with ctypes and mirrors the reference's interfaces
for Python callers: handler objects with the semantics of ``Vship_SSIMU2Init`` /
``Vship_ComputeSSIMU2*`` / ``Vship_ButteraugliInit*`` (src/VshipAPI.h) and, in ``vship_gb300.vs``,
the ``vship.SSIMULACRA2`` / ``vship.BUTTERAUGLI`` clip functions (src/VshipLib.cpp:58-64).

There is no CPU fallback: if the shared library is missing or no GPU is present, calls raise.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libvship.so")

# Vship_Exception (src/VshipAPI.h:35-58)
NoError, OutOfVRAM, OutOfRAM, DifferingInputType, NonRGBSInput, DeviceCountError, NoDeviceDetected, \
    BadDeviceArgument, BadDeviceCode, BadHandler, BadPointer, BadErrorType = range(12)
EXCEPTION_NAMES = ["NoError", "OutOfVRAM", "OutOfRAM", "DifferingInputType", "NonRGBSInput", "DeviceCountError",
                   "NoDeviceDetected", "BadDeviceArgument", "BadDeviceCode", "BadHandler", "BadPointer",
                   "BadErrorType"]

# Vship_InputType
IN_UINT8, IN_UINT16, IN_HALF, IN_FLOAT, IN_YUV = 0, 1, 2, 3, 4
IN_YUV420P10 = IN_YUV  # the default Y'CbCr format (10-bit 4:2:0, BT.709, limited, left siting)
BUTTER_HALF_BANDS = 1  # Vship_ButterHalfBands: Butteraugli UHF bands stored as FP16
SSIMU2_FP16_DELTAS = 1  # Vship_SSIMU2Fp16Deltas: the distorted pyramid as FP16 deltas from the reference's


class VshipError(RuntimeError):
    def __init__(self, code: int, where: str = ""):
        self.code = int(code)
        self.name = EXCEPTION_NAMES[self.code] if 0 <= self.code < len(EXCEPTION_NAMES) else "BadErrorType"
        super().__init__(f"{where}: {error_message(self.code)}" if where else error_message(self.code))


class Version(ctypes.Structure):
    _fields_ = [("major", ctypes.c_int), ("minor", ctypes.c_int), ("minorMinor", ctypes.c_int),
                ("backend", ctypes.c_int)]


class DeviceInfo(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 256), ("VRAMSize", ctypes.c_uint64), ("integrated", ctypes.c_int),
                ("MultiProcessorCount", ctypes.c_int), ("WarpSize", ctypes.c_int)]


class Handler(ctypes.Structure):
    _fields_ = [("id", ctypes.c_int)]


class ButteraugliScore(ctypes.Structure):
    _fields_ = [("norm2", ctypes.c_int), ("norm3", ctypes.c_int), ("norminf", ctypes.c_int)]


class DeviceFrame(ctypes.Structure):
    _fields_ = [("plane", ctypes.c_void_p * 3), ("stride", ctypes.c_int64), ("stride_c", ctypes.c_int64)]


# Every exported entry point: name -> (restype, argtypes). The tests check this list against
# include/VshipAPI.h and against the library's dynamic symbol table.
_PP = ctypes.POINTER(ctypes.c_void_p)
_H = Handler
_E = ctypes.c_int
_IP = ctypes.POINTER(ctypes.c_int)


class YuvFormat(ctypes.Structure):
    """Vship_YuvFormat: bits 8..16, log2 chroma subsampling, H.273 matrix (2 = by height), range
    (0 limited, 1 full), chroma location (0 left, 1 center, 2 top-left, 3 top, 4 bottom-left,
    5 bottom), transfer and primaries (H.273 ids)."""
    _fields_ = [("bits", ctypes.c_int), ("subsampling_w", ctypes.c_int), ("subsampling_h", ctypes.c_int),
                ("matrix", ctypes.c_int), ("range", ctypes.c_int), ("chroma_location", ctypes.c_int),
                ("transfer", ctypes.c_int), ("primaries", ctypes.c_int)]


def yuv_format(bits=10, subsampling=(1, 1), matrix=1, full_range=False, chroma_location=0, transfer=1,
               primaries=1) -> YuvFormat:
    """H.273 ids: transfer 1/6/14/15/2 (BT.709 family), 13 sRGB, 4 gamma 2.2, 5 gamma 2.8, 8 linear;
    primaries 1/2 BT.709, 9 BT.2020."""
    return YuvFormat(int(bits), int(subsampling[0]), int(subsampling[1]), int(matrix), 1 if full_range else 0,
                     int(chroma_location), int(transfer), int(primaries))


class ServeRequest(ctypes.Structure):
    _fields_ = [("request_id", ctypes.c_uint64), ("metric", ctypes.c_int), ("resolution", ctypes.c_int),
                ("source_key", ctypes.c_uint64), ("source", DeviceFrame), ("npairs", ctypes.c_int),
                ("candidates", ctypes.POINTER(DeviceFrame)), ("results", ctypes.POINTER(ctypes.c_double))]


class ServeCompletion(ctypes.Structure):
    _fields_ = [("request_id", ctypes.c_uint64), ("status", ctypes.c_int), ("latency_seconds", ctypes.c_double)]


SIGNATURES = {
    "Vship_GetVersion": (Version, []),
    "Vship_GetDeviceCount": (_E, [ctypes.POINTER(ctypes.c_int)]),
    "Vship_SetDevice": (_E, [ctypes.c_int]),
    "Vship_GetDeviceInfo": (_E, [ctypes.POINTER(DeviceInfo), ctypes.c_int]),
    "Vship_GPUFullCheck": (_E, [ctypes.c_int]),
    "Vship_GetErrorMessage": (ctypes.c_int, [ctypes.c_int, ctypes.c_char_p, ctypes.c_int]),
    "Vship_PinnedMalloc": (_E, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_uint64]),
    "Vship_PinnedFree": (_E, [ctypes.c_void_p]),
    "Vship_SSIMU2Init": (_E, [ctypes.POINTER(_H), ctypes.c_int, ctypes.c_int]),
    "Vship_SSIMU2Free": (_E, [_H]),
    "Vship_ComputeSSIMU2Float": (_E, [_H, ctypes.POINTER(ctypes.c_double), _PP, _PP, ctypes.c_int64]),
    "Vship_ComputeSSIMU2Floatv2": (_E, [_H, ctypes.POINTER(ctypes.c_double), _PP, _PP, ctypes.c_int64,
                                        ctypes.c_int64]),
    "Vship_ComputeSSIMU2Uint16": (_E, [_H, ctypes.POINTER(ctypes.c_double), _PP, _PP, ctypes.c_int64]),
    "Vship_ComputeSSIMU2Uint16v2": (_E, [_H, ctypes.POINTER(ctypes.c_double), _PP, _PP, ctypes.c_int64,
                                         ctypes.c_int64]),
    "Vship_ButteraugliInit": (_E, [ctypes.POINTER(_H), ctypes.c_int, ctypes.c_int, ctypes.c_float]),
    "Vship_ButteraugliInitv2": (_E, [ctypes.POINTER(_H), ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float]),
    "Vship_ButteraugliFree": (_E, [_H]),
    "Vship_ComputeButteraugliFloat": (_E, [_H, ctypes.POINTER(ButteraugliScore), ctypes.c_void_p, ctypes.c_int64,
                                           _PP, _PP, ctypes.c_int64]),
    "Vship_ComputeButteraugliFloatv2": (_E, [_H, ctypes.POINTER(ButteraugliScore), ctypes.c_void_p,
                                             ctypes.c_int64, _PP, _PP, ctypes.c_int64, ctypes.c_int64]),
    "Vship_ComputeButteraugliUint16": (_E, [_H, ctypes.POINTER(ButteraugliScore), ctypes.c_void_p, ctypes.c_int64,
                                            _PP, _PP, ctypes.c_int64]),
    "Vship_ComputeButteraugliUint16v2": (_E, [_H, ctypes.POINTER(ButteraugliScore), ctypes.c_void_p,
                                              ctypes.c_int64, _PP, _PP, ctypes.c_int64, ctypes.c_int64]),
    "Vship_ComputeButteraugliFloatv3": (_E, [_H, ctypes.POINTER(ctypes.c_double), ctypes.c_void_p, ctypes.c_int64,
                                             _PP, _PP, ctypes.c_int64, ctypes.c_int64]),
    "Vship_ComputeButteraugliUint16v3": (_E, [_H, ctypes.POINTER(ctypes.c_double), ctypes.c_void_p,
                                              ctypes.c_int64, _PP, _PP, ctypes.c_int64, ctypes.c_int64]),
    "Vship_ComputeSSIMU2Yuv420p10": (_E, [_H, ctypes.POINTER(ctypes.c_double), _PP, ctypes.POINTER(ctypes.c_int64),
                                          _PP, ctypes.POINTER(ctypes.c_int64)]),
    "Vship_ComputeButteraugliYuv420p10": (_E, [_H, ctypes.POINTER(ctypes.c_double), ctypes.c_void_p, ctypes.c_int64,
                                               _PP, ctypes.POINTER(ctypes.c_int64), _PP,
                                               ctypes.POINTER(ctypes.c_int64)]),
    "Vship_SSIMU2BatchInit": (_E, [ctypes.POINTER(_H), ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "Vship_SSIMU2ComputeDeviceAsync": (_E, [_H, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                            ctypes.c_void_p]),
    "Vship_SSIMU2DeviceBytes": (ctypes.c_uint64, [ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "Vship_SSIMU2InitEx": (_E, [ctypes.POINTER(_H), ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "Vship_SSIMU2BatchInitEx": (_E, [ctypes.POINTER(_H), ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "Vship_SSIMU2DeviceBytesEx": (ctypes.c_uint64, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "Vship_ButteraugliBatchInit": (_E, [ctypes.POINTER(_H), ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                        ctypes.c_int]),
    "Vship_ButteraugliComputeDeviceAsync": (_E, [_H, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                                 ctypes.c_void_p, ctypes.c_void_p]),
    "Vship_ButteraugliDeviceBytes": (ctypes.c_uint64, [ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "Vship_ButteraugliInitEx": (_E, [ctypes.POINTER(_H), ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                     ctypes.c_int]),
    "Vship_ButteraugliBatchInitEx": (_E, [ctypes.POINTER(_H), ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                          ctypes.c_float, ctypes.c_int, ctypes.c_int]),
    "Vship_ButteraugliDeviceBytesEx": (ctypes.c_uint64, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "Vship_ComputeSSIMU2DeviceNoAlloc": (_E, [ctypes.POINTER(DeviceFrame), ctypes.POINTER(DeviceFrame), ctypes.c_int,
                                              ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]),
    "Vship_MultiInit": (_E, [ctypes.POINTER(_H), ctypes.c_int, _IP, _IP, _IP, _IP, ctypes.c_int, ctypes.c_int,
                             ctypes.c_float, ctypes.c_char_p]),
    "Vship_MultiFree": (_E, [_H]),
    "Vship_MultiComputeDeviceAsync": (_E, [_H, ctypes.c_int, ctypes.POINTER(DeviceFrame), _IP, ctypes.c_int,
                                           ctypes.POINTER(DeviceFrame), _IP, ctypes.c_int, ctypes.c_void_p,
                                           ctypes.c_void_p, ctypes.c_void_p]),
    "Vship_MultiKnobs": (ctypes.c_int, [_H, ctypes.c_char_p, ctypes.c_int]),
    "Vship_MultiDeviceBytes": (ctypes.c_uint64, [ctypes.c_int, _IP, _IP, _IP, _IP, ctypes.c_int]),
    "Vship_ServeCreate": (_E, [ctypes.POINTER(_H), ctypes.c_int, _IP, _IP, ctypes.c_int, ctypes.c_uint64,
                               ctypes.c_uint64, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float]),
    "Vship_ServeSubmit": (_E, [_H, ctypes.POINTER(ServeRequest)]),
    "Vship_ServePoll": (ctypes.c_int, [_H, ctypes.POINTER(ServeCompletion), ctypes.c_int, ctypes.c_double]),
    "Vship_ServeDrain": (_E, [_H]),
    "Vship_ServeCancel": (_E, [_H, ctypes.c_uint64]),
    "Vship_ServeStats": (ctypes.c_int, [_H, ctypes.c_char_p, ctypes.c_int]),
    "Vship_ServeDestroy": (_E, [_H]),
    "Vship_SSIMU2SetYuvFormat": (_E, [_H, ctypes.POINTER(YuvFormat)]),
    "Vship_ButteraugliSetYuvFormat": (_E, [_H, ctypes.POINTER(YuvFormat)]),
    "Vship_ComputeSSIMU2Yuv": (_E, [_H, ctypes.POINTER(ctypes.c_double), _PP, ctypes.POINTER(ctypes.c_int64), _PP,
                                    ctypes.POINTER(ctypes.c_int64)]),
    "Vship_ComputeButteraugliYuv": (_E, [_H, ctypes.POINTER(ctypes.c_double), ctypes.c_void_p, ctypes.c_int64, _PP,
                                         ctypes.POINTER(ctypes.c_int64), _PP, ctypes.POINTER(ctypes.c_int64)]),
    "Vship_MultiSetYuvFormat": (_E, [_H, ctypes.POINTER(YuvFormat)]),
    "Vship_ServeSetYuvFormat": (_E, [_H, ctypes.POINTER(YuvFormat)]),
    "Vship_ProfileSetEnabled": (None, [ctypes.c_int]),
    "Vship_ProfileReport": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int]),
}

_lib = None


def lib() -> ctypes.CDLL:
    """Load libvship.so (built by ``vship_gb300.build``). Raises if it is missing."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run `python -m vship_gb300.build` (needs nvcc)")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def error_message(code: int) -> str:
    L = lib()
    n = L.Vship_GetErrorMessage(int(code), None, 0)
    buf = ctypes.create_string_buffer(n)
    L.Vship_GetErrorMessage(int(code), buf, n)
    return buf.value.decode()


def _check(rc: int, where: str):
    if rc != NoError:
        raise VshipError(rc, where)


def profile_enable(on: bool = True) -> None:
    """Bracket every kernel launch with CUDA events (see Vship_ProfileSetEnabled)."""
    lib().Vship_ProfileSetEnabled(1 if on else 0)


def profile_report() -> dict:
    """{kernel: (launches, total_ms)} since the last report; synchronises the recorded events."""
    import json
    L = lib()
    buf = ctypes.create_string_buffer(1 << 20)  # one call: a report clears the records
    L.Vship_ProfileReport(buf, len(buf))
    return {k: (int(v[0]), float(v[1])) for k, v in json.loads(buf.value.decode() or "{}").items()}


def version():
    v = lib().Vship_GetVersion()
    return (v.major, v.minor, v.minorMinor, "Cuda" if v.backend == 1 else "HIP")


def device_count() -> int:
    n = ctypes.c_int()
    _check(lib().Vship_GetDeviceCount(ctypes.byref(n)), "Vship_GetDeviceCount")
    return n.value


def device_info(gpu_id: int = 0) -> dict:
    d = DeviceInfo()
    _check(lib().Vship_GetDeviceInfo(ctypes.byref(d), gpu_id), "Vship_GetDeviceInfo")
    return {"name": d.name.decode(errors="replace"), "VRAMSize": d.VRAMSize, "integrated": d.integrated,
            "MultiProcessorCount": d.MultiProcessorCount, "WarpSize": d.WarpSize}


def gpu_full_check(gpu_id: int = 0) -> None:
    _check(lib().Vship_GPUFullCheck(gpu_id), "Vship_GPUFullCheck")


def set_device(gpu_id: int) -> None:
    _check(lib().Vship_SetDevice(gpu_id), "Vship_SetDevice")


# ------------------------------------------------------------------------------------------
# host planes

def planes_of(frame):
    """Accept a (3, H, W) array or a sequence of three (H, W) arrays (float32 or uint16, rows
    contiguous, one shared row stride). Returns (ctypes pointer array, stride, w, h, dtype, keep)."""
    planes = [np.asarray(p) for p in frame]
    if len(planes) != 3:
        raise ValueError("a frame has three planes (R, G, B)")
    dt = planes[0].dtype
    if dt not in (np.float32, np.uint16):
        raise TypeError("planes must be float32 or uint16")
    h, w = planes[0].shape
    strides = {p.strides[0] for p in planes}
    for p in planes:
        if p.dtype != dt or p.shape != (h, w) or p.strides[1] != dt.itemsize:
            raise ValueError("planes must share dtype and shape, with contiguous rows")
    if len(strides) != 1:
        raise ValueError("the three planes must share one row stride")
    arr = (ctypes.c_void_p * 3)(*[p.ctypes.data for p in planes])
    return arr, strides.pop(), w, h, dt, planes


def _yuv_planes(frame, w, h, fmt=None):
    """(Y, Cb, Cr) arrays of a w x h frame in format fmt (default 10-bit 4:2:0) -> (pointer
    array, stride array). Samples: uint8 for 8 bits, uint16 above."""
    planes = [np.asarray(p) for p in frame]
    ssw, ssh, bits = (1, 1, 10) if fmt is None else (fmt.subsampling_w, fmt.subsampling_h, fmt.bits)
    cw, ch = ((w + 1) // 2 if ssw else w), ((h + 1) // 2 if ssh else h)
    shapes = [(h, w), (ch, cw), (ch, cw)]
    dt = np.uint8 if bits == 8 else np.uint16
    for p, shp in zip(planes, shapes):
        if p.dtype != dt or p.shape != shp or p.strides[1] != p.itemsize:
            raise VshipError(DifferingInputType, f"Y'CbCr planes must be {np.dtype(dt).name} {shapes}")
    ptrs = (ctypes.c_void_p * 3)(*[p.ctypes.data for p in planes])
    strides = (ctypes.c_int64 * 3)(*[p.strides[0] for p in planes])
    return ptrs, strides


class SSIMU2Handler:
    """One SSIMULACRA2 scorer for a fixed resolution (Vship_SSIMU2Init / Compute / Free);
    fp16_deltas=True stores the distorted image's pyramid as FP16 differences from the
    reference's (Vship_SSIMU2InitEx with Vship_SSIMU2Fp16Deltas)."""

    def __init__(self, width: int, height: int, fp16_deltas: bool = False):
        self.width, self.height = int(width), int(height)
        h = Handler()
        if fp16_deltas:
            _check(lib().Vship_SSIMU2InitEx(ctypes.byref(h), self.width, self.height, SSIMU2_FP16_DELTAS),
                   "Vship_SSIMU2InitEx")
        else:
            _check(lib().Vship_SSIMU2Init(ctypes.byref(h), self.width, self.height), "Vship_SSIMU2Init")
        self._h = h  # only a created handler is ever freed

    def compute(self, reference, distorted) -> float:
        a1, s1, w, h, dt, k1 = planes_of(reference)
        a2, s2, w2, h2, dt2, k2 = planes_of(distorted)
        if (w, h) != (self.width, self.height) or (w2, h2) != (w, h) or dt != dt2:
            raise VshipError(DifferingInputType, "SSIMU2Handler.compute")
        out = ctypes.c_double()
        f = lib().Vship_ComputeSSIMU2Floatv2 if dt == np.float32 else lib().Vship_ComputeSSIMU2Uint16v2
        _check(f(self._h, ctypes.byref(out), ctypes.cast(a1, _PP), ctypes.cast(a2, _PP), s1, s2),
               "Vship_ComputeSSIMU2")
        return out.value

    def compute_yuv420p10(self, reference, distorted) -> float:
        """Score 10-bit 4:2:0 frames given as (Y, Cb, Cr) uint16 arrays (Vship_ComputeSSIMU2Yuv420p10)."""
        a1, s1 = _yuv_planes(reference, self.width, self.height)
        a2, s2 = _yuv_planes(distorted, self.width, self.height)
        out = ctypes.c_double()
        _check(lib().Vship_ComputeSSIMU2Yuv420p10(self._h, ctypes.byref(out), ctypes.cast(a1, _PP), s1,
                                                  ctypes.cast(a2, _PP), s2), "Vship_ComputeSSIMU2Yuv420p10")
        return out.value

    def set_yuv_format(self, fmt: YuvFormat) -> None:
        _check(lib().Vship_SSIMU2SetYuvFormat(self._h, ctypes.byref(fmt)), "Vship_SSIMU2SetYuvFormat")
        self._fmt = fmt

    def compute_yuv(self, reference, distorted) -> float:
        """Score Y'CbCr frames in the format set by set_yuv_format (Vship_ComputeSSIMU2Yuv)."""
        fmt = getattr(self, "_fmt", None)
        a1, s1 = _yuv_planes(reference, self.width, self.height, fmt)
        a2, s2 = _yuv_planes(distorted, self.width, self.height, fmt)
        out = ctypes.c_double()
        _check(lib().Vship_ComputeSSIMU2Yuv(self._h, ctypes.byref(out), ctypes.cast(a1, _PP), s1,
                                            ctypes.cast(a2, _PP), s2), "Vship_ComputeSSIMU2Yuv")
        return out.value

    def free(self):
        if self._h is not None:
            _check(lib().Vship_SSIMU2Free(self._h), "Vship_SSIMU2Free")
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.free()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class ButteraugliHandler:
    """One Butteraugli scorer (Vship_ButteraugliInitv2 / Compute*v3 / Free); half_bands=True stores
    the UHF bands as FP16 (Vship_ButteraugliInitEx with Vship_ButterHalfBands)."""

    def __init__(self, width: int, height: int, qnorm: int = 2, intensity_multiplier: float = 203.0,
                 half_bands: bool = False):
        self.width, self.height = int(width), int(height)
        self.qnorm, self.intensity = int(qnorm), float(intensity_multiplier)
        h = Handler()
        if half_bands:
            _check(lib().Vship_ButteraugliInitEx(ctypes.byref(h), self.width, self.height, self.qnorm,
                                                 ctypes.c_float(self.intensity), BUTTER_HALF_BANDS),
                   "Vship_ButteraugliInitEx")
        else:
            _check(lib().Vship_ButteraugliInitv2(ctypes.byref(h), self.width, self.height, self.qnorm,
                                                 ctypes.c_float(self.intensity)), "Vship_ButteraugliInitv2")
        self._h = h  # only a created handler is ever freed

    def compute(self, reference, distorted, distmap: bool = False):
        """Returns (norm_q, norm_3, norm_inf) and, with distmap=True, the float32 (H, W) map."""
        a1, s1, w, h, dt, k1 = planes_of(reference)
        a2, s2, w2, h2, dt2, k2 = planes_of(distorted)
        if (w, h) != (self.width, self.height) or (w2, h2) != (w, h) or dt != dt2:
            raise VshipError(DifferingInputType, "ButteraugliHandler.compute")
        norms = (ctypes.c_double * 3)()
        dm = np.empty((h, w), np.float32) if distmap else None
        f = lib().Vship_ComputeButteraugliFloatv3 if dt == np.float32 else lib().Vship_ComputeButteraugliUint16v3
        _check(f(self._h, norms, dm.ctypes.data if dm is not None else None, w * 4,
                 ctypes.cast(a1, _PP), ctypes.cast(a2, _PP), s1, s2), "Vship_ComputeButteraugli")
        res = (norms[0], norms[1], norms[2])
        return (res, dm) if distmap else res

    def compute_yuv420p10(self, reference, distorted, distmap: bool = False):
        """Butteraugli of 10-bit 4:2:0 frames given as (Y, Cb, Cr) uint16 arrays."""
        a1, s1 = _yuv_planes(reference, self.width, self.height)
        a2, s2 = _yuv_planes(distorted, self.width, self.height)
        norms = (ctypes.c_double * 3)()
        dm = np.empty((self.height, self.width), np.float32) if distmap else None
        _check(lib().Vship_ComputeButteraugliYuv420p10(self._h, norms, dm.ctypes.data if dm is not None else None,
                                                       self.width * 4, ctypes.cast(a1, _PP), s1,
                                                       ctypes.cast(a2, _PP), s2), "Vship_ComputeButteraugliYuv420p10")
        res = (norms[0], norms[1], norms[2])
        return (res, dm) if distmap else res

    def set_yuv_format(self, fmt: YuvFormat) -> None:
        _check(lib().Vship_ButteraugliSetYuvFormat(self._h, ctypes.byref(fmt)), "Vship_ButteraugliSetYuvFormat")
        self._fmt = fmt

    def compute_yuv(self, reference, distorted, distmap: bool = False):
        """Butteraugli of Y'CbCr frames in the format set by set_yuv_format."""
        fmt = getattr(self, "_fmt", None)
        a1, s1 = _yuv_planes(reference, self.width, self.height, fmt)
        a2, s2 = _yuv_planes(distorted, self.width, self.height, fmt)
        norms = (ctypes.c_double * 3)()
        dm = np.empty((self.height, self.width), np.float32) if distmap else None
        _check(lib().Vship_ComputeButteraugliYuv(self._h, norms, dm.ctypes.data if dm is not None else None,
                                                 self.width * 4, ctypes.cast(a1, _PP), s1,
                                                 ctypes.cast(a2, _PP), s2), "Vship_ComputeButteraugliYuv")
        res = (norms[0], norms[1], norms[2])
        return (res, dm) if distmap else res

    def free(self):
        if self._h is not None:
            _check(lib().Vship_ButteraugliFree(self._h), "Vship_ButteraugliFree")
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.free()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class SSIMU2Batch:
    """Batched device-resident SSIMU2 (Vship_SSIMU2BatchInit / Vship_SSIMU2ComputeDeviceAsync)."""

    def __init__(self, width: int, height: int, max_pairs: int, fp16_deltas: bool = False):
        self.width, self.height, self.max_pairs = int(width), int(height), int(max_pairs)
        h = Handler()
        _check(lib().Vship_SSIMU2BatchInitEx(ctypes.byref(h), self.width, self.height, self.max_pairs,
                                             SSIMU2_FP16_DELTAS if fp16_deltas else 0), "Vship_SSIMU2BatchInitEx")
        self._h = h  # only a created handler is ever freed

    def set_yuv_format(self, fmt: YuvFormat) -> None:
        _check(lib().Vship_SSIMU2SetYuvFormat(self._h, ctypes.byref(fmt)), "Vship_SSIMU2SetYuvFormat")

    def compute_async(self, frames_dev_ptr: int, npairs: int, input_type: int, scores_dev_ptr: int,
                      stream_ptr: int = 0) -> None:
        _check(lib().Vship_SSIMU2ComputeDeviceAsync(self._h, ctypes.c_void_p(frames_dev_ptr), int(npairs),
                                                    int(input_type), ctypes.c_void_p(scores_dev_ptr),
                                                    ctypes.c_void_p(stream_ptr)), "Vship_SSIMU2ComputeDeviceAsync")

    def free(self):
        if self._h is not None:
            _check(lib().Vship_SSIMU2Free(self._h), "Vship_SSIMU2Free")
            self._h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class ButteraugliBatch:
    """Batched device-resident Butteraugli (Vship_ButteraugliBatchInit / ComputeDeviceAsync)."""

    def __init__(self, width: int, height: int, max_pairs: int, qnorm: int = 2, intensity_multiplier: float = 203.0,
                 half_bands: bool = False):
        self.width, self.height, self.max_pairs = int(width), int(height), int(max_pairs)
        h = Handler()
        _check(lib().Vship_ButteraugliBatchInitEx(ctypes.byref(h), self.width, self.height, int(qnorm),
                                                  ctypes.c_float(intensity_multiplier), self.max_pairs,
                                                  BUTTER_HALF_BANDS if half_bands else 0),
               "Vship_ButteraugliBatchInitEx")
        self._h = h  # only a created handler is ever freed

    def set_yuv_format(self, fmt: YuvFormat) -> None:
        _check(lib().Vship_ButteraugliSetYuvFormat(self._h, ctypes.byref(fmt)), "Vship_ButteraugliSetYuvFormat")

    def compute_async(self, frames_dev_ptr: int, npairs: int, input_type: int, norms_dev_ptr: int,
                      distmaps_dev_ptr: int = 0, stream_ptr: int = 0) -> None:
        _check(lib().Vship_ButteraugliComputeDeviceAsync(self._h, ctypes.c_void_p(frames_dev_ptr), int(npairs),
                                                         int(input_type), ctypes.c_void_p(norms_dev_ptr),
                                                         ctypes.c_void_p(distmaps_dev_ptr or None),
                                                         ctypes.c_void_p(stream_ptr)),
               "Vship_ButteraugliComputeDeviceAsync")

    def free(self):
        if self._h is not None:
            _check(lib().Vship_ButteraugliFree(self._h), "Vship_ButteraugliFree")
            self._h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


MULTI_SSIMU2, MULTI_BUTTERAUGLI, MULTI_FP16, MULTI_NO_GRAPH, MULTI_AUTOTUNE = 1, 2, 4, 8, 16
MULTI_BUTTER_HALF = 32  # Vship_MultiButterHalfBands


def _ints(v):
    return (ctypes.c_int * len(v))(*[int(x) for x in v])


def _frames(frames):
    arr = (DeviceFrame * len(frames))()
    for i, fr in enumerate(frames):
        planes, stride = fr[0], fr[1]
        for c in range(3):
            arr[i].plane[c] = int(planes[c])
        arr[i].stride = int(stride)
        arr[i].stride_c = int(fr[2]) if len(fr) > 2 else int(stride)
    return arr


class MultiScorer:
    """Batched multi-resolution scoring with source reuse (Vship_MultiInit /
    Vship_MultiComputeDeviceAsync). ``resolutions`` is a list of (width, height); the capacities
    are per resolution."""

    def __init__(self, resolutions, max_sources, max_pairs, flags=MULTI_SSIMU2, qnorm=2,
                 intensity_multiplier=203.0, tune_cache=None):
        self.resolutions = [(int(w), int(h)) for w, h in resolutions]
        self.flags = int(flags)
        n = len(self.resolutions)
        h = Handler()
        _check(lib().Vship_MultiInit(ctypes.byref(h), n, _ints([w for w, _ in self.resolutions]),
                                     _ints([h for _, h in self.resolutions]), _ints(max_sources), _ints(max_pairs),
                                     self.flags, int(qnorm), ctypes.c_float(intensity_multiplier),
                                     tune_cache.encode() if tune_cache else None), "Vship_MultiInit")
        self._h = h  # only a created handler is ever freed

    @staticmethod
    def device_bytes(resolutions, max_sources, max_pairs, flags=MULTI_SSIMU2) -> int:
        return int(lib().Vship_MultiDeviceBytes(len(resolutions), _ints([w for w, _ in resolutions]),
                                                _ints([h for _, h in resolutions]), _ints(max_sources),
                                                _ints(max_pairs), int(flags)))

    def compute_async(self, sources, source_res, candidates, candidate_source, input_type: int,
                      ssimu2_dev_ptr: int = 0, butter_dev_ptr: int = 0, stream_ptr: int = 0) -> None:
        """sources / candidates: [(planes, stride_bytes[, chroma_stride_bytes]), ...] of device
        pointers; results land in device memory (npairs doubles / 3*npairs doubles)."""
        _check(lib().Vship_MultiComputeDeviceAsync(self._h, len(sources), _frames(sources), _ints(source_res),
                                                   len(candidates), _frames(candidates), _ints(candidate_source),
                                                   int(input_type), ctypes.c_void_p(ssimu2_dev_ptr or None),
                                                   ctypes.c_void_p(butter_dev_ptr or None),
                                                   ctypes.c_void_p(stream_ptr)), "Vship_MultiComputeDeviceAsync")

    def set_yuv_format(self, fmt: YuvFormat) -> None:
        _check(lib().Vship_MultiSetYuvFormat(self._h, ctypes.byref(fmt)), "Vship_MultiSetYuvFormat")

    def knobs(self) -> dict:
        import json

        n = lib().Vship_MultiKnobs(self._h, None, 0)
        buf = ctypes.create_string_buffer(n)
        lib().Vship_MultiKnobs(self._h, buf, n)
        return json.loads(buf.value.decode())

    def free(self):
        if self._h is not None:
            _check(lib().Vship_MultiFree(self._h), "Vship_MultiFree")
            self._h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


SERVE_SSIMU2, SERVE_BUTTERAUGLI = 0, 1
SERVE_CANCELLED = -1
SERVE_FP32_CANDIDATES = 1
SERVE_BUTTER_HALF_BANDS = 2  # Vship_ServeButterHalfBands


class Server:
    """Serving runtime (Vship_ServeCreate / Submit / Poll). ``resolutions`` is a list of
    (width, height). Results land in numpy float64 arrays the caller passes to submit (kept
    referenced here until their completion is polled)."""

    def __init__(self, resolutions, input_type=4, admission_bytes=64 << 30, cache_bytes=16 << 30,
                 max_batch_pairs=32, flags=0, qnorm=2, intensity_multiplier=203.0):
        self.resolutions = [(int(w), int(h)) for w, h in resolutions]
        h = Handler()
        self._live = {}
        _check(lib().Vship_ServeCreate(ctypes.byref(h), len(self.resolutions),
                                       _ints([w for w, _ in self.resolutions]), _ints([h for _, h in self.resolutions]),
                                       int(input_type), int(admission_bytes), int(cache_bytes), int(max_batch_pairs),
                                       int(flags), int(qnorm), ctypes.c_float(intensity_multiplier)),
               "Vship_ServeCreate")
        self._h = h  # only a created handler is ever freed

    def submit(self, request_id, metric, resolution, source_key, source, candidates, out):
        """source / candidates: (planes, stride_bytes[, chroma_stride_bytes]) of device pointers;
        out: C-contiguous float64 numpy array of npairs (SSIMU2) or 3*npairs (Butteraugli)."""
        import numpy as np
        assert out.dtype == np.float64 and out.flags["C_CONTIGUOUS"]
        src = _frames([source])
        cands = _frames(candidates)
        q = ServeRequest(int(request_id), int(metric), int(resolution), int(source_key), src[0], len(candidates),
                         ctypes.cast(cands, ctypes.POINTER(DeviceFrame)),
                         out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        self._live[int(request_id)] = out
        rc = lib().Vship_ServeSubmit(self._h, ctypes.byref(q))
        if rc:
            self._live.pop(int(request_id), None)
            _check(rc, "Vship_ServeSubmit")

    def poll(self, max_n=256, timeout=0.0):
        """[(request_id, status, latency_seconds), ...] of requests completed since the last poll."""
        buf = (ServeCompletion * max_n)()
        n = lib().Vship_ServePoll(self._h, buf, max_n, float(timeout))
        out = []
        for i in range(n):
            rid = int(buf[i].request_id)
            self._live.pop(rid, None)
            out.append((rid, int(buf[i].status), float(buf[i].latency_seconds)))
        return out

    def set_yuv_format(self, fmt: YuvFormat) -> None:
        _check(lib().Vship_ServeSetYuvFormat(self._h, ctypes.byref(fmt)), "Vship_ServeSetYuvFormat")

    def cancel(self, request_id) -> bool:
        """True when the request was still queued and is withdrawn (reported with status
        SERVE_CANCELLED)."""
        return lib().Vship_ServeCancel(self._h, int(request_id)) == 0

    def drain(self):
        _check(lib().Vship_ServeDrain(self._h), "Vship_ServeDrain")

    def stats(self) -> dict:
        import json
        n = lib().Vship_ServeStats(self._h, None, 0)
        buf = ctypes.create_string_buffer(n)
        lib().Vship_ServeStats(self._h, buf, n)
        return json.loads(buf.value.decode())

    def free(self):
        if self._h is not None:
            _check(lib().Vship_ServeDestroy(self._h), "Vship_ServeDestroy")
            self._h = None
            self._live.clear()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def device_frames_table(frames, device="cuda"):
    """Pack [(planes, stride_bytes[, chroma_stride_bytes]), ...] of device pointers into a device
    array of Vship_DeviceFrame held in a torch uint8 tensor."""
    import torch

    arr = _frames(frames)
    host = torch.frombuffer(bytearray(bytes(arr)), dtype=torch.uint8)
    return host.to(device)
