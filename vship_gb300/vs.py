"""Python mirror of Vship's VapourSynth functions (src/VshipLib.cpp:58-64).

VapourSynth scripts call ``core.vship.SSIMULACRA2(reference, distorted, numStream, gpu_id)``,
``core.vship.BUTTERAUGLI(reference, distorted, qnorm, intensity_multiplier, distmap, numStream,
gpu_id)`` and ``core.vship.GpuInfo(gpu_id)``. This module gives the same functions, arguments,
defaults, errors and frame properties for Python code that holds frames as arrays:

* a clip is a ``Clip``: a list of frames plus per-frame property dicts; a frame is three planes,
  either R'G'B' (float32 "RGBS", or uint16 "RGB48") or 10-bit 4:2:0 Y'CbCr (uint16 (Y, Cb, Cr),
  converted on the GPU -- the reference converts non-RGBS input with resize.Bicubic on the CPU,
  src/util/torgbs.hpp);
* SSIMULACRA2 returns the distorted clip with ``_SSIMULACRA2`` set on every frame
  (src/ssimu2/vapoursynth.hpp:59);
* BUTTERAUGLI returns the distorted clip, or with ``distmap=1`` a clip of float32 (H, W)
  distortion maps, with ``_BUTTERAUGLI_QNorm``, ``_BUTTERAUGLI_3Norm``, ``_BUTTERAUGLI_INFNorm``
  (src/butter/vapoursynth.hpp:71-73) and ``_BUTTERAUGLI_2Norm`` (documented in doc/BUTTERAUGLI.md;
  the reference never sets it; here it carries the Q-norm, which is the 2-norm for the default
  qnorm=2).

``numStream`` frames are scored concurrently, each stream with its own handler (the reference's
``threadSet`` of computing implementations, src/util/concurrency.hpp).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import threading
from dataclasses import dataclass, field

import numpy as np

import vship_gb300 as _v


class Error(RuntimeError):
    """Raised where the reference plugin calls vsapi->mapSetError (message = VshipException)."""


@dataclass
class Clip:
    frames: list
    props: list = field(default_factory=list)
    format: str = ""  # "RGBS", "RGB48", "YUV420P10" or "GRAYS"

    def __post_init__(self):
        if not self.props:
            self.props = [{} for _ in self.frames]
        if not self.format and self.frames:
            self.format = _detect_format(self.frames[0])

    def __len__(self):
        return len(self.frames)

    @property
    def size(self):
        f = self.frames[0]
        if self.format == "GRAYS":
            return f.shape[1], f.shape[0]
        return np.asarray(f[0]).shape[1], np.asarray(f[0]).shape[0]


def _detect_format(frame) -> str:
    planes = [np.asarray(p) for p in frame] if not isinstance(frame, np.ndarray) or frame.ndim == 3 else None
    if planes is None:
        return "GRAYS"
    if planes[0].shape != planes[1].shape:
        return "YUV420P10"
    return {np.dtype(np.float32): "RGBS", np.dtype(np.uint16): "RGB48"}.get(planes[0].dtype, "unknown")


def _vship_exception(code: int) -> Error:
    # the reference's VshipError::getErrorMessage layout (src/util/VshipExceptions.hpp:97-104)
    return Error(f"VshipException\n{_v.error_message(code)}\n")


def _check_inputs(reference: Clip, distorted: Clip, gpu_id: int):
    if reference.format not in ("RGBS", "RGB48", "YUV420P10"):
        raise _vship_exception(_v.NonRGBSInput)
    if (reference.format != distorted.format or reference.size != distorted.size or len(reference) != len(distorted)):
        raise _vship_exception(_v.DifferingInputType)
    try:
        _v.gpu_full_check(gpu_id)
    except _v.VshipError as e:
        raise _vship_exception(e.code) from None


def _streams(num_stream, default):
    n = default if num_stream is None else int(num_stream)
    return max(1, min(n, os.cpu_count() or 1))


class _Pool:
    """numStream workers, each owning one handler (created lazily on its thread)."""

    def __init__(self, n, make):
        self.local = threading.local()
        self.make = make
        self.handlers = []
        self.lock = threading.Lock()
        self.ex = cf.ThreadPoolExecutor(max_workers=n)

    def handler(self):
        h = getattr(self.local, "h", None)
        if h is None:
            h = self.make()
            self.local.h = h
            with self.lock:
                self.handlers.append(h)
        return h

    def map(self, fn, items):
        try:
            return list(self.ex.map(lambda it: fn(self.handler(), it), items))
        finally:
            self.ex.shutdown()
            for h in self.handlers:
                h.free()


def SSIMULACRA2(reference: Clip, distorted: Clip, numStream: int | None = None, gpu_id: int = 0) -> Clip:
    """src/ssimu2/vapoursynth.hpp:16-166. numStream defaults to the host thread count."""
    _check_inputs(reference, distorted, gpu_id)
    _v.set_device(gpu_id)
    w, h = reference.size
    pool = _Pool(_streams(numStream, os.cpu_count() or 1), lambda: _v.SSIMU2Handler(w, h))
    yuv = reference.format == "YUV420P10"

    def score(hd, i):
        a, b = reference.frames[i], distorted.frames[i]
        return hd.compute_yuv420p10(a, b) if yuv else hd.compute(a, b)

    scores = pool.map(score, range(len(reference)))
    props = [dict(p, _SSIMULACRA2=float(s)) for p, s in zip(distorted.props, scores)]
    return Clip(list(distorted.frames), props, distorted.format)


def BUTTERAUGLI(reference: Clip, distorted: Clip, qnorm: int = 2, intensity_multiplier: float = 203.0,
                distmap: int = 0, numStream: int | None = None, gpu_id: int = 0) -> Clip:
    """src/butter/vapoursynth.hpp:16-193. numStream defaults to 4."""
    _check_inputs(reference, distorted, gpu_id)
    _v.set_device(gpu_id)
    w, h = reference.size
    pool = _Pool(_streams(numStream, 4), lambda: _v.ButteraugliHandler(w, h, qnorm, intensity_multiplier))
    yuv = reference.format == "YUV420P10"

    def score(hd, i):
        a, b = reference.frames[i], distorted.frames[i]
        if yuv:
            return hd.compute_yuv420p10(a, b, distmap=bool(distmap))
        return hd.compute(a, b, distmap=bool(distmap))

    res = pool.map(score, range(len(reference)))
    frames, props = [], []
    for i, r in enumerate(res):
        norms, dm = (r if distmap else (r, None))
        p = dict(distorted.props[i])
        p["_BUTTERAUGLI_QNorm"] = float(norms[0])
        p["_BUTTERAUGLI_3Norm"] = float(norms[1])
        p["_BUTTERAUGLI_INFNorm"] = float(norms[2])
        p["_BUTTERAUGLI_2Norm"] = float(norms[0])
        props.append(p)
        frames.append(dm if distmap else distorted.frames[i])
    return Clip(frames, props, "GRAYS" if distmap else distorted.format)


def GpuInfo(gpu_id: int | None = None) -> str:
    """src/VshipLib.cpp:8-56: one line per GPU, or details of gpu_id."""
    try:
        n = _v.device_count()
    except _v.VshipError as e:
        raise _vship_exception(e.code) from None
    if gpu_id is None:
        return "".join(f"GPU {i}: {_v.device_info(i)['name']}\n" for i in range(n))
    if gpu_id < 0 or gpu_id >= n:
        raise _vship_exception(_v.BadDeviceArgument)
    d = _v.device_info(gpu_id)
    try:
        _v.gpu_full_check(gpu_id)
        ok = 1
    except _v.VshipError:
        ok = 0
    return (f"Name: {d['name']}\nMultiProcessorCount: {d['MultiProcessorCount']}\n"
            f"WarpSize: {d['WarpSize']}\nVRAMCapacity: {d['VRAMSize'] / 1e9} GB\n"
            f"Integrated: {d['integrated']}\nPassKernelCheck : {ok}\n")
