"""Shared test helpers: synthetic frames as numpy planes."""
from __future__ import annotations

import numpy as np

from vship_gb300 import synth


def u16_planes_from_rgb24(t):
    """(3, H, W) uint8 tensor -> list of three uint16 planes (v * 257, i.e. full 16-bit range)."""
    a = t.cpu().numpy().astype(np.uint16) * 257
    return [np.ascontiguousarray(a[c]) for c in range(3)]


def float_planes(t):
    a = t.cpu().numpy().astype(np.float32)
    return [np.ascontiguousarray(a[c]) for c in range(3)]


def padded(planes, pad_bytes: int, fill: int = 0xFF):
    """Copy planes into rows with `pad_bytes` of extra stride filled with `fill` (same layout as
    the reference's stride-padding test, test/basic_metric_math_test.cpp:21-33)."""
    out = []
    for p in planes:
        h, w = p.shape
        row = w * p.itemsize + pad_bytes
        buf = np.full((h, row), fill, np.uint8)
        buf[:, : w * p.itemsize] = p.view(np.uint8).reshape(h, -1)
        out.append(buf[:, : w * p.itemsize].view(p.dtype))
    return out


def grating_float_pair(h, w, t=0, seed=7, distortion="dct"):
    r, d = synth.rgb_float_pair(h, w, t, seed, distortion)
    return float_planes(r), float_planes(d)
