"""SSIMULACRA2 parity: libvship.so (sm_103a kernels, called through the C ABI) against the CPU
oracle.

Tolerance: 1e-3 absolute on the score against the FP64 oracle. On tiny frames the reference's own
FP32 formulation (the FP32 oracle) drifts from FP64 by more than that, because the coarse scales
hold a handful of pixels and sigma = E[x^2] - E[x]^2 cancels; there the bound is twice the FP32
formulation's own error, i.e. the GPU must be at least about as accurate as the reference's math.
The kernels form the moments on tile-shifted values, so in practice they sit closer to FP64."""
import ctypes
import threading

import numpy as np
import pytest

from helpers import float_planes, grating_float_pair, padded, u16_planes_from_rgb24
from vship_gb300 import synth

pytestmark = pytest.mark.gpu

TOL = 1e-3


def test_kat_reference_size_identical_is_100(vlib):
    # test/basic_metric_math_test.cpp:41-61: 5076x9400 float frames, stride 30000, the distorted
    # frame's padding filled with 0xFF -> exactly 100.
    w, h, stride = 5076, 9400, 30000
    z = [np.zeros((h, w), np.float32) for _ in range(3)]
    a = padded(z, stride - 4 * w, 0x00)
    b = padded(z, stride - 4 * w, 0xFF)
    with vlib.SSIMU2Handler(w, h) as hd:
        assert hd.compute(a, b) == 100.0


def test_identical_content_is_100(vlib):
    r, _ = synth.rgb24_pair(200, 120, seed=9)
    a = u16_planes_from_rgb24(r)
    with vlib.SSIMU2Handler(120, 200) as hd:
        assert hd.compute(a, a) == 100.0


def test_config1_256_rgb24(vlib, orc):
    r, d = synth.rgb24_pair(256, 256, seed=1)
    a, b = u16_planes_from_rgb24(r), u16_planes_from_rgb24(d)
    with vlib.SSIMU2Handler(256, 256) as hd:
        got = hd.compute(a, b)
    assert abs(got - orc.ssimu2(a, b, precision=64)) < TOL


def test_uint16_and_float_inputs_agree(vlib):
    r, d = synth.rgb24_pair(96, 160, seed=2)
    a16, b16 = u16_planes_from_rgb24(r), u16_planes_from_rgb24(d)
    af = [(p.astype(np.float32) / np.float32(65535.0)) for p in a16]
    bf = [(p.astype(np.float32) / np.float32(65535.0)) for p in b16]
    with vlib.SSIMU2Handler(160, 96) as hd:
        assert hd.compute(a16, b16) == hd.compute(af, bf)


@pytest.mark.parametrize("h,w", [(1, 1), (2, 3), (9, 17), (65, 33), (37, 100), (129, 257), (300, 211)])
def test_odd_sizes(vlib, orc, h, w):
    a, b = grating_float_pair(h, w, t=1)
    with vlib.SSIMU2Handler(w, h) as hd:
        got = hd.compute(a, b)
    o64 = orc.ssimu2(a, b, precision=64)
    o32 = orc.ssimu2(a, b, precision=32)
    assert abs(got - o64) <= max(TOL, 2.0 * abs(o32 - o64)), (got, o32, o64)


def test_stride_padding_is_ignored(vlib):
    a, b = grating_float_pair(70, 90, t=3)
    with vlib.SSIMU2Handler(90, 70) as hd:
        s0 = hd.compute(a, b)
        s1 = hd.compute(padded(a, 40, 0xFF), padded(b, 4, 0xFF))
    assert s0 == s1


def test_v2_separate_strides(vlib):
    a, b = grating_float_pair(64, 64, t=2)
    pa, pb = padded(a, 256, 0x55), padded(b, 12, 0xFF)
    L = vlib.lib()
    hd = vlib.SSIMU2Handler(64, 64)
    a1 = (ctypes.c_void_p * 3)(*[p.ctypes.data for p in pa])
    a2 = (ctypes.c_void_p * 3)(*[p.ctypes.data for p in pb])
    out = ctypes.c_double()
    rc = L.Vship_ComputeSSIMU2Floatv2(hd._h, ctypes.byref(out), ctypes.cast(a1, vlib._PP),
                                      ctypes.cast(a2, vlib._PP), pa[0].strides[0], pb[0].strides[0])
    assert rc == 0
    assert out.value == hd.compute(a, b)
    hd.free()


def test_1080p_yuv_pair(vlib, orc):
    a, b = grating_float_pair(1080, 1920, t=5)
    with vlib.SSIMU2Handler(1920, 1080) as hd:
        got = hd.compute(a, b)
    assert abs(got - orc.ssimu2(a, b, precision=64)) < TOL


def test_batch_device_api_matches_handler(vlib):
    import torch
    pairs = [grating_float_pair(90, 130, t=t) for t in range(5)]
    with vlib.SSIMU2Handler(130, 90) as hd:
        want = [hd.compute(a, b) for a, b in pairs]
    dev = [(torch.from_numpy(np.stack(a)).cuda(), torch.from_numpy(np.stack(b)).cuda()) for a, b in pairs]
    frames = []
    for ta, tb in dev:
        for t in (ta, tb):
            frames.append(([t[c].data_ptr() for c in range(3)], t.stride(1) * 4))
    table = vlib.device_frames_table(frames)
    scores = torch.zeros(len(pairs), dtype=torch.float64, device="cuda")
    bt = vlib.SSIMU2Batch(130, 90, 8)
    stream = torch.cuda.current_stream()
    bt.compute_async(table.data_ptr(), len(pairs), vlib.IN_FLOAT, scores.data_ptr(), stream.cuda_stream)
    torch.cuda.synchronize()
    assert scores.cpu().tolist() == want
    bt.free()


def test_concurrent_handlers(vlib):
    pairs = [grating_float_pair(120, 160, t=t) for t in range(6)]
    with vlib.SSIMU2Handler(160, 120) as hd:
        want = [hd.compute(a, b) for a, b in pairs]
    got = [None] * len(pairs)

    def worker(k):
        with vlib.SSIMU2Handler(160, 120) as h2:
            for i in range(k, len(pairs), 3):
                got[i] = h2.compute(*pairs[i])

    th = [threading.Thread(target=worker, args=(k,)) for k in range(3)]
    [t.start() for t in th]
    [t.join() for t in th]
    assert got == want


def test_handler_ids_are_reused(vlib):
    L = vlib.lib()
    h1 = vlib.Handler()
    assert L.Vship_SSIMU2Init(ctypes.byref(h1), 32, 32) == 0
    first = h1.id
    assert L.Vship_SSIMU2Free(h1) == 0
    h2 = vlib.Handler()
    assert L.Vship_SSIMU2Init(ctypes.byref(h2), 48, 40) == 0
    assert h2.id == first
    assert L.Vship_SSIMU2Free(h2) == 0
    assert L.Vship_SSIMU2Free(h2) == vlib.BadHandler


def test_device_queries(vlib):
    assert vlib.device_count() >= 1
    info = vlib.device_info(0)
    assert info["MultiProcessorCount"] > 0 and info["WarpSize"] == 32
    vlib.gpu_full_check(0)
    L = vlib.lib()
    assert L.Vship_GPUFullCheck(10 ** 6) == vlib.BadDeviceArgument
    assert L.Vship_SetDevice(-1) == vlib.BadDeviceArgument
