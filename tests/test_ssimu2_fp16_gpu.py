"""SSIMULACRA2 with the distorted image's XYB pyramid stored as FP16 deltas (Vship_SSIMU2InitEx /
Vship_SSIMU2BatchInitEx with Vship_SSIMU2Fp16Deltas): the reference pyramid FP32, the distorted
one as half(distorted - reference), all arithmetic FP32.

* Against the FP64 oracle: within the SSIMULACRA2 tolerance, 1e-3 absolute, on frames of
  480x270 and up (at 1920x1080 the storage moves the score by about 1e-5). On a 93x67 frame with
  heavy blur and noise the bound is 2e-3: the oracle's own model of this storage is 1.42e-3 from
  FP64 there, because the coarsest scales hold a few pixels and large deltas keep only FP16's 11
  significant bits.
* Against the oracle's model of the same storage (precision 17: FP64 arithmetic over a reference
  pyramid in full precision and the distorted one as FP16 deltas): within 2e-4. The two round
  the same deltas; what is left is the FP32 evaluation order of the GPU.
* Identical frames give exactly 100: every delta is exactly zero.
* The per-pair and batched entry points give the same scores bit for bit, and the form holds
  3/4 of the FP32 form's pyramid bytes.
"""
import ctypes

import numpy as np
import pytest

from helpers import grating_float_pair, u16_planes_from_rgb24
from vship_gb300 import synth

pytestmark = pytest.mark.gpu

TOL = 1e-3
MODEL_TOL = 2e-4


@pytest.mark.parametrize("h,w,distortion,tol", [(270, 480, "dct", TOL), (270, 480, "blur_noise", TOL),
                                                (131, 257, "dct", TOL), (67, 93, "blur_noise", 2e-3)])
def test_fp16_deltas_against_oracle(vlib, orc, h, w, distortion, tol):
    a, b = grating_float_pair(h, w, t=3, distortion=distortion)
    with vlib.SSIMU2Handler(w, h, fp16_deltas=True) as hd:
        got = hd.compute(a, b)
    exact = orc.ssimu2(a, b, precision=64)
    model = orc.ssimu2(a, b, precision=17)
    assert abs(got - exact) <= tol, (got, exact)
    assert abs(got - model) <= MODEL_TOL, (got, model)


def test_fp16_deltas_1080p_pair(vlib, orc):
    r, d = synth.rgb_float_pair(1080, 1920, 5, seed=7, distortion="dct")
    a = [np.ascontiguousarray(p) for p in r.numpy()]
    b = [np.ascontiguousarray(p) for p in d.numpy()]
    with vlib.SSIMU2Handler(1920, 1080, fp16_deltas=True) as hd:
        got = hd.compute(a, b)
    with vlib.SSIMU2Handler(1920, 1080) as hd:
        fp32 = hd.compute(a, b)
    exact = orc.ssimu2(a, b, precision=64)
    assert abs(got - exact) <= TOL and abs(fp32 - exact) <= TOL, (got, fp32, exact)


def test_fp16_deltas_identical_frames_are_100(vlib):
    r, _ = synth.rgb24_pair(200, 120, seed=9)
    a = u16_planes_from_rgb24(r)
    with vlib.SSIMU2Handler(120, 200, fp16_deltas=True) as hd:
        assert hd.compute(a, a) == 100.0


def test_fp16_deltas_batched_matches_per_pair(vlib):
    import torch
    w, h = 320, 184
    pairs = [grating_float_pair(h, w, t=t, distortion="dct") for t in range(3)]
    want = []
    with vlib.SSIMU2Handler(w, h, fp16_deltas=True) as hd:
        for a, b in pairs:
            want.append(hd.compute(a, b))
    dev = [(torch.from_numpy(np.stack(a)).cuda(), torch.from_numpy(np.stack(b)).cuda()) for a, b in pairs]
    frames = []
    for ta, tb in dev:
        for t in (ta, tb):
            frames.append(([t[c].data_ptr() for c in range(3)], t.stride(1) * 4))
    table = vlib.device_frames_table(frames)
    out = torch.zeros(3, dtype=torch.float64, device="cuda")
    bt = vlib.SSIMU2Batch(w, h, 3, fp16_deltas=True)
    bt.compute_async(table.data_ptr(), 3, vlib.IN_FLOAT, out.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    bt.free()
    assert out.cpu().tolist() == want


def test_fp16_deltas_device_bytes_and_flags(vlib):
    lib = vlib.lib()
    w, h, n = 1920, 1080, 4
    fp32 = lib.Vship_SSIMU2DeviceBytes(w, h, n)
    assert lib.Vship_SSIMU2DeviceBytesEx(w, h, n, 0) == fp32
    fp16 = lib.Vship_SSIMU2DeviceBytesEx(w, h, n, vlib.SSIMU2_FP16_DELTAS)
    # one channel's pyramid: per level round_up(round_up(w, 8) * h, 64) elements; both images'
    # three channels take 8 bytes per element in FP32 and 6 with the distorted one in FP16
    pe, cw, ch = 0, w, h
    for _ in range(6):
        pe += -(-(-(-cw // 8) * 8 * ch) // 64) * 64
        cw, ch = (cw + 1) // 2, (ch + 1) // 2
    assert fp32 - fp16 == 2 * 3 * pe * n
    hd = vlib.Handler()
    assert lib.Vship_SSIMU2InitEx(ctypes.byref(hd), 64, 64, 2) == vlib.BadPointer
    assert lib.Vship_SSIMU2BatchInitEx(ctypes.byref(hd), 64, 64, 1, 4) == vlib.BadPointer
