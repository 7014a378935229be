"""Butteraugli with FP16 band storage (Vship_ButterHalfBands, Vship_MultiButterHalfBands,
Vship_ServeButterHalfBands): the UHF bands (X, Y) kept as FP16, everything else FP32.

* Against the oracle with the same bands rounded to FP16 (precision 19) and against the FP64
  oracle: all three norms within the path's 1e-4 relative. The oracle puts this form's largest
  error over the frames evaluated (480x270 to 3840x2160, block-DCT and blur + noise) at 5.2e-5 on
  the inf-norm and 5.3e-6 on the Qnorm. FP16 storage of the HF or MF bands as well would not hold
  1e-4: HF alone reaches 1.0e-3 on the inf-norm, MF alone 1.3e-4 on the Qnorm, all three 2.5e-4 /
  4.5e-4 (the block-DCT frame t=5 here).
* Device bytes: each image takes 15 instead of 16 planes per scale.
* The batched, multi-resolution and serving forms give the same norms, bit for bit.
"""
import time

import numpy as np
import pytest
import torch

from helpers import grating_float_pair
from vship_gb300 import synth

pytestmark = pytest.mark.gpu

RTOL = 1e-4


def close(got, want):
    return all(abs(g - w) <= RTOL * max(abs(w), 1e-6) for g, w in zip(got, want))


@pytest.mark.parametrize("distortion,t", [("blur_noise", 2), ("dct", 2), ("dct", 5)])
@pytest.mark.parametrize("h,w", [(270, 480), (131, 257)])
def test_half_bands_parity(vlib, orc, distortion, t, h, w):
    a, b = grating_float_pair(h, w, t=t, distortion=distortion)
    with vlib.ButteraugliHandler(w, h, half_bands=True) as hd:
        got = hd.compute(a, b)
    model = orc.butteraugli(a, b, precision=19)
    exact = orc.butteraugli(a, b, precision=64)
    assert close(got, model), (got, model)
    assert close(got, exact), (got, exact)


def test_half_bands_device_bytes(vlib):
    w, h = 1920, 1080
    lib = vlib.lib()
    full = lib.Vship_ButteraugliDeviceBytes(w, h, 4)
    assert lib.Vship_ButteraugliDeviceBytesEx(w, h, 4, 0) == full
    half = lib.Vship_ButteraugliDeviceBytesEx(w, h, 4, vlib.BUTTER_HALF_BANDS)
    # per scale n = round_up(round_up(w, 8) * h, 64) floats per plane; two FP16 planes take one
    saved = 0
    cw, ch = w, h
    for _ in range(2):
        n = -(-(-(-cw // 8) * 8 * ch) // 64) * 64
        saved += n
        cw, ch = (cw + 1) // 2, (ch + 1) // 2
    assert full - half == 4 * 2 * 4 * saved  # 4 pairs x 2 images x 4 bytes


def test_half_bands_rejects_unknown_flags(vlib):
    h = vlib.Handler()
    rc = vlib.lib().Vship_ButteraugliBatchInitEx(vlib.ctypes.byref(h), 64, 64, 2, vlib.ctypes.c_float(203.0), 1, 2)
    assert rc == vlib.BadPointer


def _dev_yuv(frame, keep):
    t = [torch.from_numpy(np.asarray(p, dtype=np.int32)).to(torch.int16).cuda() for p in frame]
    keep.append(t)
    return ([x.data_ptr() for x in t], t[0].stride(0) * 2, t[1].stride(0) * 2)


def _pairs(w, h, keep, n=3):
    src = synth.yuv420p10_source(h, w, 0, 23)
    s = _dev_yuv(src, keep)
    cands = []
    for st in (4, 12, 26)[:n]:
        c = (synth.block_dct_quantise(src[0], st, 64, 940), synth.block_dct_quantise(src[1], 2 * st, 64, 960),
             synth.block_dct_quantise(src[2], 2 * st, 64, 960))
        cands.append(_dev_yuv(c, keep))
    return s, cands


def _batch_norms(vlib, w, h, src, cand):
    table = vlib.device_frames_table([src, cand])
    o = torch.zeros(3, dtype=torch.float64, device="cuda")
    bt = vlib.ButteraugliBatch(w, h, 1, half_bands=True)
    bt.compute_async(table.data_ptr(), 1, vlib.IN_YUV420P10, o.data_ptr(), 0, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    bt.free()
    return o.cpu().tolist()


def test_half_bands_multi_and_serve_match_batch(vlib):
    w, h = 200, 120
    keep = []
    src, cands = _pairs(w, h, keep)
    want = [_batch_norms(vlib, w, h, src, c) for c in cands]
    # batched multi-resolution form: the source's own stage once, its candidates against it
    sc = vlib.MultiScorer([(w, h)], [1], [len(cands)], vlib.MULTI_BUTTERAUGLI | vlib.MULTI_BUTTER_HALF)
    bn = torch.zeros(3 * len(cands), dtype=torch.float64, device="cuda")
    sc.compute_async([src], [0], cands, [0] * len(cands), vlib.IN_YUV420P10, 0, bn.data_ptr(),
                     torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    sc.free()
    assert bn.view(-1, 3).cpu().tolist() == want
    # serving runtime, the source cached between two requests
    srv = vlib.Server([(w, h)], vlib.IN_YUV420P10, flags=vlib.SERVE_BUTTER_HALF_BANDS)
    outs = [np.zeros(3 * 2), np.zeros(3)]
    srv.submit(1, vlib.SERVE_BUTTERAUGLI, 0, 77, src, cands[:2], outs[0])
    srv.submit(2, vlib.SERVE_BUTTERAUGLI, 0, 77, src, cands[2:], outs[1])
    done = {}
    t0 = time.time()
    while len(done) < 2 and time.time() - t0 < 60:
        for rid, status, _ in srv.poll(8, 5.0):
            done[rid] = status
    srv.free()
    assert done == {1: 0, 2: 0}
    assert outs[0].reshape(-1, 3).tolist() == want[:2]
    assert outs[1].reshape(-1, 3).tolist() == want[2:]
