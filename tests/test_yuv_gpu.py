"""GPU YUV 4:2:0 10-bit front-end: scores from Y'CbCr input (converted on the GPU) against
scores from the R'G'B' planes of the spec converter (vship_gb300.synth.yuv420p10_to_rgb), which is
what a reference front-end feeds the reference ABI.

The GPU conversion differs from the FP64 spec by at most one float ulp per sample; on large frames
the two input paths then agree within 1e-4. On small frames whose pairs are mostly identical
pixels, SSIMU2 in FP32 is dominated by sample quantisation (the reference's own FP32 formulation
moves by up to 5e-3 under one-ulp input changes at 64x65, the FP64 oracle by 1e-6), so there
each path is held to the parity tolerance against the FP64 oracle instead."""
import numpy as np
import pytest
import torch

from helpers import float_planes
from vship_gb300 import synth

pytestmark = pytest.mark.gpu


def yuv_pair(h, w, t, distortion="dct"):
    ref, dist = synth.yuv420p10_frames(h, w, t, seed=5, distortion=distortion)
    to16 = lambda f: [np.ascontiguousarray(p.numpy().astype(np.uint16)) for p in f]
    return (to16(ref), to16(dist)), (float_planes(synth.yuv420p10_to_rgb(ref)),
                                     float_planes(synth.yuv420p10_to_rgb(dist)))


@pytest.mark.parametrize("h,w", [(270, 480), (37, 101), (64, 65), (1080, 1920)])
def test_ssimu2_yuv_matches_rgb(vlib, orc, h, w):
    (ya, yb), (ra, rb) = yuv_pair(h, w, 3)
    with vlib.SSIMU2Handler(w, h) as hd:
        s_yuv = hd.compute_yuv420p10(ya, yb)
        s_rgb = hd.compute(ra, rb)
    if min(h, w) >= 256:
        assert abs(s_yuv - s_rgb) < 1e-4, (s_yuv, s_rgb)
    if h * w <= 300000:
        o64 = orc.ssimu2(ra, rb, precision=64)
        assert abs(s_yuv - o64) < 1e-3 and abs(s_rgb - o64) < 1e-3, (s_yuv, s_rgb, o64)


@pytest.mark.parametrize("h,w", [(270, 480), (37, 101)])
def test_butteraugli_yuv_matches_rgb(vlib, h, w):
    (ya, yb), (ra, rb) = yuv_pair(h, w, 2, "blur_noise")
    with vlib.ButteraugliHandler(w, h) as hd:
        n_yuv, d_yuv = hd.compute_yuv420p10(ya, yb, distmap=True)
        n_rgb, d_rgb = hd.compute(ra, rb, distmap=True)
    for a, b in zip(n_yuv, n_rgb):
        assert abs(a - b) <= 1e-5 * abs(b), (n_yuv, n_rgb)
    assert np.max(np.abs(d_yuv - d_rgb)) <= 1e-4 * float(d_rgb.max())


def test_yuv_padded_strides(vlib):
    (ya, yb), _ = yuv_pair(96, 130, 1)
    with vlib.SSIMU2Handler(130, 96) as hd:
        s0 = hd.compute_yuv420p10(ya, yb)
        pad = lambda p, k: np.pad(p, ((0, 0), (0, k)), constant_values=0xFFFF)[:, : p.shape[1]]
        s1 = hd.compute_yuv420p10([pad(p, 7) for p in ya], [pad(p, 3) for p in yb])
    assert s0 == s1


def test_device_async_yuv_matches_host(vlib):
    pairs = [yuv_pair(120, 200, t)[0] for t in range(3)]
    with vlib.SSIMU2Handler(200, 120) as hd:
        want = [hd.compute_yuv420p10(a, b) for a, b in pairs]
    keep, frames = [], []
    for a, b in pairs:
        for f in (a, b):
            t = [torch.from_numpy(p.astype(np.int32)).to(torch.int16).cuda() for p in f]
            keep.append(t)
            frames.append(([x.data_ptr() for x in t], t[0].stride(0) * 2, t[1].stride(0) * 2))
    table = vlib.device_frames_table(frames)
    out = torch.zeros(3, dtype=torch.float64, device="cuda")
    bt = vlib.SSIMU2Batch(200, 120, 4)
    bt.compute_async(table.data_ptr(), 3, vlib.IN_YUV420P10, out.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert out.cpu().tolist() == want
    bt.free()
