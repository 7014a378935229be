"""GPU Y'CbCr front-end over formats (depth 8-16, 4:2:0 / 4:2:2 / 4:4:4, matrices, ranges,
chroma sitings): scores from Y'CbCr planes converted on the GPU against scores from the R'G'B'
planes of the FP64 spec converter (vship_gb300.synth.yuv_to_rgb), which is what a CPU front-end
feeds the reference ABI. The two inputs differ by about one float ulp per sample, so scores
agree within 1e-4 (SSIMU2, absolute) and 1e-5 (Butteraugli, relative)."""
import numpy as np
import pytest
import torch

from helpers import float_planes
from vship_gb300 import synth

pytestmark = pytest.mark.gpu

# (bits, ssw, ssh, matrix, full range, chroma location, h, w)
FORMATS = [
    (8, 1, 1, 6, False, 1, 270, 480),    # 8-bit 4:2:0 BT.601, center siting (JPEG / MPEG-1)
    (10, 1, 0, 1, False, 0, 270, 480),   # 10-bit 4:2:2 BT.709
    (12, 0, 0, 9, True, 0, 256, 320),    # 12-bit 4:4:4 BT.2020 full range
    (16, 1, 1, 2, True, 2, 272, 336),    # 16-bit 4:2:0 full range, top-left, matrix by height (BT.470BG)
    (8, 1, 1, 7, False, 5, 257, 331),    # 8-bit 4:2:0 SMPTE 240M, bottom siting, odd sizes
    (10, 1, 1, 2, False, 4, 720, 1280),  # 10-bit 4:2:0 matrix by height (BT.709), bottom-left
]


def _pair(fmt, t, distortion):
    bits, ssw, ssh, matrix, full, loc, h, w = fmt
    ref, dist = synth.yuv_frames(h, w, t, bits, ssw, ssh, full, seed=3, distortion=distortion)
    dt = np.uint8 if bits == 8 else np.uint16
    host = lambda f: [np.ascontiguousarray(p.numpy().astype(dt)) for p in f]
    rgb = lambda f: float_planes(synth.yuv_to_rgb(f, bits, ssw, ssh, matrix, full, loc))
    return host(ref), host(dist), rgb(ref), rgb(dist)


def _fmt(vlib, fmt):
    bits, ssw, ssh, matrix, full, loc, h, w = fmt
    return vlib.yuv_format(bits, (ssw, ssh), matrix, full, loc)


@pytest.mark.parametrize("fmt", FORMATS, ids=lambda f: f"{f[0]}b-{f[1]}{f[2]}-m{f[3]}-{'full' if f[4] else 'lim'}-l{f[5]}")
def test_ssimu2_yuv_formats(vlib, fmt):
    ya, yb, ra, rb = _pair(fmt, 2, "dct")
    h, w = fmt[6], fmt[7]
    with vlib.SSIMU2Handler(w, h) as hd:
        hd.set_yuv_format(_fmt(vlib, fmt))
        s_yuv = hd.compute_yuv(ya, yb)
        s_rgb = hd.compute(ra, rb)
    assert abs(s_yuv - s_rgb) < 1e-4, (s_yuv, s_rgb)


@pytest.mark.parametrize("fmt", FORMATS[:4], ids=lambda f: f"{f[0]}b-{f[1]}{f[2]}-m{f[3]}")
def test_butteraugli_yuv_formats(vlib, fmt):
    ya, yb, ra, rb = _pair(fmt, 1, "blur_noise")
    h, w = fmt[6], fmt[7]
    with vlib.ButteraugliHandler(w, h) as hd:
        hd.set_yuv_format(_fmt(vlib, fmt))
        n_yuv = hd.compute_yuv(ya, yb)
        n_rgb = hd.compute(ra, rb)
    for a, b in zip(n_yuv, n_rgb):
        assert abs(a - b) <= 1e-5 * abs(b), (n_yuv, n_rgb)


# (bits, ssw, ssh, matrix, full, loc, h, w, transfer, primaries)
CONVERSIONS = [
    (10, 1, 1, 9, False, 2, 270, 480, 14, 9),  # BT.2020 SDR: BT.2020 matrix and primaries
    (8, 0, 0, 1, True, 0, 256, 320, 13, 1),    # sRGB transfer, full-range 4:4:4
    (12, 1, 0, 6, False, 0, 256, 256, 4, 9),   # gamma 2.2 with BT.2020 primaries
    (10, 1, 1, 1, False, 0, 144, 256, 8, 1),   # linear-light samples
]


@pytest.mark.parametrize("fmt", CONVERSIONS, ids=lambda f: f"trc{f[8]}-pri{f[9]}")
def test_transfer_and_primaries(vlib, fmt):
    """Frames in another transfer / primaries: the GPU takes them to linear BT.709 light and the
    metric skips its own linearisation; the reference path gets R'G'B' planes that linearise to
    the same light (2.4 power law of the FP64 conversion)."""
    bits, ssw, ssh, matrix, full, loc, h, w, trc, pri = fmt
    ref, dist = synth.yuv_frames(h, w, 2, bits, ssw, ssh, full, seed=4, distortion="dct")
    dt = np.uint8 if bits == 8 else np.uint16
    host = lambda f: [np.ascontiguousarray(p.numpy().astype(dt)) for p in f]
    rgb = lambda f: float_planes(synth.yuv_to_rgb(f, bits, ssw, ssh, matrix, full, loc, transfer=trc, primaries=pri))
    fm = vlib.yuv_format(bits, (ssw, ssh), matrix, full, loc, trc, pri)
    with vlib.SSIMU2Handler(w, h) as hd:
        hd.set_yuv_format(fm)
        s_yuv = hd.compute_yuv(host(ref), host(dist))
        s_rgb = hd.compute(rgb(ref), rgb(dist))
    assert abs(s_yuv - s_rgb) < 2e-4, (s_yuv, s_rgb)
    with vlib.ButteraugliHandler(w, h) as hd:
        hd.set_yuv_format(fm)
        n_yuv = hd.compute_yuv(host(ref), host(dist))
        n_rgb = hd.compute(rgb(ref), rgb(dist))
    for a, b in zip(n_yuv, n_rgb):
        assert abs(a - b) <= 2e-5 * abs(b), (n_yuv, n_rgb)


def test_default_format_unchanged(vlib):
    """A handler whose format was changed still scores the Yuv420p10 calls in 10-bit 4:2:0."""
    ref, dist = synth.yuv420p10_frames(96, 130, 1, seed=5)
    ya = [np.ascontiguousarray(p.numpy().astype(np.uint16)) for p in ref]
    yb = [np.ascontiguousarray(p.numpy().astype(np.uint16)) for p in dist]
    with vlib.SSIMU2Handler(130, 96) as hd:
        s0 = hd.compute_yuv420p10(ya, yb)
        hd.set_yuv_format(vlib.yuv_format(8, (0, 0), 6, True, 1))
        assert hd.compute_yuv420p10(ya, yb) == s0
        hd.set_yuv_format(vlib.yuv_format(10, (1, 1), 1, False, 0))
        assert hd.compute_yuv(ya, yb) == s0


def test_bad_formats_rejected(vlib):
    with vlib.SSIMU2Handler(64, 64) as hd:
        for f in [vlib.yuv_format(7), vlib.yuv_format(17), vlib.yuv_format(10, (2, 1)), vlib.yuv_format(10, matrix=3),
                  vlib.yuv_format(10, chroma_location=6), vlib.yuv_format(10, transfer=16),
                  vlib.yuv_format(10, primaries=12)]:
            with pytest.raises(vlib.VshipError):
                hd.set_yuv_format(f)


def test_device_batch_and_multi_formats(vlib):
    """4:2:2 8-bit frames through the device batch path and the batched multi form (source reuse)."""
    fmt = (8, 1, 0, 6, False, 0, 144, 256)
    bits, ssw, ssh, matrix, full, loc, h, w = fmt
    ref, dists = None, []
    for t in range(3):
        r, d = synth.yuv_frames(h, w, 0, bits, ssw, ssh, full, seed=9 + t)
        ref = ref or r
        dists.append(synth.yuv_frames(h, w, 0, bits, ssw, ssh, full, seed=9 + t)[1])
    keep = []

    def dev(f):
        t_ = [p.to(torch.uint8).cuda() for p in f]
        keep.append(t_)
        return ([x.data_ptr() for x in t_], t_[0].stride(0), t_[1].stride(0))

    src = dev(ref)
    cands = [dev(d) for d in dists]
    fm = _fmt(vlib, fmt)
    want = []
    with vlib.SSIMU2Handler(w, h) as hd:
        hd.set_yuv_format(fm)
        for d in dists:
            want.append(hd.compute_yuv([p.numpy().astype(np.uint8) for p in ref], [p.numpy().astype(np.uint8) for p in d]))
    bt = vlib.SSIMU2Batch(w, h, 3)
    bt.set_yuv_format(fm)
    table = vlib.device_frames_table([x for c in cands for x in (src, c)])
    out = torch.zeros(3, dtype=torch.float64, device="cuda")
    bt.compute_async(table.data_ptr(), 3, vlib.IN_YUV, out.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    bt.free()
    assert out.cpu().tolist() == want
    sc = vlib.MultiScorer([(w, h)], [1], [3], vlib.MULTI_SSIMU2)
    sc.set_yuv_format(fm)
    out.zero_()
    sc.compute_async([src], [0], cands, [0, 0, 0], vlib.IN_YUV, out.data_ptr(), 0,
                     torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    sc.free()
    assert out.cpu().tolist() == want
