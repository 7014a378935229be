"""Butteraugli parity: libvship.so through the C ABI against the CPU oracle. Tolerances: norms
within 1e-4 relative of the FP64 oracle; distortion map within 1e-3 of the map's maximum per
pixel (FP32 storage and evaluation order differ from the oracle's)."""
import ctypes

import numpy as np
import pytest

from helpers import grating_float_pair, padded, u16_planes_from_rgb24
from vship_gb300 import synth

pytestmark = pytest.mark.gpu

RTOL = 1e-4


def close_norms(got, want, rtol=RTOL):
    return all(abs(g - w) <= rtol * max(abs(w), 1e-6) for g, w in zip(got, want))


def test_kat_reference_size_identical_is_zero(vlib):
    # test/basic_metric_math_test.cpp:43-74: 1076x2400 float frames, stride 10000, 0xFF padding
    w, h, stride = 1076, 2400, 10000
    z = [np.zeros((h, w), np.float32) for _ in range(3)]
    a = padded(z, stride - 4 * w, 0x00)
    b = padded(z, stride - 4 * w, 0xFF)
    with vlib.ButteraugliHandler(w, h, 2, 203.0) as hd:
        norms, dm = hd.compute(a, b, distmap=True)
    assert norms == (0.0, 0.0, 0.0)
    assert not dm.any()


@pytest.mark.parametrize("distortion", ["blur_noise", "dct"])
def test_parity_480x270(vlib, orc, distortion):
    a, b = grating_float_pair(270, 480, t=2, distortion=distortion)
    with vlib.ButteraugliHandler(480, 270) as hd:
        got, dm = hd.compute(a, b, distmap=True)
    want, wdm = orc.butteraugli(a, b, precision=64, distmap=True)
    assert close_norms(got, want), (got, want)
    assert np.max(np.abs(dm - wdm)) <= 1e-3 * float(wdm.max())


@pytest.mark.parametrize("qnorm,intensity", [(1, 203.0), (3, 80.0), (5, 203.0), (6, 250.0)])
def test_qnorm_and_intensity(vlib, orc, qnorm, intensity):
    r, d = synth.rgb24_pair(72, 88, seed=6)
    a, b = u16_planes_from_rgb24(r), u16_planes_from_rgb24(d)
    with vlib.ButteraugliHandler(88, 72, qnorm, intensity) as hd:
        got = hd.compute(a, b)
    want = orc.butteraugli(a, b, qnorm=qnorm, intensity=intensity, precision=64)
    assert close_norms(got, want), (got, want)


@pytest.mark.parametrize("h,w", [(1, 1), (3, 2), (9, 17), (65, 33), (37, 100), (131, 257)])
def test_odd_sizes(vlib, orc, h, w):
    a, b = grating_float_pair(h, w, t=1, distortion="blur_noise")
    with vlib.ButteraugliHandler(w, h) as hd:
        got, dm = hd.compute(a, b, distmap=True)
    want, wdm = orc.butteraugli(a, b, precision=64, distmap=True)
    assert close_norms(got, want, 2e-4), (got, want)
    assert np.max(np.abs(dm - wdm)) <= 1e-3 * max(float(wdm.max()), 1e-6)


def test_int_score_struct_truncates(vlib):
    a, b = grating_float_pair(64, 96, t=4, distortion="blur_noise")
    hd = vlib.ButteraugliHandler(96, 64)
    exact = hd.compute(a, b)
    L = vlib.lib()
    a1 = (ctypes.c_void_p * 3)(*[p.ctypes.data for p in a])
    a2 = (ctypes.c_void_p * 3)(*[p.ctypes.data for p in b])
    sc = vlib.ButteraugliScore()
    assert L.Vship_ComputeButteraugliFloat(hd._h, ctypes.byref(sc), None, 0, ctypes.cast(a1, vlib._PP),
                                           ctypes.cast(a2, vlib._PP), a[0].strides[0]) == 0
    assert (sc.norm2, sc.norm3, sc.norminf) == tuple(int(np.float32(x)) for x in exact)
    hd.free()


def test_distmap_stride(vlib):
    a, b = grating_float_pair(50, 70, t=2, distortion="blur_noise")
    hd = vlib.ButteraugliHandler(70, 50)
    _, dm = hd.compute(a, b, distmap=True)
    L = vlib.lib()
    stride = 70 * 4 + 100
    out = np.full((50, stride), 0xEE, np.uint8)
    a1 = (ctypes.c_void_p * 3)(*[p.ctypes.data for p in a])
    a2 = (ctypes.c_void_p * 3)(*[p.ctypes.data for p in b])
    norms = (ctypes.c_double * 3)()
    assert L.Vship_ComputeButteraugliFloatv3(hd._h, norms, out.ctypes.data, stride, ctypes.cast(a1, vlib._PP),
                                             ctypes.cast(a2, vlib._PP), a[0].strides[0], b[0].strides[0]) == 0
    assert np.array_equal(out[:, : 70 * 4].view(np.float32), dm)
    assert (out[:, 70 * 4:] == 0xEE).all()
    # a distmap stride shorter than a row is refused before any work, and leaves the buffer and
    # the handler as they were
    out[:] = 0xEE
    assert L.Vship_ComputeButteraugliFloatv3(hd._h, norms, out.ctypes.data, 70 * 4 - 4, ctypes.cast(a1, vlib._PP),
                                             ctypes.cast(a2, vlib._PP), a[0].strides[0],
                                             b[0].strides[0]) == vlib.BadPointer
    assert (out == 0xEE).all()
    assert L.Vship_ComputeButteraugliFloatv3(hd._h, norms, out.ctypes.data, stride, ctypes.cast(a1, vlib._PP),
                                             ctypes.cast(a2, vlib._PP), a[0].strides[0], b[0].strides[0]) == 0
    assert np.array_equal(out[:, : 70 * 4].view(np.float32), dm)
    hd.free()


def test_4k_pair(vlib, orc):
    a, b = grating_float_pair(2160, 3840, t=0, distortion="blur_noise")
    with vlib.ButteraugliHandler(3840, 2160) as hd:
        got = hd.compute(a, b)
    want = orc.butteraugli(a, b, precision=64)
    assert close_norms(got, want), (got, want)


def test_threads_on_own_and_shared_handlers(vlib):
    """test/apibenchmark.cpp:132-157 drives Butteraugli from 3 threads that share one handler
    (which the reference's API does not allow); here threads on their own handlers and threads
    sharing one (calls on one handler are serialised) give the single-thread results."""
    import threading
    pairs = [grating_float_pair(96, 128, t=t, distortion="blur_noise") for t in range(6)]
    with vlib.ButteraugliHandler(128, 96, 2, 80.0) as hd:
        want = [hd.compute(a, b) for a, b in pairs]
    for shared in (False, True):
        got = [None] * len(pairs)
        common = vlib.ButteraugliHandler(128, 96, 2, 80.0) if shared else None

        def worker(k):
            h = common or vlib.ButteraugliHandler(128, 96, 2, 80.0)
            for i in range(k, len(pairs), 3):
                got[i] = h.compute(*pairs[i])
            if not shared:
                h.free()

        th = [threading.Thread(target=worker, args=(k,)) for k in range(3)]
        [t.start() for t in th]
        [t.join() for t in th]
        if common:
            common.free()
        assert got == want, shared


def test_init_rejects_bad_sizes(vlib):
    L = vlib.lib()
    import ctypes
    h = vlib.Handler()
    for w, hh in [(0, 10), (10, 0), (-4, 8)]:
        assert L.Vship_ButteraugliInitv2(ctypes.byref(h), w, hh, 2, ctypes.c_float(203.0)) == vlib.BadPointer
        assert L.Vship_SSIMU2Init(ctypes.byref(h), w, hh) == vlib.BadPointer


def test_near_identical_frames_stay_finite(vlib, orc):
    # differences of one float ulp around mid-grey: the band differences and the arguments of the
    # diff kernel's square roots get tiny; the norms must stay finite and match the oracle
    rs = np.random.default_rng(5)
    a = [np.full((96, 128), 0.5, np.float32) + rs.uniform(-0.1, 0.1, (96, 128)).astype(np.float32)
         for _ in range(3)]
    b = [np.nextafter(p, np.float32(2.0)) if c == 1 else p.copy() for c, p in enumerate(a)]
    with vlib.ButteraugliHandler(128, 96) as hd:
        got, dm = hd.compute(a, b, distmap=True)
    assert all(np.isfinite(x) for x in got) and np.isfinite(dm).all()
    # the norms are ~1e-5 here, where FP32 rounding alone (the FP32 oracle) moves them 2-6x: an
    # absolute bound, far below any visible distortion
    want = orc.butteraugli(a, b, precision=64)
    assert all(abs(g - w) <= 1e-4 for g, w in zip(got, want)), (got, want)
