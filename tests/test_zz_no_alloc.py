"""The SSIMU2 entry point that allocates nothing (Vship_ComputeSSIMU2DeviceNoAlloc).

It exists for callers that may not allocate GPU memory while they run -- programs whose GPU
memory plan is fixed at start-up and plugins inside frameworks that own the device memory. Its
scratch is a fixed 32 MiB array in the library's device code. These tests call it through the
C ABI and check it against the batched device entry point (Vship_SSIMU2ComputeDeviceAsync) on
the same frames -- the same kernels on the same data, so the scores must be equal bit for bit --
and against the FP64 oracle within the SSIMU2 tolerance, with two calls in a row sharing the
array; after a first call, further calls must leave the device's free memory unchanged. The file
is collected last so a failure here never hides another test's result, and it sets everything
up itself so it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

from helpers import grating_float_pair

pytestmark = pytest.mark.gpu

TOL = 1e-3  # the SSIMU2 parity tolerance used by the other GPU tests


def _device_frame(vlib, t):
    f = vlib.DeviceFrame()
    for c in range(3):
        f.plane[c] = t[c].data_ptr()
    f.stride = t.stride(1) * t.element_size()
    return f


def _no_alloc(vlib, ta, tb, w, h, out_ptr, stream):
    fa, fb = _device_frame(vlib, ta), _device_frame(vlib, tb)
    return vlib.lib().Vship_ComputeSSIMU2DeviceNoAlloc(ctypes.byref(fa), ctypes.byref(fb), w, h, vlib.IN_FLOAT,
                                                       ctypes.c_void_p(out_ptr), ctypes.c_void_p(stream))


@pytest.mark.parametrize("h,w", [(270, 480), (720, 1280)])
def test_no_alloc_matches_device_entry_point_and_oracle(vlib, orc, h, w):
    import torch
    pairs = [grating_float_pair(h, w, t=t) for t in (1, 2)]
    dev = [(torch.from_numpy(np.stack(a)).cuda(), torch.from_numpy(np.stack(b)).cuda()) for a, b in pairs]
    stream = torch.cuda.current_stream()

    # the existing device entry point, both pairs in one batch
    frames = []
    for ta, tb in dev:
        for t in (ta, tb):
            frames.append(([t[c].data_ptr() for c in range(3)], t.stride(1) * 4))
    table = vlib.device_frames_table(frames)
    want = torch.zeros(2, dtype=torch.float64, device="cuda")
    bt = vlib.SSIMU2Batch(w, h, 2)
    bt.compute_async(table.data_ptr(), 2, vlib.IN_FLOAT, want.data_ptr(), stream.cuda_stream)

    # the no-allocation entry point: two calls in a row on one stream, sharing its scratch
    got = torch.full((2,), -1.0, dtype=torch.float64, device="cuda")
    for i, (ta, tb) in enumerate(dev):
        rc = _no_alloc(vlib, ta, tb, w, h, got.data_ptr() + 8 * i, stream.cuda_stream)
        assert rc == vlib.NoError, vlib.error_message(rc)
    torch.cuda.synchronize()
    bt.free()
    w_, g_ = want.cpu().tolist(), got.cpu().tolist()
    assert w_[0] != w_[1]
    assert g_ == w_, (g_, w_)
    for (a, b), g in zip(pairs, g_):
        fp64 = orc.ssimu2(a, b, precision=64)
        assert abs(g - fp64) <= TOL, (g, fp64)


def test_no_alloc_calls_leave_free_memory_unchanged(vlib):
    import torch
    w, h = 640, 360
    a, b = grating_float_pair(h, w, t=3)
    ta, tb = torch.from_numpy(np.stack(a)).cuda(), torch.from_numpy(np.stack(b)).cuda()
    out = torch.zeros(8, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    assert _no_alloc(vlib, ta, tb, w, h, out.data_ptr(), stream) == vlib.NoError  # commits the array
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for i in range(1, 8):
        assert _no_alloc(vlib, ta, tb, w, h, out.data_ptr() + 8 * i, stream) == vlib.NoError
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    vals = out.cpu().tolist()
    assert len(set(vals)) == 1 and 0.0 < vals[0] < 100.0


def test_no_alloc_refuses_frames_beyond_its_scratch(vlib):
    import torch
    L = vlib.lib()
    w, h = 1920, 1080
    t = torch.zeros((3, h, w), dtype=torch.float32, device="cuda")
    f = _device_frame(vlib, t)
    out = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    rc = L.Vship_ComputeSSIMU2DeviceNoAlloc(ctypes.byref(f), ctypes.byref(f), w, h, vlib.IN_FLOAT,
                                            ctypes.c_void_p(out.data_ptr()), None)
    assert rc == vlib.OutOfVRAM
    torch.cuda.synchronize()
    assert out.item() == -1.0
