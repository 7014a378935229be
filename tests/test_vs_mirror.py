"""vship_gb300.vs: the VapourSynth functions' semantics (arguments, defaults, frame properties,
distmap clip, errors) on array clips."""
import numpy as np
import pytest

from helpers import grating_float_pair
from vship_gb300 import synth, vs


def _clip_pair(n=3, h=64, w=96):
    refs, dists = [], []
    for t in range(n):
        a, b = grating_float_pair(h, w, t=t)
        refs.append(a)
        dists.append(b)
    return vs.Clip(refs), vs.Clip(dists)


def test_clip_formats():
    r, d = _clip_pair(1)
    assert r.format == "RGBS" and r.size == (96, 64)
    y, _ = synth.yuv420p10_frames(16, 20, 0)
    assert vs.Clip([[np.asarray(p, np.uint16) for p in y]]).format == "YUV420P10"
    assert vs.Clip([np.zeros((4, 5), np.float32)]).format == "GRAYS"


def test_errors_without_gpu_are_vship_exceptions():
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("GPU present")
    except ImportError:
        pass
    r, d = _clip_pair(1)
    with pytest.raises(vs.Error) as e:
        vs.SSIMULACRA2(r, d)
    assert str(e.value).startswith("VshipException\n")


def test_differing_inputs_rejected_before_any_gpu_work():
    r, _ = _clip_pair(2, 64, 96)
    _, d = _clip_pair(2, 64, 80)
    with pytest.raises(vs.Error) as e:
        vs.SSIMULACRA2(r, d)
    assert "DifferingInputType" in str(e.value)
    with pytest.raises(vs.Error):
        vs.BUTTERAUGLI(r, vs.Clip(d.frames[:1]))


@pytest.mark.gpu
def test_ssimulacra2_props(vlib):
    r, d = _clip_pair(4)
    out1 = vs.SSIMULACRA2(r, d, numStream=1)
    out3 = vs.SSIMULACRA2(r, d, numStream=3)
    with vlib.SSIMU2Handler(96, 64) as hd:
        want = [hd.compute(a, b) for a, b in zip(r.frames, d.frames)]
    assert [p["_SSIMULACRA2"] for p in out1.props] == want
    assert [p["_SSIMULACRA2"] for p in out3.props] == want
    assert out1.frames[0] is d.frames[0]


@pytest.mark.gpu
def test_butteraugli_props_and_distmap(vlib):
    r, d = _clip_pair(3)
    out = vs.BUTTERAUGLI(r, d, qnorm=2, intensity_multiplier=203.0)
    dm = vs.BUTTERAUGLI(r, d, distmap=1, numStream=2)
    with vlib.ButteraugliHandler(96, 64, 2, 203.0) as hd:
        for i in range(3):
            norms, m = hd.compute(r.frames[i], d.frames[i], distmap=True)
            p = out.props[i]
            assert (p["_BUTTERAUGLI_QNorm"], p["_BUTTERAUGLI_3Norm"], p["_BUTTERAUGLI_INFNorm"]) == norms
            assert p["_BUTTERAUGLI_2Norm"] == norms[0]
            assert dm.format == "GRAYS" and np.array_equal(dm.frames[i], m)


@pytest.mark.gpu
def test_yuv_clip(vlib):
    refs, dists = [], []
    for t in range(2):
        a, b = synth.yuv420p10_frames(48, 64, t, seed=3)
        refs.append([np.asarray(p, np.uint16) for p in a])
        dists.append([np.asarray(p, np.uint16) for p in b])
    out = vs.SSIMULACRA2(vs.Clip(refs), vs.Clip(dists), numStream=2)
    with vlib.SSIMU2Handler(64, 48) as hd:
        assert [p["_SSIMULACRA2"] for p in out.props] == [hd.compute_yuv420p10(a, b) for a, b in zip(refs, dists)]


@pytest.mark.gpu
def test_gpu_info(vlib):
    s = vs.GpuInfo()
    assert s.startswith("GPU 0: ")
    d = vs.GpuInfo(0)
    assert "MultiProcessorCount" in d and "PassKernelCheck : 1" in d
    with pytest.raises(vs.Error) as e:
        vs.GpuInfo(99)
    assert "BadDeviceArgument" in str(e.value)
