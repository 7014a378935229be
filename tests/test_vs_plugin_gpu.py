"""The VapourSynth filters of vship_gb300/csrc/vs_plugin.cpp, run end to end.

VapourSynth is not installed here, so tests/native/vs_harness.cpp stands in for its core: it
dlopens a plugin library built from vs_plugin.cpp (linked against libvship.so, exactly as the
shipped library carries the plugin when built with the VapourSynth SDK headers), calls
VapourSynthPluginInit2, invokes vship.SSIMULACRA2 / vship.BUTTERAUGLI / vship.GpuInfo with the
reference plugin's argument names (src/VshipLib.cpp:58-64), and pulls every frame through the
filter's getFrame (arInitial, then arAllFramesReady) from several threads at once with
numStream > 1. The frame properties (_SSIMULACRA2, _BUTTERAUGLI_QNorm / _2Norm / _3Norm /
_INFNorm; src/ssimu2/vapoursynth.hpp:59, src/butter/vapoursynth.hpp:71-73) and the distmap=1
GrayS clip must equal the C ABI's results on the same frames bit for bit: the filters call that
ABI.

The SDK headers come from $VAPOURSYNTH_INCLUDE, else from the reference's vendored copy staged
under oracle/_ref/src/include by oracle/ref_build.py.
"""
from __future__ import annotations

import json
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CANDIDATES = [os.environ.get("VAPOURSYNTH_INCLUDE"), os.path.join(ROOT, "oracle", "_ref", "src", "include")]
SDK = next((d for d in CANDIDATES if d and os.path.exists(os.path.join(d, "VapourSynth4.h"))), None)

pytestmark = pytest.mark.skipif(SDK is None, reason="no VapourSynth SDK headers")


def _build_harness(out_dir):
    exe = os.path.join(out_dir, "vs_harness")
    r = subprocess.run(["g++", "-O1", "-std=c++17", "-I" + SDK, os.path.join(ROOT, "tests", "native", "vs_harness.cpp"),
                        "-o", exe, "-ldl", "-lpthread"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def _build_plugin(out_dir):
    libdir = os.path.join(ROOT, "vship_gb300")
    so = os.path.join(out_dir, "vship_vs.so")
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-fvisibility=hidden", "-I" + SDK,
                        "-I" + os.path.join(ROOT, "include"), os.path.join(libdir, "csrc", "vs_plugin.cpp"),
                        "-L" + libdir, "-lvship", "-Wl,-rpath," + libdir, "-o", so], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return so


def test_harness_and_plugin_compile(tmp_path):
    # CPU: both sides of the harness build (the plugin only needs libvship.so to link against)
    _build_harness(str(tmp_path))
    if os.path.exists(os.path.join(ROOT, "vship_gb300", "libvship.so")):
        so = _build_plugin(str(tmp_path))
        syms = subprocess.run(["nm", "-D", "--defined-only", so], capture_output=True, text=True).stdout
        assert " T VapourSynthPluginInit2" in syms


@pytest.fixture(scope="module")
def harness(vlib, tmp_path_factory):
    d = str(tmp_path_factory.mktemp("vs"))
    return _build_harness(d), _build_plugin(d), d


def _frames(w, h, n):
    from vship_gb300 import synth
    out = []
    for t in range(n):
        r, d = synth.rgb_float_pair(h, w, t, seed=21, distortion="dct" if t % 2 else "blur_noise")
        out.append((r.numpy().astype(np.float32), d.numpy().astype(np.float32)))
    return out


def _write(path, frames):
    h, w = frames[0][0].shape[1:]
    with open(path, "wb") as f:
        f.write(np.array([w, h, len(frames)], np.int32).tobytes())
        for r, d in frames:
            f.write(np.ascontiguousarray(r).tobytes())
            f.write(np.ascontiguousarray(d).tobytes())


def _run(harness, frames_path, fn, threads, out_path, *args):
    exe, so, _ = harness
    r = subprocess.run([exe, so, frames_path, fn, str(threads), out_path, *args], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.strip()]
    return lines




@pytest.mark.gpu
def test_plugin_registers_reference_surface(harness):
    lines = _run(harness, "-", "GpuInfo", 1, "-")
    assert lines[0] == {"plugin": "com.lumen.vship", "namespace": "vship", "name": "VapourSynth GPU Perceptual Metrics"}
    fns = {x["function"]: x["args"] for x in lines if "function" in x}
    assert fns["SSIMULACRA2"] == "reference:vnode;distorted:vnode;numStream:int:opt;gpu_id:int:opt;"
    assert fns["BUTTERAUGLI"] == ("reference:vnode;distorted:vnode;qnorm:int:opt;intensity_multiplier:float:opt;"
                                  "distmap:int:opt;numStream:int:opt;gpu_id:int:opt;")
    assert fns["GpuInfo"] == "gpu_id:int:opt;"
    listing = lines[-1]["gpu_human_data"]
    assert listing.startswith("GPU 0: ")
    detail = _run(harness, "-", "GpuInfo", 1, "-", "gpu_id=0")[-1]["gpu_human_data"]
    assert "Name: " in detail and "MultiProcessorCount: " in detail and "PassKernelCheck : 1" in detail
    bad = _run(harness, "-", "GpuInfo", 1, "-", "gpu_id=99")[-1]
    assert bad["error"].startswith("VshipException\nBadDeviceArgument")


@pytest.mark.gpu
def test_ssimulacra2_filter_matches_c_abi(vlib, harness):
    w, h, n = 256, 192, 6
    frames = _frames(w, h, n)
    path = os.path.join(harness[2], "ssimu2.raw")
    _write(path, frames)
    lines = _run(harness, path, "SSIMULACRA2", 4, "-", "numStream=3")
    per_frame = {x["frame"]: x for x in lines if "frame" in x}
    assert len(per_frame) == n
    with vlib.SSIMU2Handler(w, h) as hd:
        for t, (r, d) in enumerate(frames):
            want = hd.compute(list(r), list(d))
            assert per_frame[t]["_SSIMULACRA2"] == want, (t, per_frame[t], want)


@pytest.mark.gpu
def test_butteraugli_filter_and_distmap_clip_match_c_abi(vlib, harness):
    w, h, n = 200, 136, 4
    frames = _frames(w, h, n)
    path = os.path.join(harness[2], "butter.raw")
    out = os.path.join(harness[2], "distmap.raw")
    _write(path, frames)
    lines = _run(harness, path, "BUTTERAUGLI", 3, out, "qnorm=3", "intensity_multiplier=80.0", "distmap=1",
                 "numStream=2")
    info = next(x["output"] for x in lines if "output" in x)
    assert info == {"width": w, "height": h, "frames": n, "color_family": 1, "bits": 32}  # cfGray, 32-bit float
    per_frame = {x["frame"]: x for x in lines if "frame" in x}
    maps = np.fromfile(out, np.float32).reshape(n, h, w)
    with vlib.ButteraugliHandler(w, h, 3, 80.0) as hd:
        for t, (r, d) in enumerate(frames):
            (q, n3, ninf), dm = hd.compute(list(r), list(d), distmap=True)
            p = per_frame[t]
            assert (p["_BUTTERAUGLI_QNorm"], p["_BUTTERAUGLI_3Norm"], p["_BUTTERAUGLI_INFNorm"]) == (q, n3, ninf)
            assert p["_BUTTERAUGLI_2Norm"] == q
            assert np.array_equal(maps[t], dm)


@pytest.mark.gpu
def test_butteraugli_filter_default_arguments(vlib, harness):
    # no qnorm / intensity / distmap / numStream: Qnorm 2, intensity 203, the distorted clip out
    w, h, n = 160, 96, 2
    frames = _frames(w, h, n)
    path = os.path.join(harness[2], "butter_default.raw")
    _write(path, frames)
    lines = _run(harness, path, "BUTTERAUGLI", 2, "-")
    info = next(x["output"] for x in lines if "output" in x)
    assert info["color_family"] == 2 and info["bits"] == 32  # cfRGB float: the distorted clip
    per_frame = {x["frame"]: x for x in lines if "frame" in x}
    with vlib.ButteraugliHandler(w, h, 2, 203.0) as hd:
        for t, (r, d) in enumerate(frames):
            q, n3, ninf = hd.compute(list(r), list(d))
            assert per_frame[t]["_BUTTERAUGLI_QNorm"] == q and per_frame[t]["_BUTTERAUGLI_INFNorm"] == ninf
