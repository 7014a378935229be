"""Differential parity against the reference's own CUDA build.

Two sources of reference results:

* ``tests/golden/ref_golden.json`` / ``ref_golden_maps.npz``: scores, norms and distortion maps
  that the reference's CUDA build (pkp24/Vship src/VshipLib.cpp, built by oracle/ref_build.py)
  produced on a GB300 for stored inputs and for regenerated 1080p / 4K workload pairs
  (tests/golden/make_ref_golden.py). These tests need only libvship.so.
* the reference library itself (oracle/_ref/libvship_ref.so), when it has been built on this
  machine: the same inputs go through both libraries' C ABIs in one process.

Tolerances are the ones the path is specified to: SSIMU2 within 1e-3 absolute of the reference;
Butteraugli norms within 1e-4 relative; distortion maps within 1e-3 of the map's maximum per pixel.
Where the reference's own FP32 result is further than the tolerance from the FP64 oracle (SSIMU2
on frames of a few thousand pixels, whose coarsest scales hold a handful of pixels), libvship
must instead be within the tolerance of the FP64 oracle: there the reference's rounding error,
not a difference of method, is what separates the two.
"""
from __future__ import annotations

import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")
SSIMU2_TOL = 1e-3
NORM_RTOL = 1e-4
MAP_TOL = 1e-3


def _gold():
    p = os.path.join(GOLD, "ref_golden.json")
    if not os.path.exists(p):
        pytest.skip("no reference fixtures (tests/golden/make_ref_golden.py writes them)")
    return json.load(open(p))["cases"]


def _maps():
    return np.load(os.path.join(GOLD, "ref_golden_maps.npz"))


def _cases(metric, source=None):
    p = os.path.join(GOLD, "ref_golden.json")
    if not os.path.exists(p):
        return []
    return [c for c in json.load(open(p))["cases"]
            if c["metric"] == metric and (source is None or c["source"] in source)]


def _stored_frames(c):
    if c["source"] == "oracle_inputs.npz":
        d = np.load(os.path.join(GOLD, "oracle_inputs.npz"))
        return list(d[c["name"] + "_ref"]), list(d[c["name"] + "_dist"])
    d = np.load(os.path.join(GOLD, "ref_inputs.npz"))
    key = c.get("input_name", c["name"])
    f = lambda a: [np.ascontiguousarray(a[i].astype(np.uint16) * 257) for i in range(3)]
    return f(d[key + "_ref"]), f(d[key + "_dist"])


def _ssimu2_agrees(mine, ref, fp64):
    if abs(mine - ref) <= SSIMU2_TOL:
        return True
    return fp64 is not None and abs(ref - fp64) > SSIMU2_TOL and abs(mine - fp64) <= SSIMU2_TOL


def _norms_agree(mine, ref, rtol=NORM_RTOL):
    return all(abs(g - w) <= rtol * max(abs(w), 1e-6) for g, w in zip(mine, ref))


# ------------------------------------------------------------------------------------------
# against the committed reference fixtures

@pytest.mark.parametrize("case", _cases("ssimu2", ("oracle_inputs.npz", "ref_inputs.npz")), ids=lambda c: c["name"])
def test_ssimu2_stored_inputs_match_reference(vlib, orc, case):
    a, b = _stored_frames(case)
    with vlib.SSIMU2Handler(case["w"], case["h"]) as h:
        mine = h.compute(a, b)
    fp64 = orc.ssimu2(a, b, precision=64)
    assert _ssimu2_agrees(mine, case["score"], fp64), (mine, case["score"], fp64)


@pytest.mark.parametrize("case", _cases("butter", ("oracle_inputs.npz", "ref_inputs.npz")), ids=lambda c: c["name"])
def test_butteraugli_stored_inputs_match_reference(vlib, case):
    a, b = _stored_frames(case)
    with vlib.ButteraugliHandler(case["w"], case["h"], case["qnorm"], case["intensity"]) as h:
        mine, dm = h.compute(a, b, distmap=True)
    assert _norms_agree(mine, case["norms"]), (mine, case["norms"])
    ref_dm = _maps()[case["name"]]
    assert np.max(np.abs(dm - ref_dm)) <= MAP_TOL * max(float(ref_dm.max()), 1e-6)


def _regenerate(case):
    import sys
    sys.path.insert(0, GOLD)
    import make_ref_golden as mk
    spec = mk.SSIMU2_1080P if case["metric"] == "ssimu2" else mk.BUTTER_4K
    fr, fd, ysha, rsha = mk.large_pair(spec, case["t"])
    assert ysha == case["yuv_sha256"], "regenerated Y'CbCr planes differ from the ones the reference scored"
    return fr, fd, mk


def test_ssimu2_1080p_workload_pairs_match_reference(vlib):
    cases = _cases("ssimu2", ("synth",))
    if not cases:
        pytest.skip("no reference fixtures")
    with vlib.SSIMU2Handler(1920, 1080) as h:
        for c in cases:
            fr, fd, mk = _regenerate(c)
            got_f = h.compute(list(fr), list(fd))
            got_u = h.compute(list(mk.rgb48(fr)), list(mk.rgb48(fd)))
            assert abs(got_f - c["score_float"]) <= SSIMU2_TOL, (c["name"], got_f, c["score_float"])
            assert abs(got_u - c["score_rgb48"]) <= SSIMU2_TOL, (c["name"], got_u, c["score_rgb48"])


def test_butteraugli_4k_workload_pairs_match_reference(vlib):
    cases = _cases("butter", ("synth",))
    if not cases:
        pytest.skip("no reference fixtures")
    maps = _maps()
    with vlib.ButteraugliHandler(3840, 2160, 2, 203.0) as h:
        for c in cases:
            fr, fd, _ = _regenerate(c)
            mine, dm = h.compute(list(fr), list(fd), distmap=True)
            assert _norms_agree(mine, c["norms"]), (c["name"], mine, c["norms"])
            sub = dm[::c["distmap_sub"], ::c["distmap_sub"]]
            ref_sub = maps[c["name"] + "_sub"]
            assert np.max(np.abs(sub - ref_sub)) <= MAP_TOL * c["distmap_max"], c["name"]
            assert abs(float(dm.max()) - c["distmap_max"]) <= NORM_RTOL * c["distmap_max"]
            assert abs(float(dm.astype(np.float64).sum()) - c["distmap_sum"]) <= NORM_RTOL * c["distmap_sum"]


# ------------------------------------------------------------------------------------------
# against the reference library, live

@pytest.fixture(scope="module")
def refcuda():
    from oracle import ref_build, reference_cuda
    if not reference_cuda.available():
        if ref_build.staged():
            pytest.fail("reference sources are staged but oracle/_ref/libvship_ref.so was not built")
        pytest.skip("reference CUDA build not present on this machine")
    reference_cuda.lib()
    return reference_cuda


LIVE = [
    # (w, h, input, distortion, t)
    (256, 256, "float", "dct", 0),
    (640, 360, "uint16", "blur_noise", 1),
    (333, 187, "float", "blur_noise", 2),
    (1280, 720, "uint16", "dct", 3),
]


def _live_frames(w, h, kind, distortion, t):
    from vship_gb300 import synth
    r, d = synth.rgb_float_pair(h, w, t, seed=13, distortion=distortion)
    fr, fd = r.numpy(), d.numpy()
    if kind == "uint16":
        cv = lambda x: np.round(np.clip(x, 0, 1) * 65535.0).astype(np.uint16)
        fr, fd = cv(fr), cv(fd)
    return [np.ascontiguousarray(p) for p in fr], [np.ascontiguousarray(p) for p in fd]


@pytest.mark.parametrize("w,h,kind,distortion,t", LIVE)
def test_ssimu2_live_against_reference(vlib, orc, refcuda, w, h, kind, distortion, t):
    a, b = _live_frames(w, h, kind, distortion, t)
    with vlib.SSIMU2Handler(w, h) as hd:
        mine = hd.compute(a, b)
    with refcuda.SSIMU2(w, h) as hr:
        ref = hr.compute(a, b)
    fp64 = orc.ssimu2(a, b, precision=64) if w * h <= 400_000 else None
    assert _ssimu2_agrees(mine, ref, fp64), (mine, ref, fp64)


@pytest.mark.parametrize("w,h,kind,distortion,t", LIVE)
@pytest.mark.parametrize("qnorm,intensity", [(2, 203.0), (3, 80.0)])
def test_butteraugli_live_against_reference(vlib, refcuda, w, h, kind, distortion, t, qnorm, intensity):
    a, b = _live_frames(w, h, kind, distortion, t)
    with vlib.ButteraugliHandler(w, h, qnorm, intensity) as hd:
        mine, dm = hd.compute(a, b, distmap=True)
    with refcuda.Butteraugli(w, h, qnorm, intensity) as hr:
        ref, rdm = hr.compute(a, b, distmap=True)
    assert _norms_agree(mine, ref), (mine, ref)
    assert np.max(np.abs(dm - rdm)) <= MAP_TOL * max(float(rdm.max()), 1e-6)


def test_identical_frames_reference_and_ours(vlib, refcuda):
    # the reference's own known answer (test/basic_metric_math_test.cpp:40-79), through both builds
    w, h = 320, 192
    z = [np.zeros((h, w), np.float32) for _ in range(3)]
    with vlib.SSIMU2Handler(w, h) as hd, refcuda.SSIMU2(w, h) as hr:
        assert hd.compute(z, z) == hr.compute(z, z) == 100.0
    with vlib.ButteraugliHandler(w, h) as hd, refcuda.Butteraugli(w, h) as hr:
        assert tuple(hd.compute(z, z)) == tuple(hr.compute(z, z)) == (0.0, 0.0, 0.0)
