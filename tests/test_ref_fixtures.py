"""The oracle against the reference's own CUDA build: the fixtures in tests/golden/ref_golden.json
were produced by the reference library (pkp24/Vship src/VshipLib.cpp, built for sm_103a by
oracle/ref_build.py) on a GB300 (tests/golden/make_ref_golden.py). These pin the oracle's
restatement to the reference's actual outputs on non-trivial inputs.

Bounds (the reference computes in FP32; the oracle's FP64 instantiation is the error reference):
* Butteraugli: norms within 1e-5 relative of the FP64 oracle (the path's tolerance is 1e-4), the
  distortion map within 1e-4 of its maximum per pixel.
* SSIMU2: within 1e-3 absolute at 256x256 and above. On frames of a few thousand pixels the
  coarsest of the six scales holds a handful of pixels and the reference's FP32 pooled sums
  drift further from FP64 (up to about 3e-3 on the stored 64x48 to 139x87 cases); there the
  bound is 5e-3.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")
sys.path.insert(0, GOLD)

CASES = json.load(open(os.path.join(GOLD, "ref_golden.json")))["cases"]


def _frames(c):
    if c["source"] == "oracle_inputs.npz":
        d = np.load(os.path.join(GOLD, "oracle_inputs.npz"))
        return list(d[c["name"] + "_ref"]), list(d[c["name"] + "_dist"])
    d = np.load(os.path.join(GOLD, "ref_inputs.npz"))
    key = c.get("input_name", c["name"])
    f = lambda a: [np.ascontiguousarray(a[i].astype(np.uint16) * 257) for i in range(3)]
    return f(d[key + "_ref"]), f(d[key + "_dist"])


def _stored(metric):
    return [c for c in CASES if c["metric"] == metric and c["source"] != "synth"]


def test_fixtures_cover_the_workloads():
    names = {c["name"] for c in CASES}
    assert {"cfg1_rgb24_256", "cfg1_rgb24_256_q2_i203"} <= names
    assert sum(c["metric"] == "ssimu2" and c["source"] == "synth" for c in CASES) == 4
    assert sum(c["metric"] == "butter" and c["source"] == "synth" for c in CASES) == 4


@pytest.mark.parametrize("case", _stored("ssimu2"), ids=lambda c: c["name"])
def test_oracle_ssimu2_matches_reference_stored(orc, case):
    a, b = _frames(case)
    fp64 = orc.ssimu2(a, b, precision=64)
    bound = 1e-3 if case["w"] * case["h"] >= 256 * 256 else 5e-3
    assert abs(case["score"] - fp64) <= bound, (case["score"], fp64)


@pytest.mark.parametrize("case", _stored("butter"), ids=lambda c: c["name"])
def test_oracle_butteraugli_matches_reference_stored(orc, case):
    a, b = _frames(case)
    for prec in (64, 32):
        got, dm = orc.butteraugli(a, b, qnorm=case["qnorm"], intensity=case["intensity"], precision=prec,
                                  distmap=True)
        for g, r in zip(got, case["norms"]):
            assert abs(g - r) <= 1e-5 * abs(r), (prec, got, case["norms"])
        ref_dm = np.load(os.path.join(GOLD, "ref_golden_maps.npz"))[case["name"]]
        assert np.max(np.abs(dm - ref_dm)) <= 1e-4 * float(ref_dm.max())


def _regenerate(case):
    import make_ref_golden as mk
    spec = mk.SSIMU2_1080P if case["metric"] == "ssimu2" else mk.BUTTER_4K
    fr, fd, ysha, _ = mk.large_pair(spec, case["t"])
    assert ysha == case["yuv_sha256"], "the seeded Y'CbCr planes regenerate differently on this host"
    return fr, fd, mk


@pytest.mark.parametrize("case", [c for c in CASES if c["metric"] == "ssimu2" and c["source"] == "synth"],
                         ids=lambda c: c["name"])
def test_oracle_ssimu2_matches_reference_1080p(orc, case):
    fr, fd, mk = _regenerate(case)
    fp64 = orc.ssimu2(list(fr), list(fd), precision=64)
    assert abs(case["score_float"] - fp64) <= 1e-3
    fp64u = orc.ssimu2(list(mk.rgb48(fr)), list(mk.rgb48(fd)), precision=64)
    assert abs(case["score_rgb48"] - fp64u) <= 1e-3


def test_oracle_butteraugli_matches_reference_4k(orc):
    case = next(c for c in CASES if c["name"] == "butter_4k_blur_noise_0")
    fr, fd, _ = _regenerate(case)
    got, dm = orc.butteraugli(list(fr), list(fd), qnorm=2, intensity=203.0, precision=64, distmap=True)
    for g, r in zip(got, case["norms"]):
        assert abs(g - r) <= 1e-5 * abs(r), (got, case["norms"])
    sub = np.load(os.path.join(GOLD, "ref_golden_maps.npz"))[case["name"] + "_sub"]
    s = case["distmap_sub"]
    assert np.max(np.abs(dm[::s, ::s] - sub)) <= 1e-4 * case["distmap_max"]
