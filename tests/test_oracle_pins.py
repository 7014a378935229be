"""Pins of the CPU oracle.

1. The reference's only known-answer test (test/basic_metric_math_test.cpp:40-79): identical
   frames -> SSIMU2 exactly 100, Butteraugli (0, 0, 0) and an all-zero distortion map, with
   0xFF bytes in the stride padding ignored. The reference runs it at 5076x9400 (SSIMU2) and
   1076x2400 (Butteraugli); the CPU oracle runs scaled-down sizes with the same padding pattern
   (the GPU tests run the full sizes).
2. The oracle's constant tables against the reference source text (skipped where the reference
   tree is absent).
3. Committed golden outputs of the oracle (tests/golden/oracle_golden.json, made by
   tests/golden/make_golden.py) so the oracle gives the same numbers on every host.
"""
import json
import os
import re

import numpy as np
import pytest

from helpers import padded, u16_planes_from_rgb24, float_planes
from vship_gb300 import synth

from conftest import REFERENCE_TREE

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "oracle_golden.json")
GOLDEN_INPUTS = os.path.join(os.path.dirname(__file__), "golden", "oracle_inputs.npz")


@pytest.mark.parametrize("precision", [32, 64])
def test_kat_identical_ssimu2_is_100(orc, precision):
    z = [np.zeros((94, 507), np.float32) for _ in range(3)]
    a = padded(z, 3000 - 507 * 4, 0x00)
    b = padded(z, 3000 - 507 * 4, 0xFF)
    assert orc.ssimu2(a, b, precision=precision) == 100.0


@pytest.mark.parametrize("precision", [32, 64])
def test_kat_identical_butteraugli_is_zero(orc, precision):
    z = [np.zeros((240, 107), np.float32) for _ in range(3)]
    a = padded(z, 1000 - 107 * 4, 0x00)
    b = padded(z, 1000 - 107 * 4, 0xFF)
    norms, dm = orc.butteraugli(a, b, precision=precision, distmap=True)
    assert norms == (0.0, 0.0, 0.0)
    assert not dm.any()


def test_identical_nonzero_frames(orc):
    r, _ = synth.rgb24_pair(64, 48, seed=3)
    a = u16_planes_from_rgb24(r)
    assert orc.ssimu2(a, a) == 100.0
    assert orc.butteraugli(a, a) == (0.0, 0.0, 0.0)


def test_stride_padding_ignored(orc):
    r, d = synth.rgb24_pair(40, 56, seed=5)
    a, b = u16_planes_from_rgb24(r), u16_planes_from_rgb24(d)
    s0 = orc.ssimu2(a, b)
    s1 = orc.ssimu2(padded(a, 64, 0xFF), padded(b, 16, 0x7F))
    assert s0 == s1
    n0 = orc.butteraugli(a, b)
    n1 = orc.butteraugli(padded(a, 32, 0xFF), padded(b, 8, 0xAB))
    assert n0 == n1


def test_fp32_close_to_fp64(orc):
    r, d = synth.rgb24_pair(128, 96, seed=11)
    a, b = u16_planes_from_rgb24(r), u16_planes_from_rgb24(d)
    assert abs(orc.ssimu2(a, b, precision=32) - orc.ssimu2(a, b)) < 1e-3
    n32 = orc.butteraugli(a, b, precision=32)
    n64 = orc.butteraugli(a, b)
    for x, y in zip(n32, n64):
        assert abs(x - y) <= 1e-4 * abs(y)


def test_golden(orc):
    with open(GOLDEN) as f:
        gold = json.load(f)
    inputs = np.load(GOLDEN_INPUTS)
    for case in gold["cases"]:
        frames = list(inputs[case["name"] + "_ref"]), list(inputs[case["name"] + "_dist"])
        if case["metric"] == "ssimu2":
            got = orc.ssimu2(*frames, precision=case["precision"])
            assert got == pytest.approx(case["score"], abs=1e-9), case["name"]
        else:
            got = orc.butteraugli(*frames, qnorm=case["qnorm"], intensity=case["intensity"],
                                  precision=case["precision"])
            assert got == pytest.approx(tuple(case["norms"]), rel=1e-9), case["name"]


# ------------------------------------------------------------------------------------------
# constant tables vs the reference source text

ref_missing = not os.path.isdir(os.path.join(REFERENCE_TREE, "src"))


def _read(rel):
    with open(os.path.join(REFERENCE_TREE, rel)) as f:
        return f.read()


@pytest.mark.skipif(ref_missing, reason="reference tree not present")
def test_weights_match_reference_source(orc):
    src = _read("src/ssimu2/score.hpp")
    blk = src[src.index("const float weights[108]"):]
    blk = blk[blk.index("{") + 1: blk.index("};")]
    ref = [float(x.strip().rstrip("f")) for x in blk.split(",") if x.strip()]
    assert len(ref) == 108
    assert orc.ssimu2_weights() == ref


def _parse_malta(unit_src):
    pats = []
    for block in unit_src.split("retval += sum * sum;")[:-1]:
        expr = block[block.rindex("float sum ="):]
        taps = []
        for idx in re.findall(r"d\[([^\]]+)\]", expr):
            e = idx.replace(" ", "")
            dx = dy = 0
            for sign, term in re.findall(r"([+-]?)([^+-]+)", e):
                s = -1 if sign == "-" else 1
                if term == "xs3":
                    dy += 3 * s
                elif term == "xs":
                    dy += s
                else:
                    dx += s * int(term)
            taps.append((dx, dy))
        pats.append(taps)
    return pats


@pytest.mark.skipif(ref_missing, reason="reference tree not present")
def test_malta_patterns_match_reference_source(orc):
    src = _read("src/butter/maltaDiff.hpp")
    lf = src[src.index("float MaltaUnitLF("): src.index("float MaltaUnit(")]
    hf = src[src.index("float MaltaUnit("): src.index("__global__ void MaltaDiffMap_Kernel")]
    for unit_src, is_hf in ((lf, False), (hf, True)):
        ref = _parse_malta(unit_src)
        assert len(ref) == 16
        for i, taps in enumerate(ref):
            assert orc.malta_pattern(is_hf, i) == taps, (is_hf, i)


@pytest.mark.skipif(ref_missing, reason="reference tree not present")
def test_kernel_sources_carry_the_same_malta_patterns():
    """The CUDA kernel spells the patterns out as macros; compare them with the reference too."""
    here = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    with open(os.path.join(here, "vship_gb300", "csrc", "butter.cu")) as f:
        cu = f.read()
    src = _read("src/butter/maltaDiff.hpp")
    lf = _parse_malta(src[src.index("float MaltaUnitLF("): src.index("float MaltaUnit(")])
    hf = _parse_malta(src[src.index("float MaltaUnit("): src.index("__global__ void MaltaDiffMap_Kernel")])
    for name, ref in (("MALTA_HF_BODY", hf), ("MALTA_LF_BODY", lf)):
        body = cu[cu.index("#define " + name):]
        lines = [ln for ln in body.split("\n")[1:17]]
        got = [[(int(a), int(b)) for a, b in re.findall(r"W\((-?\d+), (-?\d+)\)", ln)] for ln in lines]
        assert got == ref, name


@pytest.mark.skipif(ref_missing, reason="reference tree not present")
def test_butter_sigmas_and_constants_match_reference_source():
    g = _read("src/butter/gaussianblur.hpp")
    assert "{1.2, 1.56416327805, 2.7, 3.22489901262, 7.15593339443}" in g
    here = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    with open(os.path.join(here, "oracle", "oracle.cpp")) as f:
        orc_src = f.read()
    # every float literal of the reference's butteraugli constant sets appears in the oracle
    for rel in ("src/butter/main.hpp", "src/butter/separatefrequencies.hpp", "src/butter/combineMasks.hpp",
                "src/butter/maskPsycho.hpp", "src/butter/colors.hpp"):
        for lit in re.findall(r"\b\d+\.\d{4,}f?\b", _read(rel)):
            assert lit.rstrip("f") in orc_src, (rel, lit)
