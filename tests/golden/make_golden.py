"""Regenerate tests/golden/oracle_inputs.npz and oracle_golden.json.

Inputs are small seeded synthetic frame pairs (vship_gb300.synth); outputs are the oracle's
scores at FP64 and FP32. Stored inputs make the pin independent of the generator's host math.
Run from the repository root: python tests/golden/make_golden.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402
from vship_gb300 import synth  # noqa: E402

CASES = [
    dict(name="ssimu2_rgb24_64x48", metric="ssimu2", input="rgb24", h=48, w=64, seed=3),
    dict(name="ssimu2_dct_72x56", metric="ssimu2", input="dct", h=56, w=72, seed=7, t=2),
    dict(name="butter_blur_72x56", metric="butter", input="blur_noise", h=56, w=72, seed=7, t=1, qnorm=2,
         intensity=203.0),
    dict(name="butter_rgb24_q5_i80", metric="butter", input="rgb24", h=48, w=64, seed=4, qnorm=5, intensity=80.0),
]


def frames(case):
    if case["input"] == "rgb24":
        r, d = synth.rgb24_pair(case["h"], case["w"], seed=case["seed"])
        f = lambda t: np.ascontiguousarray(t.numpy().astype(np.uint16) * 257)
    else:
        r, d = synth.rgb_float_pair(case["h"], case["w"], case["t"], case["seed"], case["input"])
        f = lambda t: np.ascontiguousarray(t.numpy().astype(np.float32))
    return f(r), f(d)


def main():
    arrays = {}
    out = []
    for case in CASES:
        a, b = frames(case)
        arrays[case["name"] + "_ref"] = a
        arrays[case["name"] + "_dist"] = b
        for prec in (64, 32):
            c = dict(case, precision=prec)
            if case["metric"] == "ssimu2":
                c["score"] = oracle.ssimu2(list(a), list(b), precision=prec)
            else:
                c["norms"] = list(oracle.butteraugli(list(a), list(b), qnorm=case["qnorm"],
                                                     intensity=case["intensity"], precision=prec))
            out.append(c)
    np.savez_compressed(os.path.join(HERE, "oracle_inputs.npz"), **arrays)
    with open(os.path.join(HERE, "oracle_golden.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py", "cases": out}, f, indent=1)


if __name__ == "__main__":
    main()
