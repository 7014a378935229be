"""Score fixed inputs with the reference's own CUDA build and write the results as fixtures.

Runs on a machine with a GPU and the reference library built (``python -m oracle.ref_build``,
which ``__graft_entry__.build()`` also runs). Writes ``ref_golden.json`` and
``ref_golden_maps.npz`` into ``--out``; they are committed under ``tests/golden/``:

  python tests/golden/make_ref_golden.py --out tests/golden

Cases (every one through the reference's handler calls, oracle/reference_cuda.py):

* the stored-input cases of ``oracle_inputs.npz`` (SSIMU2 scores; Butteraugli float norms and
  full distortion maps), except sizes at which the reference's Butteraugli reads outside its own
  allocations (``oracle.reference_cuda.butteraugli_size_safe``: 72x56 is one);
* ``ref_inputs.npz`` (written here on first use, committed): the 256x256 RGB24 pair of the
  single-pair workload (seed 1) and a 139x87 RGB24 pair (seed 5), each scored by SSIMU2 and by
  Butteraugli (Qnorm 2, intensity 203; Qnorm 5, intensity 80) with full distortion maps;
* 4 pairs of the 1920x1080 YUV420P10 block-DCT workload (seed 7, pairs 0-3), converted to float32
  R'G'B' and to RGB48 by ``vship_gb300.synth``: SSIMU2 on both;
* 4 pairs of the 3840x2160 YUV420P10 blur + noise workload (seed 11, pairs 0-3) as float32
  R'G'B': Butteraugli norms (Qnorm 2, intensity 203), distortion-map sum and maximum, and every
  32nd pixel of every 32nd row of the map.

The large inputs are not stored: tests regenerate them and first check the SHA-256 of the
integer Y'CbCr planes recorded here (``yuv_sha256``), and of the R'G'B' planes (``rgb_sha256``).
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

SUB = 32  # 4K distortion-map subsampling step (rows and columns)

STORED_SMALL = [
    dict(name="cfg1_rgb24_256", h=256, w=256, seed=1),
    dict(name="rgb24_139x87", h=87, w=139, seed=5),
]
SSIMU2_1080P = dict(h=1080, w=1920, seed=7, distortion="dct", pairs=4)
BUTTER_4K = dict(h=2160, w=3840, seed=11, distortion="blur_noise", pairs=4)


def sha(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def small_inputs(path: str) -> dict:
    """The stored small RGB24 pairs (uint8, (3, H, W)); generated once, then read back."""
    if os.path.exists(path):
        d = np.load(path)
        return {k: d[k] for k in d.files}
    from vship_gb300 import synth
    arrays = {}
    for c in STORED_SMALL:
        r, d = synth.rgb24_pair(c["h"], c["w"], seed=c["seed"])
        arrays[c["name"] + "_ref"] = r.numpy()
        arrays[c["name"] + "_dist"] = d.numpy()
    np.savez_compressed(path, **arrays)
    return arrays


def large_pair(spec: dict, t: int):
    """(float32 ref (3,H,W), float32 dist, yuv sha256, rgb sha256) of pair t of a large workload."""
    from vship_gb300 import synth
    r, d = synth.yuv420p10_frames(spec["h"], spec["w"], t, seed=spec["seed"], distortion=spec["distortion"])
    fr = synth.yuv420p10_to_rgb(r).numpy()
    fd = synth.yuv420p10_to_rgb(d).numpy()
    ysha = sha(*[p.numpy().astype(np.int32) for p in r + d])
    return fr, fd, ysha, sha(fr, fd)


def rgb48(x: np.ndarray) -> np.ndarray:
    return np.round(np.clip(x, 0.0, 1.0) * 65535.0).astype(np.uint16)


def u16(x: np.ndarray) -> np.ndarray:
    return x.astype(np.uint16) * 257


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=HERE)
    ap.add_argument("--skip-large", action="store_true")
    args = ap.parse_args()
    from oracle import reference_cuda as R

    R.lib()
    os.makedirs(args.out, exist_ok=True)
    cases, maps = [], {}

    # 1. the oracle's stored-input cases
    gold = json.load(open(os.path.join(HERE, "oracle_golden.json")))
    inp = np.load(os.path.join(HERE, "oracle_inputs.npz"))
    seen = set()
    for c in gold["cases"]:
        if c["name"] in seen:
            continue
        seen.add(c["name"])
        a, b = inp[c["name"] + "_ref"], inp[c["name"] + "_dist"]
        if c["metric"] == "butter" and not R.butteraugli_size_safe(c["w"], c["h"]):
            continue
        rec = {"name": c["name"], "source": "oracle_inputs.npz", "metric": c["metric"], "h": c["h"], "w": c["w"]}
        if c["metric"] == "ssimu2":
            with R.SSIMU2(c["w"], c["h"]) as h:
                rec["score"] = h.compute(list(a), list(b))
        else:
            rec.update(qnorm=c["qnorm"], intensity=c["intensity"])
            with R.Butteraugli(c["w"], c["h"], c["qnorm"], c["intensity"]) as h:
                n, dm = h.compute(list(a), list(b), distmap=True)
            rec["norms"] = list(n)
            maps[c["name"]] = dm
        cases.append(rec)

    # 2. stored small RGB24 pairs, both metrics
    small = small_inputs(os.path.join(HERE, "ref_inputs.npz"))
    for c in STORED_SMALL:
        a, b = u16(small[c["name"] + "_ref"]), u16(small[c["name"] + "_dist"])
        with R.SSIMU2(c["w"], c["h"]) as h:
            cases.append({"name": c["name"], "source": "ref_inputs.npz", "metric": "ssimu2", "h": c["h"], "w": c["w"],
                          "input": "uint16 (8-bit x 257)", "score": h.compute(list(a), list(b))})
        for q, it in ((2, 203.0), (5, 80.0)):
            with R.Butteraugli(c["w"], c["h"], q, it) as h:
                n, dm = h.compute(list(a), list(b), distmap=True)
            nm = f"{c['name']}_q{q}_i{int(it)}"
            cases.append({"name": nm, "source": "ref_inputs.npz", "input_name": c["name"], "metric": "butter",
                          "h": c["h"], "w": c["w"], "input": "uint16 (8-bit x 257)", "qnorm": q, "intensity": it,
                          "norms": list(n)})
            maps[nm] = dm

    # 3. large workloads, regenerated from their seeds
    if not args.skip_large:
        s = SSIMU2_1080P
        with R.SSIMU2(s["w"], s["h"]) as h:
            for t in range(s["pairs"]):
                fr, fd, ysha, rsha = large_pair(s, t)
                cases.append({"name": f"ssimu2_1080p_dct_{t}", "source": "synth", "metric": "ssimu2", "h": s["h"],
                              "w": s["w"], "seed": s["seed"], "t": t, "distortion": s["distortion"],
                              "yuv_sha256": ysha, "rgb_sha256": rsha,
                              "score_float": h.compute(list(fr), list(fd)),
                              "score_rgb48": h.compute(list(rgb48(fr)), list(rgb48(fd)))})
        s = BUTTER_4K
        with R.Butteraugli(s["w"], s["h"], 2, 203.0) as h:
            for t in range(s["pairs"]):
                fr, fd, ysha, rsha = large_pair(s, t)
                n, dm = h.compute(list(fr), list(fd), distmap=True)
                nm = f"butter_4k_blur_noise_{t}"
                cases.append({"name": nm, "source": "synth", "metric": "butter", "h": s["h"], "w": s["w"],
                              "seed": s["seed"], "t": t, "distortion": s["distortion"], "qnorm": 2,
                              "intensity": 203.0, "yuv_sha256": ysha, "rgb_sha256": rsha, "norms": list(n),
                              "distmap_sum": float(dm.astype(np.float64).sum()), "distmap_max": float(dm.max()),
                              "distmap_sub": SUB})
                maps[nm + "_sub"] = np.ascontiguousarray(dm[::SUB, ::SUB])

    meta = {"generator": "tests/golden/make_ref_golden.py",
            "library": "reference CUDA build (oracle/ref_build.py), sm_103a",
            "cases": cases}
    with open(os.path.join(args.out, "ref_golden.json"), "w") as f:
        json.dump(meta, f, indent=1)
    np.savez_compressed(os.path.join(args.out, "ref_golden_maps.npz"), **maps)
    print(f"wrote {len(cases)} cases, {len(maps)} maps to {args.out}")


if __name__ == "__main__":
    main()
