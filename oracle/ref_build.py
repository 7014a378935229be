"""Build the reference's own CUDA library (pkp24/Vship ``src/VshipLib.cpp``) for sm_103a.

Test and benchmark infrastructure only: the differential parity tests, the reference-fixture
script (``tests/golden/make_ref_golden.py``) and ``bench.py``'s ``reference_cuda`` leg load the
result, ``oracle/_ref/libvship_ref.so``. The product library never links or loads it.

Two steps, because the reference sources exist only in the container that holds the reference
checkout, while the library must be compiled on the machine that runs it (an Arm host with the
GPU; binaries built elsewhere do not travel):

* ``stage()`` copies the files the scored path compiles from (``src/VshipLib.cpp``,
  ``src/VshipAPI.h``, ``src/ssimu2``, ``src/butter``, ``src/util`` and the VapourSynth SDK
  headers the reference vendors in ``include/``) into ``oracle/_ref/src`` -- a build-staging
  copy, git-ignored, never committed -- unedited, and puts ``oracle/ref_cvvdp_stub.hpp`` where
  ``src/cvvdp/vapoursynth.hpp`` would be (CVVDP needs rapidjson, which is not vendored).
* ``build()`` compiles the staged copy the way the reference's Makefile ``buildcuda`` target
  does (``nvcc -x cu src/VshipLib.cpp -std=c++17 -I include -shared``, Makefile:49-50) with
  ``-O3`` and the sm_103a target, through ``oracle/ref_shim.cu``: one translation unit that
  includes ``VshipLib.cpp`` after two constants that make its v2 entry points' unqualified
  ``run<FLOAT>`` / ``run<UINT16>`` compile, and adds ``VshipRef_ComputeButteraugli``, the
  Butteraugli call with float norms (the reference's C ABI truncates them to ints). Nothing of
  the reference's own build system runs.

Usage: ``python -m oracle.ref_build [stage|build]`` (both when no argument is given).
"""
from __future__ import annotations

import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
STAGE = os.path.join(OUT, "src")
LIB = os.path.join(OUT, "libvship_ref.so")
STAMP = os.path.join(OUT, "staged.sha256")
SHIM = os.path.join(HERE, "ref_shim.cu")
CVVDP_STUB = os.path.join(HERE, "ref_cvvdp_stub.hpp")

# Where the reference checkout lies in the container that holds it.
REFERENCE = os.environ.get("VSHIP_REFERENCE_SRC", "/root/reference")

SRC_FILES = ["src/VshipLib.cpp", "src/VshipAPI.h"]
SRC_DIRS = ["src/ssimu2", "src/butter", "src/util"]
INCLUDE_FILES = ["include/VapourSynth4.h", "include/VSHelper4.h", "include/VSConstants4.h"]


def _digest(root: str) -> str:
    h = hashlib.sha256()
    for dp, _dn, fns in sorted(os.walk(root)):
        for fn in sorted(fns):
            p = os.path.join(dp, fn)
            h.update(os.path.relpath(p, root).encode())
            with open(p, "rb") as f:
                h.update(f.read())
    return h.hexdigest()


def staged() -> bool:
    return os.path.exists(os.path.join(STAGE, "src", "VshipLib.cpp"))


def stage(verbose: bool = False) -> bool:
    """Copy the reference's scored-path sources into oracle/_ref/src. Returns False (and leaves
    any earlier staging in place) when the reference checkout is not on this machine."""
    if not os.path.exists(os.path.join(REFERENCE, "src", "VshipLib.cpp")):
        return False
    tmp = STAGE + ".tmp"
    if os.path.exists(tmp):
        shutil.rmtree(tmp)
    for rel in SRC_FILES + INCLUDE_FILES:
        s = os.path.join(REFERENCE, rel)
        if not os.path.exists(s):
            continue
        d = os.path.join(tmp, rel)
        os.makedirs(os.path.dirname(d), exist_ok=True)
        shutil.copyfile(s, d)
    for rel in SRC_DIRS:
        shutil.copytree(os.path.join(REFERENCE, rel), os.path.join(tmp, rel))
    os.makedirs(os.path.join(tmp, "src", "cvvdp"), exist_ok=True)
    shutil.copyfile(CVVDP_STUB, os.path.join(tmp, "src", "cvvdp", "vapoursynth.hpp"))
    digest = _digest(tmp)
    old = open(STAMP).read().strip() if os.path.exists(STAMP) else None
    if old == digest and staged():
        shutil.rmtree(tmp)
        return True
    if os.path.exists(STAGE):
        shutil.rmtree(STAGE)
    os.replace(tmp, STAGE)
    with open(STAMP, "w") as f:
        f.write(digest + "\n")
    if verbose:
        print(f"staged reference sources from {REFERENCE} into {STAGE}", flush=True)
    return True


def build_command(nvcc: str = "nvcc") -> list[str]:
    return [nvcc, "-x", "cu", SHIM, "-std=c++17", "-O3", "-gencode", "arch=compute_103a,code=sm_103a",
            "-I", os.path.join(STAGE, "include"), "-I", os.path.join(STAGE, "src"),
            "-shared", "-Xcompiler", "-fPIC", "-w", "-o", LIB]


def _nvcc() -> str | None:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    return None


def up_to_date() -> bool:
    if not (os.path.exists(LIB) and staged()):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(p) <= t for p in (STAMP, SHIM))


def start_build(verbose: bool = False) -> subprocess.Popen | None:
    """Start the nvcc build of the staged reference in the background (None when there is
    nothing to do or nothing staged). ``finish_build`` waits for it."""
    if not staged() or up_to_date():
        return None
    nvcc = _nvcc()
    if nvcc is None:
        return None
    cmd = build_command(nvcc)
    if verbose:
        print(" ".join(cmd), flush=True)
    return subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)


def finish_build(proc: subprocess.Popen | None) -> str | None:
    if proc is None:
        return LIB if os.path.exists(LIB) else None
    out, _ = proc.communicate()
    if proc.returncode != 0:
        raise RuntimeError("reference CUDA build failed:\n" + out)
    return LIB


def build(verbose: bool = False) -> str | None:
    """Stage (where the checkout is) and compile; returns the library path, or None when no staged
    copy exists on this machine."""
    stage(verbose)
    return finish_build(start_build(verbose))


def available() -> bool:
    return os.path.exists(LIB)


if __name__ == "__main__":
    what = sys.argv[1] if len(sys.argv) > 1 else "all"
    if what == "stage":
        print("staged" if stage(True) else "reference checkout not found")
    elif what == "build":
        print(finish_build(start_build(True)))
    else:
        print(build(True))
