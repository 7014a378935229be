"""Build libvship.so (the product) in-tree with nvcc for sm_103a.

Usage: ``python -m vship_gb300.build`` or ``vship_gb300.build.build()``.
Translation units compile in parallel into ``vship_gb300/_build`` and link into
``vship_gb300/libvship.so`` (CUDA runtime linked statically, only the C ABI exported).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libvship.so")
ROOT = os.path.dirname(HERE)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-fvisibility=hidden",
    "-I" + os.path.join(ROOT, "include"), "-I" + CSRC,
]
SOURCES = ["ssimu2.cu", "butter.cu", "api.cu", "profile.cu", "noalloc.cu", "multi.cu", "serve.cu"]
CLI = os.path.join(HERE, "ffvship")


def nvcc_path() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libvship.so")


def vapoursynth_include() -> str | None:
    """Directory holding the VapourSynth SDK headers, if any (VAPOURSYNTH_INCLUDE or the usual
    system locations). libvship.so is also a VapourSynth plugin when they are found."""
    for d in (os.environ.get("VAPOURSYNTH_INCLUDE"), "/usr/include/vapoursynth", "/usr/local/include/vapoursynth"):
        if d and os.path.exists(os.path.join(d, "VapourSynth4.h")) and os.path.exists(os.path.join(d, "VSHelper4.h")):
            return d
    return None


def _needs_rebuild(obj: str, deps: list[str]) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, extra_flags: list[str] | None = None) -> str:
    nvcc = nvcc_path()
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "VshipAPI.h"))
    flags = NVCC_FLAGS + list(extra_flags or [])
    jobs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        if _needs_rebuild(o, [s] + headers) or extra_flags:
            jobs.append([nvcc] + flags + ["-c", s, "-o", o])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        return r

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        list(ex.map(run, jobs))
    objs = [os.path.join(BUILD, s.replace(".cu", ".o")) for s in SOURCES]
    vsinc = vapoursynth_include()
    if vsinc:
        src = os.path.join(CSRC, "vs_plugin.cpp")
        obj = os.path.join(BUILD, "vs_plugin.o")
        if _needs_rebuild(obj, [src] + headers):
            run(["g++", "-O2", "-std=c++17", "-fPIC", "-fvisibility=hidden", "-I" + vsinc,
                 "-I" + os.path.join(ROOT, "include"), "-c", src, "-o", obj])
            jobs.append("vs_plugin")
        objs.append(obj)
    if jobs or not os.path.exists(LIB):
        run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lpthread", "-ldl"])
    cli_src = os.path.join(CSRC, "ffvship.cpp")
    if _needs_rebuild(CLI, [cli_src, LIB, os.path.join(ROOT, "include", "VshipAPI.h")]):
        # the FFVship-compatible command-line tool, linked against the library next to it
        run(["g++", "-O2", "-std=c++17", cli_src, "-I" + os.path.join(ROOT, "include"), "-L" + HERE, "-lvship",
             "-Wl,-rpath,$ORIGIN", "-lpthread", "-o", CLI])
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
