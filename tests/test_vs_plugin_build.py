"""The VapourSynth plugin entry (vship_gb300/csrc/vs_plugin.cpp) compiles against the VapourSynth
SDK headers and exports VapourSynthPluginInit2 -- the symbol VapourSynth looks up when it loads
libvship.so as a plugin. The SDK headers are taken from the reference tree's vendored copy when
present (this test only compiles; VapourSynth itself is not installed here)."""
import os
import subprocess

import pytest

from conftest import REFERENCE_TREE

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SDK = os.environ.get("VAPOURSYNTH_INCLUDE") or os.path.join(REFERENCE_TREE, "include")


@pytest.mark.skipif(not os.path.exists(os.path.join(SDK, "VapourSynth4.h")), reason="no VapourSynth SDK headers")
def test_plugin_compiles_and_exports_entry(tmp_path):
    obj = tmp_path / "vs_plugin.o"
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-fPIC", "-fvisibility=hidden", "-I" + SDK,
                        "-I" + os.path.join(ROOT, "include"), "-c", os.path.join(ROOT, "vship_gb300", "csrc",
                                                                                 "vs_plugin.cpp"), "-o", str(obj)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    syms = subprocess.run(["nm", "-g", "--defined-only", str(obj)], capture_output=True, text=True).stdout
    assert " T VapourSynthPluginInit2" in syms
