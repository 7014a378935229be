"""The decoders divide samples by constants with a reciprocal product and one FMA residual
correction; this checks on the host, for every numerator they can see, that the result equals
IEEE division (the reference divides: util/float3operations.hpp:201-218)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_division_by_constants_is_exact(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "div_check")
    subprocess.run([cxx, "-std=c++17", "-O2", "-ffp-contract=off", os.path.join(HERE, "native", "div_check.cpp"),
                    "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True)
    assert out.returncode == 0 and out.stdout.strip() == "ok", out.stdout
