"""Host policy of the serving runtime (admission, LRU source cache with pinning, FIFO continuous
batching), compiled from vship_gb300/csrc/serve_policy.h with the host C++ compiler and run on
the CPU."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_serve_policy(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "serve_policy_check")
    subprocess.run([cxx, "-std=c++17", "-O1", "-Wall", "-Werror", os.path.join(HERE, "native", "serve_policy_check.cpp"),
                    "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.split() == ["ok", "charges", "ok", "admission", "ok", "cache", "ok", "batching"]
