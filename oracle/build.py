"""Build the oracle (test infrastructure only): oracle/liboracle.so from oracle/oracle.cpp.

The oracle is the CPU restatement used as the checker by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg. The product library never links or loads it.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "oracle.cpp")
LIB = os.path.join(HERE, "liboracle.so")

# -ffp-contract=off: no implicit FMA contraction, so x86 and Arm hosts round the same way.
FLAGS = ["-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-Wall", "-Wno-unused-function"]


def build(verbose: bool = False) -> str:
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cmd = ["g++"] + FLAGS + [SRC, "-o", LIB, "-lpthread"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
