"""Build recipe of the CPU oracle (test infrastructure).

Compiles oracle/*.cpp into oracle/_build/liboracle.so with g++ (C++17, OpenMP).  FMA contraction
is disabled so that float results are reproducible bit-for-bit against the CUDA library, which is
built with --fmad=false.  No x86- or Arm-specific flags: the same recipe runs on both hosts.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
SOURCES = ["oracle_lbvh.cpp", "oracle_step.cpp"]
HEADERS = ["oracle_lbvh.h", "oracle_math.h", os.path.join("..", "include", "xrt.h")]


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    for f in SOURCES + HEADERS + ["build.py"]:
        if os.path.getmtime(os.path.join(HERE, f)) > t:
            return True
    return False


def build(force: bool = False) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-fno-fast-math", "-Wall", "-Wno-unused-function", "-o", LIB + ".tmp"]
    cmd += [os.path.join(HERE, s) for s in SOURCES]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
