"""Build recipe for the CPU oracle (test infrastructure only).

Compiles the plain-C++ restatement in this folder into
``oracle/_build/libd2o.so``.  ``-ffp-contract=off`` keeps every multiply and
add separately rounded, the evaluation model the GPU kernels mirror; no
``-march`` flag so the same source gives the same bits on x86-64 and Arm.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libd2o.so")
SOURCES = ["d2o_capi.cpp"]
HEADERS = ["d2o_math.hpp", "d2o_geom.hpp", "d2o_collide.hpp", "d2o_solve.hpp"]


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(os.path.join(HERE, f)) > t for f in SOURCES + HEADERS + ["build.py"])


def build(force=False, verbose=False):
    if not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           "-o", LIB] + [os.path.join(HERE, s) for s in SOURCES]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
