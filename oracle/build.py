"""Build recipe for the CPU oracle (test infrastructure only).

Compiles the plain-C++ restatement in this folder twice:

* ``oracle/_build/libd2o.so`` (``-O2``, no ``-march``): the parity checker the
  tests load; the same source gives the same bits on x86-64 and Arm;
* ``oracle/_build/libd2o_fast.so`` (``-O3`` and ``-march=native`` on x86-64,
  ``-mcpu=native`` on Arm): the build the benchmark's CPU baselines time,
  tuned for the host it runs on.

Both keep ``-ffp-contract=off`` and no fast-math, so every multiply and add is
rounded on its own (the evaluation model the GPU kernels mirror) and the two
builds give identical results (``tests/test_oracle_golden.py`` checks it on
the benchmark workload).
"""
import concurrent.futures as cf
import os
import platform
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libd2o.so")
LIB_FAST = os.path.join(OUT_DIR, "libd2o_fast.so")
SOURCES = ["d2o_capi.cpp"]
HEADERS = ["d2o_math.hpp", "d2o_geom.hpp", "d2o_collide.hpp", "d2o_solve.hpp", "d2o_tree.hpp", "d2o_mass.hpp"]


def _stale(lib):
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    return any(os.path.getmtime(os.path.join(HERE, f)) > t for f in SOURCES + HEADERS + ["build.py"])


def _native_flag():
    return "-mcpu=native" if platform.machine().lower() in ("aarch64", "arm64") else "-march=native"


def _compile(lib, opt, verbose):
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = lib + ".tmp"
    cmd = ["g++", "-std=c++17"] + opt + ["-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-o", tmp] + \
        [os.path.join(HERE, s) for s in SOURCES]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(tmp, lib)
    return lib


def build(force=False, verbose=False, fast=False):
    """Compile (if stale) and return the path of the checker build, or with
    fast=True of the host-tuned build the CPU baselines time."""
    lib, opt = (LIB_FAST, ["-O3", _native_flag()]) if fast else (LIB, ["-O2"])
    if not force and not _stale(lib):
        return lib
    return _compile(lib, opt, verbose)


def build_all(force=False, verbose=False):
    with cf.ThreadPoolExecutor(2) as ex:
        return list(ex.map(lambda f: build(force, verbose, fast=f), [False, True]))


if __name__ == "__main__":
    print(build_all(force="--force" in sys.argv, verbose=True))
