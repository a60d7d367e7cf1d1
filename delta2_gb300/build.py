"""Build the sm_103a CUDA library ``delta2_gb300/_lib/libd2g.so``.

Device code: ``nvcc -gencode arch=compute_103a,code=sm_103a -fmad=false``
(every FP64 multiply and add rounded on its own, the evaluation model the
CPU oracle uses).  Host code: ``g++ -ffp-contract=off`` (no FMA contraction
on Arm either).  Translation units compile in parallel; the result is loaded
in-tree by ``delta2_gb300/__init__.py``.
"""
import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
ROOT = os.path.dirname(HERE)
OUT = os.path.join(HERE, "_lib")
OBJ = os.path.join(OUT, "obj")
LIB = os.path.join(OUT, "libd2g.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

CU_SOURCES = ["d2g_engine.cu", "d2g_step.cu", "d2g_solve.cu", "d2g_broadphase.cu", "d2g_mlp.cu", "d2g_mesh.cu"]
CPP_SOURCES = ["d2g_capi.cpp", "d2g_world.cpp", "host/d2g_scene.cpp", "host/d2g_broad.cpp", "host/d2g_treefile.cpp",
               "host/d2g_obj.cpp"]


def _cuda_home():
    for c in [os.environ.get("CUDA_HOME"), "/usr/local/cuda"]:
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build delta2_gb300")


def _all_inputs():
    files = []
    for d, _, fs in os.walk(CSRC):
        files += [os.path.join(d, f) for f in fs if f.endswith((".cu", ".cuh", ".cpp", ".hpp", ".h", ".map"))]
    files.append(os.path.join(ROOT, "include", "d2g.h"))
    files.append(os.path.abspath(__file__))
    return sorted(files)


def _fingerprint():
    h = hashlib.sha256()
    for f in _all_inputs():
        h.update(f.encode())
        with open(f, "rb") as fh:
            h.update(fh.read())
    h.update(os.uname().machine.encode())
    return h.hexdigest()


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(force=False, verbose=False):
    """Compile (if sources changed) and return the library path."""
    fp = _fingerprint()
    stamp = os.path.join(OUT, "fingerprint")
    if not force and os.path.exists(LIB) and os.path.exists(stamp) and open(stamp).read() == fp:
        return LIB
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(OBJ, exist_ok=True)
    jobs = []
    for src in CU_SOURCES:
        o = os.path.join(OBJ, os.path.basename(src).replace(".cu", ".o"))
        jobs.append([nvcc, "-c", os.path.join(CSRC, src), "-o", o, ARCH, "-lineinfo", "-O3", "-std=c++17",
                     "-fmad=false", "-Xptxas=-v" if verbose else "-Xptxas=-O3",
                     "-Xcompiler=-fPIC,-ffp-contract=off", "-I" + CSRC])
    for src in CPP_SOURCES:
        o = os.path.join(OBJ, os.path.basename(src).replace(".cpp", ".o"))
        jobs.append(["g++", "-c", os.path.join(CSRC, src), "-o", o, "-O2", "-std=c++17", "-fPIC",
                     "-ffp-contract=off", "-fno-fast-math", "-pthread", "-Wall", "-Wno-unused-function",
                     "-I" + os.path.join(cuda, "include"), "-I" + CSRC])
    with cf.ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            if o.strip():
                print(o)
    objs = [j[j.index("-o") + 1] for j in jobs]
    tmp = LIB + ".tmp"
    _run([nvcc, "-shared", ARCH, "-o", tmp] + objs +
         ["-Xcompiler=-fPIC,-pthread", "-Xlinker=--version-script=" + os.path.join(CSRC, "d2g.map")])
    os.replace(tmp, LIB)
    with open(stamp, "w") as f:
        f.write(fp)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
