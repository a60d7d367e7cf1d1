"""The C++ layer (include/d2g.hpp) on the GPU: tests/cpp_consumer.cpp, a
C++17 host using the reference's names, runs compareTreesFull,
filterContacts, findContactsBucketComparison, separateCollisionClusters,
solve and compareTreesFullContinuous on a 2x2x2 cube scene and writes its
results; they must equal the oracle's bit for bit."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import delta2_gb300 as D
from oracle import oracle as O
from tests.clusters import separate

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _rd(path, dtype, cols=None):
    a = np.fromfile(path, dtype=dtype)
    return a.reshape(-1, cols) if cols else a


def _same(got, ref, what):
    got = np.ascontiguousarray(got, dtype=np.float64)
    ref = np.ascontiguousarray(ref, dtype=np.float64)
    assert got.shape == ref.shape, (what, got.shape, ref.shape)
    assert np.array_equal(got.view(np.uint64), ref.view(np.uint64)), what


def test_cpp_layer_device_methods_match_oracle(gpu_required, tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    from delta2_gb300 import build as B

    lib = B.build()
    libdir = os.path.dirname(lib)
    exe = tmp_path / "cpp_consumer"
    subprocess.run(["g++", "-std=c++17", "-Wall", "-Wextra", "-pedantic", "-Werror",
                    "-I" + os.path.join(ROOT, "include"), os.path.join(HERE, "cpp_consumer.cpp"), "-L" + libdir,
                    "-ld2g", "-Wl,-rpath," + libdir, "-o", str(exe)], check=True)
    out = subprocess.run([str(exe), str(tmp_path)], check=True, capture_output=True, text=True).stdout.strip()
    assert not out.startswith("FAIL"), out
    got = dict(kv.split("=") for kv in out.split())
    assert got["ctx"] == "0", out
    d = str(tmp_path)

    sc = D.make_scene(1, nx=2, ny=2, nz=2, spacing=1.12, speed_sigma=3.0, seed=1)
    pairs = D.broad_phase(sc)
    assert int(got["dev_pairs"]) == len(pairs)
    # compareTreesFull and filterContacts per pair
    ref, ref_off, _ = O.narrowphase(sc.copy(), pairs)
    assert np.array_equal(_rd(d + "/np_off.bin", np.int32), ref_off)
    _same(_rd(d + "/np.bin", np.float64, 14), ref, "compareTreesFull")
    kept = [O.filter_contacts(ref[ref_off[i]:ref_off[i + 1]], 0.0).reshape(-1, 14) for i in range(len(pairs))]
    kept_off = np.concatenate([[0], np.cumsum([len(k) for k in kept])])
    assert np.array_equal(_rd(d + "/kept_off.bin", np.int32), kept_off)
    _same(_rd(d + "/kept.bin", np.float64, 14), np.concatenate(kept), "filterContacts")
    # findContactsBucketComparison on pair 0's root level
    a, b = int(pairs[0, 0]), int(pairs[0, 1])
    level = [[int(sc.mesh_node_off[sc.mesh[a]]), int(sc.mesh_node_off[sc.mesh[b]])]]
    bref, bused = O.bucket_comparison(sc, a, b, level)
    assert _rd(d + "/bucket_used.bin", np.int32).tolist() == bused.tolist()
    _same(_rd(d + "/bucket.bin", np.float64, 14), bref, "findContactsBucketComparison")
    # separateCollisionClusters (first cluster) and its solve
    clusters = separate(pairs, sc.is_static, sc.n_bodies)
    parts, inter = clusters[0]
    assert _rd(d + "/cluster0.bin", np.int32).tolist() == list(parts)
    idx = [int(np.nonzero((pairs[:, 0] == i) & (pairs[:, 1] == j))[0][0]) for i, j in inter]
    hits = np.concatenate([kept[i] for i in idx])
    assert int(got["dev_hits"]) == len(hits) > 0
    w = O.World(sc.copy(), sc.opt_dt, sc.gravity_z)
    ok, _ = w.solve(parts, float(np.float32(sc.opt_dt)), hits)
    assert int(got["dev_accepted"]) == int(ok)
    _same(_rd(d + "/fut.bin", np.float64, 14), w.get_bodies().fut, "solve: future states")
    # compareTreesFullContinuous over 0.05 s
    cref, coff, _, _ = O.ccd(sc.copy(), pairs, np.full(len(pairs), 0.05))
    assert np.array_equal(_rd(d + "/ccd_off.bin", np.int32), coff)
    _same(_rd(d + "/ccd.bin", np.float64, 14), cref, "compareTreesFullContinuous")
    assert len(cref) > 0
