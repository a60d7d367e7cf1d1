"""Native hosts of the library: a plain C11 program (tests/c_consumer.c)
and a C++17 one through include/d2g.hpp (tests/cpp_consumer.cpp).  The header
compiles as C, the library links, and the scene builder, the tree file and
the host broad phase give what the Python mirror gives; creating a context
reports the missing device instead of faking one."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import delta2_gb300 as D

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_c_program_uses_the_abi(tmp_path):
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    from delta2_gb300 import build as B

    lib = B.build()
    libdir = os.path.dirname(lib)
    exe = tmp_path / "c_consumer"
    subprocess.run(["gcc", "-std=c11", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I" + os.path.join(ROOT, "include"),
                    os.path.join(HERE, "c_consumer.c"), "-L" + libdir, "-ld2g", "-Wl,-rpath," + libdir, "-o",
                    str(exe)], check=True)
    out = subprocess.run([str(exe), str(tmp_path / "scene.trees")], check=True, capture_output=True,
                         text=True).stdout.strip()
    assert out.startswith("ok "), out
    got = dict(kv.split("=") for kv in out.split()[1:])
    # the same scene through the Python mirror
    cube_v = [[0.5 * a, 0.5 * b, 0.5 * c] for a, b, c in
              [[1, 1, 1], [1, 1, -1], [1, -1, 1], [1, -1, -1], [-1, 1, 1], [-1, 1, -1], [-1, -1, 1], [-1, -1, -1]]]
    cube_f = [[0, 2, 1], [1, 2, 3], [2, 6, 3], [3, 6, 7], [4, 5, 6], [5, 7, 6], [4, 0, 1], [4, 1, 5], [0, 4, 6],
              [0, 6, 2], [3, 7, 1], [7, 5, 1]]
    b = D.SceneBuilder(dt=1 / 240, gravity_z=-9.8)
    plane, _ = b.add_mesh([[50, 50, 0], [50, -50, 0], [-50, 50, 0], [-50, -50, 0]], [[0, 2, 1], [1, 2, 3]],
                          surface=True)
    cube, _ = b.add_mesh(cube_v, cube_f)
    b.add_body(plane, static=True)
    for k in range(3):
        b.add_body(cube, position=(1.5 * k, 0.0, 0.6), velocity=(0.0, 0.0, -1.0))
    s = b.finish()
    pairs = D.broad_phase(s)
    assert int(got["meshes"]) == 2 and int(got["nodes"]) == int(s.mesh_node_off[-1])
    assert int(got["bodies"]) == s.n_bodies
    assert np.float64(got["mass1"]) == s.mass[1]
    assert int(got["pairs"]) == len(pairs) > 0
    assert int(got["ctx"]) in (0, -3)  # D2G_OK with a GPU, D2G_ERR_NO_DEVICE without


def test_cpp_layer_uses_the_abi(tmp_path):
    # include/d2g.hpp (the C++ layer with the reference's names) in a C++17
    # host: a generated scene and one built from OBJ files, the host broad
    # phase; without a GPU, Context reports D2G_ERR_NO_DEVICE as an Error.
    # The library exports only its C ABI, so the host's own classes of the
    # same names as the library's internals cannot interpose on them.
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
    gen = D.make_scene(1)
    assert int(got["gen_bodies"]) == gen.n_bodies
    assert int(got["gen_pairs"]) == len(D.broad_phase(gen))
    assert int(got["own_bodies"]) == 4 and int(got["own_nodes"]) == 10 and int(got["own_pairs"]) == 5
    assert int(got["ctx"]) in (0, -3)


def test_library_exports_only_the_c_abi():
    # a version script keeps every symbol but d2g_* local to the library
    if shutil.which("nm") is None:
        pytest.skip("nm not available")
    from delta2_gb300 import build as B

    out = subprocess.run(["nm", "-D", "--defined-only", B.build()], check=True, capture_output=True,
                         text=True).stdout
    names = [ln.split()[-1] for ln in out.splitlines() if ln.strip()]
    assert names and all(n.startswith("d2g_") for n in names), [n for n in names if not n.startswith("d2g_")][:5]
