"""CPU tests of the product's host side: the C-ABI library loads and exports
every entry point of include/d2g.h; scenes and surrogate trees are built as
the reference builds them (no GPU is used)."""
import os
import re

import numpy as np
import pytest

import delta2_gb300 as D
from delta2_gb300 import build as B

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="session", autouse=True)
def built():
    B.build()


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "d2g.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(d2g_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    import ctypes
    L = ctypes.CDLL(D.library_path())
    syms = declared_symbols()
    assert len(syms) >= 15
    missing = [s for s in syms if not hasattr(L, s)]
    assert not missing, missing


def test_no_device_is_reported_not_faked():
    # On a machine without a GPU the context fails with D2G_ERR_NO_DEVICE.
    from tests.conftest import has_gpu
    if has_gpu():
        pytest.skip("GPU present")
    with pytest.raises(D.D2GError) as e:
        D.Context()
    assert e.value.code == -3


def point_tri_dist(p, t):
    """Independent brute-force point-triangle distance (projection + edges)."""
    a, b, c = t[0:3], t[3:6], t[6:9]
    n = np.cross(b - a, c - a)
    n = n / np.linalg.norm(n)
    q = p - np.dot(p - a, n) * n
    m = np.array([b - a, c - a]).T
    uv, *_ = np.linalg.lstsq(m, q - a, rcond=None)
    if uv[0] >= 0 and uv[1] >= 0 and uv[0] + uv[1] <= 1:
        return abs(np.dot(p - a, n))
    best = np.inf
    for u, v in [(a, b), (b, c), (c, a)]:
        d = v - u
        s = np.clip(np.dot(p - u, d) / np.dot(d, d), 0, 1)
        best = min(best, np.linalg.norm(p - (u + s * d)))
    return best


def test_cube_scene_matches_reference_conventions():
    s = D.make_scene(1)
    assert s.n_bodies == 65 and s.is_static[0] == 1 and not s.is_static[1:].any()
    # 1 m cube at 1000 kg/m^3; inertia m*(1+1)/12 (model/test_mesh_data.cpp:6-22 scaled)
    assert np.allclose(s.mass[1:], 1000.0)
    assert np.allclose(s.inv_inertia[1].reshape(3, 3), np.eye(3) / (1000.0 * 2 / 12), rtol=1e-12)
    # 12-triangle cube: root inner node (8 surrogates) + 8 leaves (surrogate_tree.cpp:52-107)
    lo, hi = s.mesh_node_off[1], s.mesh_node_off[2]
    assert hi - lo == 9
    assert s.nodes[lo].tolist()[1:] == [8, 1, 0]
    assert s.ntris[lo + 1:hi].sum() == 12
    assert np.all(s.last_dt == np.float32(1 / 120))
    # bodies start 0.25 m clear of the ground (no initial intersection)
    z = s.cur[1:, 10]
    assert z.min() - 0.8660254037844386 - 0.125 >= 0.25 - 1e-12


def test_tree_eps_bounds_children():
    """Every original triangle below surrogate i lies within eps[i] of it
    (construct_surrogate_tree.h:172-185)."""
    s = D.make_scene(2, nx=2, ny=2, nz=1)
    for m in range(1, len(s.mesh_node_off) - 1):
        lo, hi = s.mesh_node_off[m], s.mesh_node_off[m + 1]

        def leaves(g):
            if s.nodes[g, 2] == 0:
                return [s.tris[g, i] for i in range(s.ntris[g])]
            out = []
            for c in range(s.nodes[g, 1]):
                out += leaves(s.nodes[g, 0] + c)
            return out

        for g in range(lo, hi):
            if s.nodes[g, 2]:
                assert s.nodes[g, 1] == 8 and s.ntris[g] == 8
                for i in range(8):
                    child = s.nodes[g, 0] + i
                    for t in leaves(child):
                        for v in range(3):
                            d = point_tri_dist(t[3 * v:3 * v + 3], s.tris[g, i])
                            assert d <= s.eps[g, i] + 1e-9
                            assert d >= s.inner_eps[g, i] - 1e-9
        # the leaves hold real mesh triangles: positive area, each inside its
        # parent surrogate's eps band (checked above), none repeated in this
        # mesh's tree (copies arise only for degenerate groupings)
        leaf = [tuple(s.tris[g, i]) for g in range(lo, hi) if s.nodes[g, 2] == 0 for i in range(s.ntris[g])]
        assert len(leaf) == len(set(leaf)) > 0
        for t in leaf:
            a, b, c = np.array(t[0:3]), np.array(t[3:6]), np.array(t[6:9])
            assert np.linalg.norm(np.cross(b - a, c - a)) > 0.0


def test_tree_build_deterministic_and_consumes_rng():
    s = D.make_scene(1)
    lo = s.mesh_node_off[1]
    V = s.tris[lo + 1:lo + 9].reshape(-1, 9)
    # rebuild the cube tree from its 12 triangles with the (42, 54) stream
    tris = np.concatenate([s.tris[g, :s.ntris[g]] for g in range(lo + 1, lo + 9)])
    Vx = tris.reshape(-1, 3)
    F = np.arange(len(Vx)).reshape(-1, 3)
    a = D.build_tree(Vx, F)
    b = D.build_tree(Vx, F)
    for x, y in zip(a[:5], b[:5]):
        assert np.array_equal(x, y)
    assert a[5] != D.pcg32_seed(42, 54)
    assert a[0][0].tolist()[1:] == [8, 1, 0]
    assert V.shape[1] == 9


def test_pcg32_matches_published_stream():
    # O'Neill's pcg32 demo (pcg32-demo.c) seeded (42, 54) prints 0xa15c02b7 first.
    s = D.pcg32_seed(42, 54)
    state, inc = s
    mask = (1 << 64) - 1
    old = state
    xorshifted = (((old >> 18) ^ old) >> 27) & 0xffffffff
    rot = old >> 59
    out = ((xorshifted >> rot) | (xorshifted << ((-rot) & 31))) & 0xffffffff
    assert out == 0xa15c02b7
    assert (state * 6364136223846793005 + inc) & mask != state


def test_invalid_inputs_rejected_on_host():
    with pytest.raises(D.D2GError):
        D.make_scene(4)
    with pytest.raises(D.D2GError):
        D.build_tree(np.zeros((2, 3)), np.zeros((1, 3), np.int32))


def test_broad_phase_matches_oracle():
    from oracle import oracle as O
    for cfg, kw in [(1, {}), (2, dict(nx=4, ny=4, nz=2)), (1, dict(spacing=1.12, speed_sigma=3.0, seed=3))]:
        s = D.make_scene(cfg, **kw)
        for i in range(s.n_bodies):  # the outer step projects futures before the broad phase
            s.fut[i] = O.state_extrapolate(s.cur[i], s.last_dt[i], s.inv_inertia[i])
        ref = O.World(s.copy(), s.opt_dt).broad_phase()
        got = D.broad_phase(s)
        assert np.array_equal(got, ref), (cfg, len(got), len(ref))
        assert len(got) > 0


def test_tuning_file_loader(tmp_path):
    # the autotuner's output format: settings by name; no file means defaults
    from delta2_gb300 import autotune

    assert autotune.load(str(tmp_path / "absent.json")) == {}
    f = tmp_path / "t.json"
    f.write_text('{"gpu": "x", "settings": {"ee_first_iters": 3, "grid_min_parts": 256}}')
    got = autotune.load(str(f))
    assert got == {"ee_first_iters": 3, "grid_min_parts": 256}
    assert set(got) <= set(D.TUNE_NAMES)


def test_grid_threshold_choice():
    # the fastest total wins; within 1% of it, the smallest threshold (the
    # piles the tuner times stop at 401 parts, larger clusters gain from the grid)
    from delta2_gb300 import autotune

    assert autotune.choose_grid_threshold({64: 135.9, 512: 129.08, 1000000: 129.07}) == 512
    assert autotune.choose_grid_threshold({64: 100.0, 512: 120.0, 1000000: 130.0}) == 64
    assert autotune.choose_grid_threshold({64: 140.0, 512: 131.0, 1000000: 129.0}) == 1000000


def test_open_box_scene_and_parallel_trees():
    # the noisy-icosphere scene: one static open box, then one mesh and tree per
    # body built on all host cores from per-mesh streams (same trees every time)
    a = D.make_scene(5, nx=2, ny=1, nz=1)
    b = D.make_scene(5, nx=2, ny=1, nz=1)
    assert a.n_bodies == 3 and a.is_static.tolist() == [1, 0, 0]
    assert len(a.mesh_node_off) == 4  # box + one mesh per body
    assert np.array_equal(a.tris, b.tris) and np.array_equal(a.nodes, b.nodes)
    lo, hi = a.local_aabb[0, :3], a.local_aabb[0, 3:]
    assert np.allclose(hi[:2] - lo[:2], 40.0) and np.isclose(hi[2] - lo[2], 20.0)


def test_tree_file_round_trip(tmp_path):
    # the versioned tree file stores the flattened trees exactly
    s = D.make_scene(3)
    path = tmp_path / "trees.bin"
    D.save_trees(s, path)
    t = D.load_trees(path)
    for f in ["mesh_node_off", "nodes", "ntris", "tris", "eps", "inner_eps"]:
        assert np.array_equal(np.asarray(t[f]), np.asarray(getattr(s, f))), f


def test_scene_tree_file_builds_then_loads(tmp_path):
    # the first call builds the trees and writes the file, the second loads
    # it; both scenes are the same, field by field
    path = str(tmp_path / "c5.trees")
    a = D.make_scene(5, nx=2, ny=2, nz=1, tree_file=path)
    assert os.path.exists(path)
    b = D.make_scene(5, nx=2, ny=2, nz=1, tree_file=path)
    c = D.make_scene(5, nx=2, ny=2, nz=1)
    for f in ["mesh_node_off", "nodes", "ntris", "tris", "eps", "inner_eps", "mesh", "cur", "mass"]:
        assert np.array_equal(getattr(a, f), getattr(b, f)), f
        assert np.array_equal(getattr(a, f), getattr(c, f)), f


def test_tree_file_rejects_corruption_and_other_meshes(tmp_path):
    path = tmp_path / "t.bin"
    D.save_trees(D.make_scene(1, nx=2, ny=1, nz=1), path)
    raw = bytearray(path.read_bytes())
    raw[-3] ^= 0x40  # a payload byte
    bad = tmp_path / "bad.bin"
    bad.write_bytes(bytes(raw))
    with pytest.raises(D.D2GError, match="checksum"):
        D.load_trees(bad)
    short = tmp_path / "short.bin"
    short.write_bytes(path.read_bytes()[:100])
    with pytest.raises(D.D2GError):
        D.load_trees(short)
    # trees of the 2-cube scene do not fit the mixed scene's meshes
    with pytest.raises(D.D2GError):
        D.make_scene(3, tree_file=str(path))


CUBE_V = [[1, 1, 1], [1, 1, -1], [1, -1, 1], [1, -1, -1], [-1, 1, 1], [-1, 1, -1], [-1, -1, 1], [-1, -1, -1]]
CUBE_F = [[0, 2, 1], [1, 2, 3], [2, 6, 3], [3, 6, 7], [4, 5, 6], [5, 7, 6], [4, 0, 1], [4, 1, 5], [0, 4, 6],
          [0, 6, 2], [3, 7, 1], [7, 5, 1]]


def _write_obj(path, V, F, quads=()):
    with open(path, "w") as f:
        f.write("# test mesh\no m\n")
        for v in V:
            f.write("v %r %r %r\n" % tuple(v))
        f.write("vt 0 0\nvn 0 0 1\n")
        for t in F:
            f.write("f %d/1/1 %d//1 %d\n" % tuple(k + 1 for k in t))
        for q in quads:
            f.write("f " + " ".join(str(k - len(V)) for k in q) + "\n")  # negative (relative) indices


def test_obj_loader(tmp_path):
    p = tmp_path / "m.obj"
    _write_obj(p, [[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]], [[0, 1, 2]], quads=[[0, 1, 2, 3]])
    V, F = D.load_obj(p)
    assert V.shape == (4, 3) and F.tolist() == [[0, 1, 2], [0, 1, 2], [0, 2, 3]]


def test_scene_builder_reproduces_the_cube_scene(tmp_path):
    # the 1-cube configuration rebuilt from OBJ files: ground plane (surface
    # mass model) and a unit cube (volume model), same bodies, same trees
    ref = D.make_scene(1, nx=1, ny=1, nz=1)
    _write_obj(tmp_path / "cube.obj", [[0.5 * c for c in v] for v in CUBE_V], CUBE_F)
    _write_obj(tmp_path / "plane.obj", [[50, 50, 0], [50, -50, 0], [-50, 50, 0], [-50, -50, 0]], [[0, 2, 1], [1, 2, 3]])
    b = D.SceneBuilder(dt=ref.opt_dt, gravity_z=ref.gravity_z)
    plane, pcom = b.add_mesh(*D.load_obj(tmp_path / "plane.obj"), surface=True)
    cube, ccom = b.add_mesh(*D.load_obj(tmp_path / "cube.obj"))
    assert np.allclose(pcom, 0) and np.allclose(ccom, 0)
    b.add_body(plane, static=True, density=1000.0, geo_eps=ref.geo_eps[0], mu=ref.mu[0])
    b.add_body(cube, position=ref.cur[1, 8:11], quaternion=ref.cur[1, 1:5], velocity=ref.cur[1, 11:14],
               density=1000.0, geo_eps=ref.geo_eps[1], mu=ref.mu[1])
    got = b.finish()
    for f in ["mesh_node_off", "nodes", "ntris", "tris", "eps", "inner_eps", "mesh", "is_static", "geo_eps", "mu",
              "mass", "inv_inertia", "last", "cur", "fut", "last_dt", "bounding_radius", "local_aabb"]:
        assert np.array_equal(getattr(got, f), getattr(ref, f)), f


def test_native_obj_reader_matches_python_reader(tmp_path):
    # d2g_scene_add_obj (the library's C++ reader) and load_obj + add_mesh
    # give the same scene, array for array: triangles in v/vt/vn forms,
    # quads and pentagons with negative references (fans), comments, CRLF
    # line ends, records that are ignored
    pent = tmp_path / "pent.obj"
    with open(pent, "w", newline="") as f:
        f.write("# prism with pentagonal caps\r\nmtllib none.mtl\r\n")
        import math
        for z in (0.0, 0.7):
            for k in range(5):
                a = 2 * math.pi * k / 5
                f.write("v %r %r %r\r\n" % (math.cos(a), math.sin(a), z))
        f.write("vt 0 0\r\nvn 0 0 1\r\ns off\r\n")
        f.write("f 5 4 3 2 1\r\n")              # bottom cap, outward (-z)
        f.write("f -5 -4 -3 -2 -1\r\n")         # top cap: vertices 6..10
        for k in range(5):
            a, b = k + 1, (k + 1) % 5 + 1
            f.write("f %d/1/1 %d//1 %d/1 %d\r\n" % (a, b, b + 5, a + 5))
    _write_obj(tmp_path / "cube.obj", [[0.5 * c for c in v] for v in CUBE_V], CUBE_F)
    scenes = []
    for native in (False, True):
        b = D.SceneBuilder(dt=0.005)
        ids = []
        for name, surface in (("cube.obj", False), ("pent.obj", False), ("cube.obj", True)):
            if native:
                ids.append(b.add_obj(tmp_path / name, surface=surface))
            else:
                ids.append(b.add_mesh(*D.load_obj(tmp_path / name), surface=surface))
        for k, (mid, com) in enumerate(ids):
            b.add_body(mid, position=(3.0 * k, 0.0, 1.0 + k), static=(k == 2))
        scenes.append((b.finish(), ids))
    (a, ia), (n, inat) = scenes
    for (m0, c0), (m1, c1) in zip(ia, inat):
        assert m0 == m1 and np.array_equal(c0, c1)
    for f in ["mesh_node_off", "nodes", "ntris", "tris", "eps", "inner_eps", "mesh", "is_static", "mass",
              "inv_inertia", "cur", "bounding_radius", "local_aabb"]:
        assert np.array_equal(getattr(a, f), getattr(n, f)), f
    assert len(D.load_obj(pent)[1]) == 2 * 3 + 5 * 2


def test_native_obj_reader_rejects_bad_files(tmp_path):
    b = D.SceneBuilder()
    with pytest.raises(D.D2GError, match="cannot open"):
        b.add_obj(tmp_path / "missing.obj")
    bad = tmp_path / "bad.obj"
    bad.write_text("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 7\n")
    with pytest.raises(D.D2GError, match="out of range"):
        b.add_obj(bad)
    bad.write_text("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 -4\n")
    with pytest.raises(D.D2GError, match="out of range"):
        b.add_obj(bad)
    bad.write_text("v 0 0 x\n")
    with pytest.raises(D.D2GError, match="bad vertex"):
        b.add_obj(bad)
    bad.write_text("v 0 0 0\nf 1 a 1\n")
    with pytest.raises(D.D2GError, match="bad face"):
        b.add_obj(bad)


def test_scene_builder_rejects_invalid_meshes():
    b = D.SceneBuilder()
    with pytest.raises(D.D2GError, match="no volume"):
        b.add_mesh([[0, 0, 0], [1, 0, 0], [0, 1, 0]], [[0, 1, 2]])  # open surface
    with pytest.raises(D.D2GError, match="out of range"):
        b.add_mesh([[0, 0, 0], [1, 0, 0], [0, 1, 0]], [[0, 1, 5]])
    with pytest.raises(D.D2GError):
        b.finish()  # no body
