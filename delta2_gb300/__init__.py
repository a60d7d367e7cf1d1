"""delta2_gb300 — GB300 (sm_103a) contact hot path of the Delta2 rigid-body simulator.

Python mirror of the C ABI in ``include/d2g.h``.  The names follow the
reference's functions (``compare_trees_full`` = ``compareTreesFull``,
``compare_trees_full_continuous`` = ``compareTreesFullContinuous``); the
compute always runs in the CUDA library ``_lib/libd2g.so``.  There is no CPU
fallback: a missing library or GPU raises.
"""
import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_lib", "libd2g.so")
_lib = None

STATE_LEN = 14
CONTACT_LEN = 14

I32P = C.POINTER(C.c_int32)
F64P = C.POINTER(C.c_double)
F32P = C.POINTER(C.c_float)
U8P = C.POINTER(C.c_uint8)
I64P = C.POINTER(C.c_int64)
U64P = C.POINTER(C.c_uint64)


class D2GError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"d2g error {code}: {msg}")
        self.code = code


class CapacityError(D2GError):
    pass


class SolveFailed(D2GError):
    pass


class Trees(C.Structure):
    _fields_ = [("n_meshes", C.c_int32), ("mesh_node_off", I32P), ("nodes", I32P), ("ntris", I32P),
                ("tris", F64P), ("eps", F64P), ("inner_eps", F64P)]


class Bodies(C.Structure):
    _fields_ = [("n", C.c_int32), ("mesh", I32P), ("is_static", U8P), ("geo_eps", F64P), ("mu", F64P),
                ("mass", F64P), ("inv_inertia", F64P), ("last", F64P), ("cur", F64P), ("fut", F64P),
                ("last_dt", F64P), ("sleep_steps", I32P), ("sleeping", U8P), ("bounding_radius", F64P)]


class DeviceScene(C.Structure):
    _fields_ = [("n_meshes", C.c_int32), ("n_nodes", C.c_int32), ("mesh_node_off", C.c_void_p),
                ("nodes", C.c_void_p), ("ntris", C.c_void_p), ("tris", C.c_void_p), ("eps", C.c_void_p),
                ("inner_eps", C.c_void_p), ("n_bodies", C.c_int32), ("mesh", C.c_void_p), ("fut", C.c_void_p),
                ("geo_eps", C.c_void_p)]


NOALLOC_MAX_PAIRS = 2048
NOALLOC_MAX_NODE_PAIRS = 2048
NOALLOC_MAX_CONTACTS = 32768


def compare_trees_full_noalloc(device_scene, d_pairs, n_pairs, d_contacts, capacity, d_offsets, stream=0):
    """Allocation-free compareTreesFull over device buffers (see include/d2g.h).

    ``device_scene`` is a DeviceScene of device pointers; the other pointers
    are device addresses (ints).  Returns the number of contacts."""
    n = C.c_int32()
    _check(lib().d2g_compare_trees_full_noalloc(C.byref(device_scene), C.c_void_p(d_pairs), int(n_pairs),
                                                C.c_void_p(d_contacts), int(capacity), C.c_void_p(d_offsets),
                                                C.byref(n), C.c_void_p(stream)))
    return n.value


class SceneOpts(C.Structure):
    _fields_ = [("config", C.c_int32), ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
                ("spacing", C.c_double), ("speed_sigma", C.c_double), ("seed", C.c_uint64), ("dt", C.c_float),
                ("gravity_z", C.c_double), ("mu", C.c_double), ("hull_points", C.c_int32), ("count", C.c_int32),
                ("tree_file", C.c_char_p)]


def library_path():
    return _LIB_PATH


def lib():
    """Load the CUDA library (it must have been built with ``delta2_gb300.build``)."""
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            raise RuntimeError(f"{_LIB_PATH} is missing: build it with `python -m delta2_gb300.build` "
                               "(or __graft_entry__.build()); there is no CPU fallback")
        L = C.CDLL(_LIB_PATH)
        L.d2g_last_error.restype = C.c_char_p
        L.d2g_version.restype = C.c_char_p
        L.d2g_ctx_destroy.restype = None
        L.d2g_scene_free.restype = None
        L.d2g_tree_file_free.restype = None
        _lib = L
    return _lib


def _check(rc):
    if rc == 0:
        return rc
    msg = lib().d2g_last_error().decode(errors="replace")
    if rc == 2:
        raise CapacityError(rc, msg)
    if rc == 1:
        raise SolveFailed(rc, msg)
    raise D2GError(rc, msg)


def _p(a, t):
    return a.ctypes.data_as(t)


WORLD_STATS = ["ccd_pairs", "ccd_contacts", "np_pairs", "np_contacts", "solves", "failures", "normal_iters",
               "friction_iters", "ccd_node_pairs", "ccd_tri_pairs", "ccd_leaf_pairs", "np_node_pairs", "np_tri_pairs"]


WORLD_PHASES = ["project", "broad_phase", "clusters", "select", "sleeping", "narrowphase", "filter", "solve",
                "bookkeeping", "reserved"]


class Scene:
    """Flattened trees and bodies (numpy arrays in the C ABI layout)."""

    FIELDS_TREE = ["mesh_node_off", "nodes", "ntris", "tris", "eps", "inner_eps"]
    FIELDS_BODY = ["mesh", "is_static", "geo_eps", "mu", "mass", "inv_inertia", "last", "cur", "fut", "last_dt",
                   "sleep_steps", "sleeping", "bounding_radius"]

    def copy(self):
        s = Scene()
        for k, v in self.__dict__.items():
            setattr(s, k, v.copy() if isinstance(v, np.ndarray) else v)
        return s

    def trees_struct(self):
        self.mesh_node_off = np.ascontiguousarray(self.mesh_node_off, dtype=np.int32)
        self.nodes = np.ascontiguousarray(self.nodes, dtype=np.int32)
        self.ntris = np.ascontiguousarray(self.ntris, dtype=np.int32)
        for k in ["tris", "eps", "inner_eps"]:
            setattr(self, k, np.ascontiguousarray(getattr(self, k), dtype=np.float64))
        return Trees(len(self.mesh_node_off) - 1, _p(self.mesh_node_off, I32P), _p(self.nodes, I32P),
                     _p(self.ntris, I32P), _p(self.tris, F64P), _p(self.eps, F64P), _p(self.inner_eps, F64P))

    def bodies_struct(self):
        for k, dt in [("mesh", np.int32), ("is_static", np.uint8), ("sleep_steps", np.int32),
                      ("sleeping", np.uint8)]:
            setattr(self, k, np.ascontiguousarray(getattr(self, k), dtype=dt))
        for k in ["geo_eps", "mu", "mass", "inv_inertia", "last", "cur", "fut", "last_dt", "bounding_radius"]:
            setattr(self, k, np.ascontiguousarray(getattr(self, k), dtype=np.float64))
        return Bodies(len(self.mesh), _p(self.mesh, I32P), _p(self.is_static, U8P), _p(self.geo_eps, F64P),
                      _p(self.mu, F64P), _p(self.mass, F64P), _p(self.inv_inertia, F64P), _p(self.last, F64P),
                      _p(self.cur, F64P), _p(self.fut, F64P), _p(self.last_dt, F64P), _p(self.sleep_steps, I32P),
                      _p(self.sleeping, U8P), _p(self.bounding_radius, F64P))

    @property
    def n_bodies(self):
        return len(self.mesh)


def concat_scenes(scenes):
    """Independent scenes as one: trees and bodies concatenated (mesh ids and
    the inner nodes' first-child indices shifted); returns the scene and the
    scene index of every body.  Positions are left as they are, so every scene
    computes exactly as it would alone."""
    out = Scene()
    node_base, mesh_base = 0, 0
    offs, nodes, scene_of = [0], [], []
    for k, sc in enumerate(scenes):
        nd = np.array(sc.nodes, dtype=np.int32).copy()
        inner = nd[:, 2] != 0
        nd[inner, 0] += node_base
        nodes.append(nd)
        offs += [node_base + int(x) for x in sc.mesh_node_off[1:]]
        node_base += len(nd)
        scene_of.append(np.full(sc.n_bodies, k, np.int32))
    out.mesh_node_off = np.array(offs, np.int32)
    out.nodes = np.concatenate(nodes)
    for f in ["ntris", "tris", "eps", "inner_eps"]:
        setattr(out, f, np.concatenate([getattr(sc, f) for sc in scenes]))
    meshes = []
    for sc in scenes:
        meshes.append(np.asarray(sc.mesh, np.int32) + mesh_base)
        mesh_base += len(sc.mesh_node_off) - 1
    out.mesh = np.concatenate(meshes)
    for f in Scene.FIELDS_BODY:
        if f != "mesh":
            setattr(out, f, np.concatenate([getattr(sc, f) for sc in scenes]))
    out.local_aabb = np.concatenate([sc.local_aabb for sc in scenes])
    out.opt_dt = scenes[0].opt_dt
    out.gravity_z = scenes[0].gravity_z
    return out, np.concatenate(scene_of)


def split_bodies(batch, scene_of, k):
    """Body arrays of scene k out of a batched scene (a view for comparisons)."""
    sel = scene_of == k
    out = Scene()
    for f in Scene.FIELDS_BODY:
        setattr(out, f, getattr(batch, f)[sel])
    return out


def _trees_struct(scene):
    t = Trees()
    t.n_meshes = len(scene.mesh_node_off) - 1
    scene._tree_keep = [np.ascontiguousarray(scene.mesh_node_off, dtype=np.int32),
                        np.ascontiguousarray(scene.nodes, dtype=np.int32),
                        np.ascontiguousarray(scene.ntris, dtype=np.int32),
                        np.ascontiguousarray(scene.tris, dtype=np.float64),
                        np.ascontiguousarray(scene.eps, dtype=np.float64),
                        np.ascontiguousarray(scene.inner_eps, dtype=np.float64)]
    k = scene._tree_keep
    t.mesh_node_off, t.nodes, t.ntris = _p(k[0], I32P), _p(k[1], I32P), _p(k[2], I32P)
    t.tris, t.eps, t.inner_eps = _p(k[3], F64P), _p(k[4], F64P), _p(k[5], F64P)
    return t


def save_trees(scene, path):
    """Write the scene's trees to a tree file (d2g_trees_save)."""
    _check(lib().d2g_trees_save(C.byref(_trees_struct(scene)), str(path).encode()))


def load_trees(path):
    """Arrays of a tree file: mesh_node_off, nodes, ntris, tris, eps, inner_eps."""
    L = lib()
    h = C.c_void_p()
    _check(L.d2g_trees_load(str(path).encode(), C.byref(h)))
    try:
        t = Trees()
        _check(L.d2g_tree_file_view(h, C.byref(t)))
        M = t.n_meshes
        off = np.ctypeslib.as_array(t.mesh_node_off, (M + 1,)).copy()
        N = int(off[-1])
        return {"mesh_node_off": off,
                "nodes": np.ctypeslib.as_array(t.nodes, (N, 4)).copy() if N else np.zeros((0, 4), np.int32),
                "ntris": np.ctypeslib.as_array(t.ntris, (N,)).copy() if N else np.zeros(0, np.int32),
                "tris": np.ctypeslib.as_array(t.tris, (N, 8, 9)).copy() if N else np.zeros((0, 8, 9)),
                "eps": np.ctypeslib.as_array(t.eps, (N, 8)).copy() if N else np.zeros((0, 8)),
                "inner_eps": np.ctypeslib.as_array(t.inner_eps, (N, 8)).copy() if N else np.zeros((0, 8))}
    finally:
        L.d2g_tree_file_free(h)


def make_batch(n_scenes=256, seed=0, min_bodies=8, max_bodies=512, dt=0.0):
    """The batched configuration: n_scenes independent mixed scenes (cubes,
    64-point hulls and subdivision-2 icospheres in turn), each on its own
    ground plane, with body counts drawn uniformly from [min_bodies,
    max_bodies] by a seeded generator.  Returns (scene, scene_of_body,
    per-scene list)."""
    rng = np.random.default_rng(0xD2 + 3 + seed)
    counts = rng.integers(min_bodies, max_bodies + 1, size=n_scenes)
    scenes = []
    for k, cnt in enumerate(counts):
        nz = (int(cnt) + 63) // 64
        scenes.append(make_scene(3, nx=8, ny=8, nz=nz, count=int(cnt), seed=seed * 100003 + k, dt=dt))
    batch, scene_of = concat_scenes(scenes)
    return batch, scene_of, scenes


def make_scene(config=2, nx=0, ny=0, nz=0, spacing=0.0, speed_sigma=-1.0, seed=0, dt=0.0, gravity_z=-9.8, mu=0.0,
               hull_points=64, count=0, tree_file=None):
    """Synthetic scene of a benchmark configuration (host set-up, no GPU).
    With tree_file, the trees are loaded from that file when it exists, else
    built and saved there."""
    L = lib()
    o = SceneOpts(config, nx, ny, nz, spacing, speed_sigma, seed, dt, gravity_z, mu, hull_points, count,
                  tree_file.encode() if tree_file else None)
    h = C.c_void_p()
    _check(L.d2g_scene_make(C.byref(o), C.byref(h)))
    try:
        return _scene_view(L, h, config)
    finally:
        L.d2g_scene_free(h)


def _scene_view(L, h, config):
    """Scene object with copies of a d2g_scene handle's arrays."""
    if True:
        t = Trees()
        b = Bodies()
        aabb = F32P()
        odt = C.c_float()
        gz = C.c_double()
        _check(L.d2g_scene_view(h, C.byref(t), C.byref(b), C.byref(aabb), C.byref(odt), C.byref(gz)))
        s = Scene()
        M = t.n_meshes
        s.mesh_node_off = np.ctypeslib.as_array(t.mesh_node_off, (M + 1,)).copy()
        N = int(s.mesh_node_off[-1])
        s.nodes = np.ctypeslib.as_array(t.nodes, (N, 4)).copy()
        s.ntris = np.ctypeslib.as_array(t.ntris, (N,)).copy()
        s.tris = np.ctypeslib.as_array(t.tris, (N, 8, 9)).copy()
        s.eps = np.ctypeslib.as_array(t.eps, (N, 8)).copy()
        s.inner_eps = np.ctypeslib.as_array(t.inner_eps, (N, 8)).copy()
        n = b.n
        s.mesh = np.ctypeslib.as_array(b.mesh, (n,)).copy()
        s.is_static = np.ctypeslib.as_array(b.is_static, (n,)).copy()
        s.geo_eps = np.ctypeslib.as_array(b.geo_eps, (n,)).copy()
        s.mu = np.ctypeslib.as_array(b.mu, (n,)).copy()
        s.mass = np.ctypeslib.as_array(b.mass, (n,)).copy()
        s.inv_inertia = np.ctypeslib.as_array(b.inv_inertia, (n, 9)).copy()
        for k in ["last", "cur", "fut"]:
            setattr(s, k, np.ctypeslib.as_array(getattr(b, k), (n, STATE_LEN)).copy())
        s.last_dt = np.ctypeslib.as_array(b.last_dt, (n,)).copy()
        s.sleep_steps = np.ctypeslib.as_array(b.sleep_steps, (n,)).copy()
        s.sleeping = np.ctypeslib.as_array(b.sleeping, (n,)).copy()
        s.bounding_radius = np.ctypeslib.as_array(b.bounding_radius, (n,)).copy()
        s.local_aabb = np.ctypeslib.as_array(aabb, (n, 6)).copy()
        s.opt_dt = float(odt.value)
        s.gravity_z = float(gz.value)
        s.config = config
        return s


def load_obj(path):
    """Vertices [n][3] and triangles [m][3] (0-based) of a Wavefront OBJ file
    (v and f records; polygons are split into fans; v/vt/vn index forms and
    negative indices are read; everything else is ignored), as the
    reference's mesh import does (model/mesh.cpp:9-21, igl::readOBJ)."""
    V, F = [], []
    with open(path) as f:
        for line in f:
            parts = line.split()
            if not parts:
                continue
            if parts[0] == "v" and len(parts) >= 4:
                V.append([float(x) for x in parts[1:4]])
            elif parts[0] == "f" and len(parts) >= 4:
                idx = []
                for tok in parts[1:]:
                    k = int(tok.split("/")[0])
                    idx.append(k - 1 if k > 0 else len(V) + k)
                for j in range(1, len(idx) - 1):
                    F.append([idx[0], idx[j], idx[j + 1]])
    V = np.asarray(V, dtype=np.float64).reshape(-1, 3)
    F = np.asarray(F, dtype=np.int32).reshape(-1, 3)
    if len(F) and (F.min() < 0 or F.max() >= len(V)):
        raise ValueError(f"{path}: face index out of range")
    return V, F


class SceneBuilder:
    """A scene of the caller's meshes and bodies (d2g_scene_create):

        b = SceneBuilder(dt=1/240)
        box, com = b.add_mesh(*load_obj("box.obj"), surface=True)
        b.add_body(box, position=com, static=True)
        rock, _ = b.add_mesh(V, F)
        b.add_body(rock, position=(0, 0, 2), velocity=(0, 0, -1))
        scene = b.finish()

    Meshes are centred at their centre of mass (add_mesh returns it)."""

    def __init__(self, dt=0.01, gravity_z=-9.8):
        self.h = C.c_void_p()
        _check(lib().d2g_scene_create(C.c_float(dt), C.c_double(gravity_z), C.byref(self.h)))

    def add_mesh(self, V, F, surface=False):
        V = np.ascontiguousarray(V, dtype=np.float64).reshape(-1, 3)
        F = np.ascontiguousarray(F, dtype=np.int32).reshape(-1, 3)
        com = np.zeros(3)
        mid = C.c_int32()
        _check(lib().d2g_scene_add_mesh(self.h, _p(V, F64P), len(V), _p(F, I32P), len(F), int(bool(surface)),
                                        _p(com, F64P), C.byref(mid)))
        return mid.value, com

    def add_obj(self, path, surface=False):
        """add_mesh of a Wavefront OBJ file read by the library's own reader
        (d2g_scene_add_obj; the same rules as load_obj)."""
        com = np.zeros(3)
        mid = C.c_int32()
        _check(lib().d2g_scene_add_obj(self.h, os.fsencode(str(path)), int(bool(surface)), _p(com, F64P),
                                       C.byref(mid)))
        return mid.value, com

    def add_body(self, mesh_id, position=(0, 0, 0), quaternion=(1, 0, 0, 0), velocity=(0, 0, 0), static=False,
                 density=1000.0, geo_eps=0.01, mu=0.5):
        x = np.ascontiguousarray(position, dtype=np.float64)
        q = np.ascontiguousarray(quaternion, dtype=np.float64)
        v = np.ascontiguousarray(velocity, dtype=np.float64)
        _check(lib().d2g_scene_add_body(self.h, int(mesh_id), int(bool(static)), C.c_double(density),
                                        C.c_double(geo_eps), C.c_double(mu), _p(x, F64P), _p(q, F64P),
                                        _p(v, F64P)))

    def finish(self):
        L = lib()
        _check(L.d2g_scene_finish(self.h))
        try:
            return _scene_view(L, self.h, 0)
        finally:
            L.d2g_scene_free(self.h)
            self.h = None


def build_tree(V, F, rng_state=None):
    """Surrogate tree of one mesh (model/surrogate_tree.cpp:39-112).

    Returns (nodes, ntris, tris, eps, inner_eps, rng_state); child indices are
    local to the mesh.  ``rng_state`` is the PCG32 (state, inc) pair; None =
    the reference's Options stream seeded (42, 54)."""
    L = lib()
    V = np.ascontiguousarray(V, dtype=np.float64).reshape(-1, 3)
    F = np.ascontiguousarray(F, dtype=np.int32).reshape(-1, 3)
    if rng_state is None:
        rng_state = pcg32_seed(42, 54)
    rng = np.array(rng_state, dtype=np.uint64)
    n = C.c_int32()
    _check(L.d2g_tree_build(_p(V, F64P), len(V), _p(F, I32P), len(F), _p(rng, U64P), C.byref(n), None, None, None,
                            None, None, 0))
    N = n.value
    nodes = np.zeros((N, 4), np.int32)
    ntris = np.zeros(N, np.int32)
    tris = np.zeros((N, 8, 9))
    eps = np.zeros((N, 8))
    ieps = np.zeros((N, 8))
    _check(L.d2g_tree_build(_p(V, F64P), len(V), _p(F, I32P), len(F), _p(rng, U64P), C.byref(n), _p(nodes, I32P),
                            _p(ntris, I32P), _p(tris, F64P), _p(eps, F64P), _p(ieps, F64P), N))
    return nodes, ntris, tris, eps, ieps, (int(rng[0]), int(rng[1]))


def broad_phase(scene):
    """Candidate body pairs (i < j) of a scene (host broad phase, no GPU)."""
    L = lib()
    b = scene.bodies_struct()
    aabb = np.ascontiguousarray(scene.local_aabb, dtype=np.float32)
    n = C.c_int32()
    _check(L.d2g_broad_phase(C.byref(b), _p(aabb, F32P), None, 0, C.byref(n)))
    out = np.zeros((max(n.value, 1), 2), np.int32)
    _check(L.d2g_broad_phase(C.byref(b), _p(aabb, F32P), _p(out, I32P), n.value, C.byref(n)))
    return out[:n.value].copy()


PROF_SOUP_FILTER, PROF_SOUP_CCD, PROF_CONN, PROF_NP, PROF_SOLVE = range(5)
CCD_STATS = ["ee_tests_cut", "newton_iters_saved", "pairs_predicted_clear", "pairs_certified", "pairs_missed",
             "pairs_seen", "node_pairs_witnessed", "witnesses_written"]
(TUNE_EE_FIRST_ITERS, TUNE_GRID_MIN_PARTS, TUNE_SOLVE_LANES, TUNE_SPIN_LIMIT, TUNE_GRID_CONTACTS,
 TUNE_SOLVE_CLUSTER) = range(6)
TUNE_NAMES = {"ee_first_iters": TUNE_EE_FIRST_ITERS, "grid_min_parts": TUNE_GRID_MIN_PARTS,
              "solve_lanes": TUNE_SOLVE_LANES, "spin_limit": TUNE_SPIN_LIMIT, "grid_contacts": TUNE_GRID_CONTACTS,
              "solve_cluster": TUNE_SOLVE_CLUSTER}
TUNE_NAMES_INV = {v: k for k, v in TUNE_NAMES.items()}


def pcg32_seed(initstate, initseq):
    """PCG32 srandom: returns (state, inc)."""
    mask = (1 << 64) - 1
    inc = ((initseq << 1) | 1) & mask
    state = 0
    state = (state * 6364136223846793005 + inc) & mask
    state = (state + initstate) & mask
    state = (state * 6364136223846793005 + inc) & mask
    return state, inc


class Context:
    """A CUDA context of the library: trees and bodies resident in HBM."""

    def __init__(self, device=0):
        L = lib()
        h = C.c_void_p()
        _check(L.d2g_ctx_create(int(device), C.byref(h)))
        self.h = h
        self.scene = None

    def close(self):
        if getattr(self, "h", None):
            lib().d2g_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def stream(self):
        s = C.c_void_p()
        _check(lib().d2g_ctx_stream(self.h, C.byref(s)))
        return s.value

    def sync(self):
        _check(lib().d2g_ctx_sync(self.h))

    def set_scene(self, scene):
        self.scene = scene
        self._t = scene.trees_struct()
        _check(lib().d2g_ctx_set_trees(self.h, C.byref(self._t)))
        self.set_bodies(scene)

    def set_bodies(self, scene):
        self._b = scene.bodies_struct()
        _check(lib().d2g_ctx_set_bodies(self.h, C.byref(self._b)))

    def set_fp32_bounds(self, enable):
        """FP32 candidate bounds before the FP64 primitive tests (default on;
        results are identical either way)."""
        _check(lib().d2g_ctx_set_fp32_bounds(self.h, int(bool(enable))))

    def set_ccd_certificates(self, enable):
        """Conservative-advancement cut-off of edge-edge CCD tests (default on;
        results are identical either way)."""
        _check(lib().d2g_ctx_set_ccd_certificates(self.h, int(bool(enable))))

    def mass_properties(self, meshes, surface=None, thickness=0.01):
        """Mass properties of meshes [(V, F), ...] on the device
        (d2g_mass_properties) -> [n, 22]: volume, centre of mass, unit-density
        inertia tensor (row major), its inverse."""
        Vs = [np.ascontiguousarray(V, dtype=np.float64).reshape(-1, 3) for V, _ in meshes]
        Fs = [np.ascontiguousarray(F, dtype=np.int32).reshape(-1, 3) for _, F in meshes]
        voff = np.concatenate([[0], np.cumsum([len(v) for v in Vs])]).astype(np.int32)
        foff = np.concatenate([[0], np.cumsum([len(f) for f in Fs])]).astype(np.int32)
        V = np.ascontiguousarray(np.concatenate(Vs) if Vs else np.zeros((0, 3)))
        F = np.ascontiguousarray(np.concatenate(Fs) if Fs else np.zeros((0, 3), np.int32), dtype=np.int32)
        surf = np.ascontiguousarray(surface if surface is not None else np.zeros(len(meshes)), dtype=np.uint8)
        out = np.zeros((max(1, len(meshes)), 22))
        _check(lib().d2g_mass_properties(self.h, _p(V, F64P), len(V), _p(F, I32P), len(F), _p(voff, I32P),
                                         _p(foff, I32P), _p(surf, U8P), len(meshes), C.c_double(thickness),
                                         _p(out, F64P)))
        return out[:len(meshes)]

    def ccd_features(self, pairs, max_time):
        """The proposal's features [n, 20] of CCD pair queries (d2g_ccd_features)."""
        pairs = np.ascontiguousarray(pairs, dtype=np.int32).reshape(-1, 2)
        mt = np.ascontiguousarray(np.broadcast_to(np.asarray(max_time, dtype=np.float64), (len(pairs),)))
        out = np.zeros((max(1, len(pairs)), 20), np.float32)
        _check(lib().d2g_ccd_features(self.h, _p(pairs, I32P), _p(mt, F64P), len(pairs), _p(out, F32P)))
        return out[:len(pairs)]

    def set_ccd_witnesses(self, enable):
        """Separation witnesses in every CCD call (d2g_ctx_set_ccd_witnesses;
        results are identical either way)."""
        _check(lib().d2g_ctx_set_ccd_witnesses(self.h, int(bool(enable))))

    def set_ccd_proposal(self, mlp, threshold=0.5):
        """The learned proposal in every CCD call (d2g_ctx_set_ccd_proposal):
        queries the network predicts contact-free (hit probability below
        threshold) are skipped when the root certificate proves it; mlp None
        turns it off.  Results are identical."""
        self._proposal = mlp
        _check(lib().d2g_ctx_set_ccd_proposal(self.h, mlp.h if mlp is not None else None, C.c_float(threshold)))

    def ccd_stats(self, reset=False):
        """CCD counters (d2g_ctx_ccd_stats) as a dict."""
        out = np.zeros(len(CCD_STATS), np.int64)
        _check(lib().d2g_ctx_ccd_stats(self.h, int(bool(reset)), _p(out, I64P), len(CCD_STATS)))
        return dict(zip(CCD_STATS, out.tolist()))

    def set_tuning(self, key, value):
        """Launch-shape setting (TUNE_*); results are identical for every value."""
        _check(lib().d2g_ctx_set_tuning(self.h, int(key), int(value)))

    def get_tuning(self, key):
        v = C.c_int32()
        _check(lib().d2g_ctx_get_tuning(self.h, int(key), C.byref(v)))
        return v.value

    def solve_layout(self):
        """How the last solve call spread its clusters: counts per layout and
        the hardware-cluster sizes used."""
        v = np.zeros(4, np.int32)
        _check(lib().d2g_ctx_solve_layout(self.h, _p(v, I32P), 4))
        return {"block": int(v[0]), "thread_block_cluster": int(v[1]), "grid": int(v[2]), "cluster_size": int(v[3])}

    def set_level_budget(self, nbytes):
        """Cap the bytes a traversal level may use (0: a sixth of the device);
        larger calls run in chunks of body pairs, with identical results."""
        _check(lib().d2g_ctx_set_level_budget(self.h, C.c_int64(int(nbytes))))

    def apply_tuning(self, settings):
        """Apply {name: value} settings, e.g. those written by delta2_gb300.autotune."""
        for name, value in settings.items():
            self.set_tuning(TUNE_NAMES[name], value)

    def set_scenes(self, scene_of_body):
        """Batch independent scenes: scene index of every body (after set_bodies)."""
        self._scene_of = np.ascontiguousarray(scene_of_body, dtype=np.int32)
        _check(lib().d2g_ctx_set_scenes(self.h, _p(self._scene_of, I32P)))

    def get_bodies(self, scene=None):
        scene = scene or self.scene
        b = scene.bodies_struct()
        _check(lib().d2g_ctx_get_bodies(self.h, C.byref(b)))
        return scene

    def launches(self):
        n = C.c_int64()
        _check(lib().d2g_ctx_launches(self.h, C.byref(n)))
        return n.value

    def set_profiling(self, enable):
        _check(lib().d2g_ctx_set_profiling(self.h, int(bool(enable))))

    def profile(self, kind):
        ms = C.c_double()
        n = C.c_int64()
        items = C.c_int64()
        _check(lib().d2g_ctx_profile(self.h, int(kind), C.byref(ms), C.byref(n), C.byref(items)))
        return ms.value, n.value, items.value

    def compare_trees_full_continuous_device(self, d_pairs, d_max_time, n_pairs):
        """Device-resident CCD: pointers (ints) to int32 pairs and float64 max_time in HBM.
        Returns (n_contacts, d_contacts_ptr, d_offsets_ptr, counters)."""
        n = C.c_int32()
        dc = C.c_void_p()
        do = C.c_void_p()
        cnt = np.zeros(4, np.int64)
        _check(lib().d2g_compare_trees_full_continuous_device(self.h, C.c_void_p(d_pairs), C.c_void_p(d_max_time),
                                                              int(n_pairs), C.byref(n), C.byref(dc), C.byref(do),
                                                              _p(cnt, I64P)))
        return n.value, dc.value, do.value, cnt

    def select_time_steps(self, pairs, clusters, opt_dt):
        """fineCollisionClustersWithTimeStepSelection + clamp for clusters given as
        a list of (particles, interaction index range) -> array of steps.

        ``pairs`` [n,2] holds every cluster's interactions, cluster after
        cluster; ``clusters`` is a list of (particle_list, n_interactions)."""
        pairs = np.ascontiguousarray(pairs, dtype=np.int32).reshape(-1, 2)
        pair_off = np.zeros(len(clusters) + 1, np.int32)
        part_off = np.zeros(len(clusters) + 1, np.int32)
        parts = []
        for k, (plist, ni) in enumerate(clusters):
            pair_off[k + 1] = pair_off[k] + ni
            part_off[k + 1] = part_off[k] + len(plist)
            parts += list(plist)
        parts = np.ascontiguousarray(parts, dtype=np.int32)
        out = np.zeros(max(1, len(clusters)))
        cnt = np.zeros(4, np.int64)
        _check(lib().d2g_select_time_steps(self.h, _p(pairs, I32P), len(pairs), _p(pair_off, I32P),
                                           _p(part_off, I32P), _p(parts, I32P), len(clusters), C.c_float(opt_dt),
                                           _p(out, F64P), _p(cnt, I64P)))
        return out[:len(clusters)].copy(), cnt

    def broad_phase_device(self, scene=None):
        """broadPhaseEmbree over the device bodies -> pairs [n, 2] (ascending)."""
        scene = scene or self.scene
        aabb = np.ascontiguousarray(scene.local_aabb, dtype=np.float32)
        n = C.c_int32()
        _check(lib().d2g_ctx_broad_phase(self.h, _p(aabb, F32P), None, 0, C.byref(n)))
        out = np.zeros((max(1, n.value), 2), np.int32)
        _check(lib().d2g_ctx_broad_phase(self.h, _p(aabb, F32P), _p(out, I32P), n.value, C.byref(n)))
        return out[:n.value].copy()

    def separate_clusters(self, pairs):
        """separateCollisionClusters on the device (rolls the device states back)
        -> list of (particles, interactions [m, 2], min_current_time, step, sleeping)."""
        pairs = np.ascontiguousarray(pairs, dtype=np.int32).reshape(-1, 2)
        nb = self.scene.n_bodies
        ncl = C.c_int32()
        poff = np.zeros(nb + 1, np.int32)
        parts = np.zeros(nb + len(pairs) + 1, np.int32)
        qoff = np.zeros(nb + 1, np.int32)
        cp = np.zeros((max(1, len(pairs)), 2), np.int32)
        mct = np.zeros(nb)
        step = np.zeros(nb)
        sl = np.zeros(nb, np.uint8)
        _check(lib().d2g_ctx_separate_clusters(self.h, _p(pairs, I32P), len(pairs), C.byref(ncl), _p(poff, I32P),
                                               _p(parts, I32P), _p(qoff, I32P), _p(cp, I32P), _p(mct, F64P),
                                               _p(step, F64P), _p(sl, U8P)))
        return [(parts[poff[k]:poff[k + 1]].tolist(), cp[qoff[k]:qoff[k + 1]].copy(), float(mct[k]), float(step[k]),
                 bool(sl[k])) for k in range(ncl.value)]

    def filter_contacts(self, contacts, offsets, margin=0.0):
        """filterContacts per group -> (kept contacts [m,14], out_offsets [n_groups+1])."""
        c = np.ascontiguousarray(contacts, dtype=np.float64).reshape(-1, CONTACT_LEN)
        off = np.ascontiguousarray(offsets, dtype=np.int32)
        ng = len(off) - 1
        cap = max(1, len(c))
        out = np.zeros((cap, CONTACT_LEN))
        out_off = np.zeros(ng + 1, np.int32)
        _check(lib().d2g_filter_contacts(self.h, _p(c, F64P), _p(off, I32P), ng, C.c_double(margin), _p(out, F64P),
                                         cap, _p(out_off, I32P)))
        return out[:out_off[-1]].copy(), out_off

    def solve_clusters(self, clusters, gravity_z=-9.8):
        """SequentialImpulses::solve for clusters given as a list of
        (particles, step, contacts [m,14], pair_count [m], warm [m] (NaN = none)).
        Updates the device future states; returns (status [k], iterations [k,2],
        impulses and body pairs per cluster in the solver's sorted order)."""
        part_off = np.zeros(len(clusters) + 1, np.int32)
        con_off = np.zeros(len(clusters) + 1, np.int32)
        parts, steps, recs, cnts, warms = [], [], [], [], []
        for k, (plist, step, con, cnt, warm) in enumerate(clusters):
            con = np.asarray(con, dtype=np.float64).reshape(-1, CONTACT_LEN)
            part_off[k + 1] = part_off[k] + len(plist)
            con_off[k + 1] = con_off[k] + len(con)
            parts += list(plist)
            steps.append(step)
            recs.append(con)
            cnts.append(np.asarray(cnt, dtype=np.int32).reshape(-1))
            warms.append(np.asarray(warm, dtype=np.float64).reshape(-1))
        parts = np.ascontiguousarray(parts, dtype=np.int32)
        steps = np.ascontiguousarray(steps, dtype=np.float64)
        rec = np.ascontiguousarray(np.concatenate(recs) if recs else np.zeros((0, CONTACT_LEN)))
        cnt = np.ascontiguousarray(np.concatenate(cnts) if cnts else np.zeros(0, np.int32), dtype=np.int32)
        warm = np.ascontiguousarray(np.concatenate(warms) if warms else np.zeros(0), dtype=np.float64)
        n = len(rec)
        status = np.zeros(max(1, len(clusters)), np.int32)
        iters = np.zeros((max(1, len(clusters)), 2), np.int32)
        imp = np.zeros(max(1, n))
        ab = np.zeros((max(1, n), 2), np.int32)
        rc = lib().d2g_solve_clusters(self.h, len(clusters), _p(part_off, I32P), _p(parts, I32P), _p(steps, F64P),
                                      _p(rec, F64P), _p(con_off, I32P), _p(cnt, I32P), _p(warm, F64P),
                                      C.c_double(gravity_z), _p(status, I32P), _p(iters, I32P), _p(imp, F64P),
                                      _p(ab, I32P))
        if rc not in (0, 1):
            _check(rc)
        k = len(clusters)
        return (status[:k].copy(), iters[:k].copy(),
                [imp[con_off[i]:con_off[i + 1]].copy() for i in range(k)],
                [ab[con_off[i]:con_off[i + 1]].copy() for i in range(k)])

    def world_configure(self, scene=None, opt_dt=None, gravity_z=None):
        """Set up the adaptive cluster stepper over the context's bodies."""
        scene = scene or self.scene
        self._aabb = np.ascontiguousarray(scene.local_aabb, dtype=np.float32)
        dt = scene.opt_dt if opt_dt is None else opt_dt
        g = scene.gravity_z if gravity_z is None else gravity_z
        _check(lib().d2g_world_configure(self.h, _p(self._aabb, F32P), C.c_float(dt), C.c_double(g)))

    def world_step(self, n=1):
        """n outer steps (BroadPhaseEmbreeCluster::step) on the GPU."""
        _check(lib().d2g_world_step(self.h, int(n)))

    def world_stats(self):
        out = np.zeros(13, dtype=np.int64)
        _check(lib().d2g_world_stats(self.h, _p(out, I64P)))
        return dict(zip(WORLD_STATS, out.tolist()))

    def world_timing(self):
        """Cumulative host wall time (ms) per stepper phase (instrumentation)."""
        out = np.zeros(10)
        _check(lib().d2g_world_timing(self.h, _p(out, F64P), 10))
        return dict(zip(WORLD_PHASES, out.tolist()))

    def world_warm(self):
        n = C.c_int32()
        _check(lib().d2g_world_warm(self.h, None, None, 0, C.byref(n)))
        m = max(1, n.value)
        keys = np.zeros((m, 2), np.int32)
        vals = np.zeros(m)
        _check(lib().d2g_world_warm(self.h, _p(keys, I32P), _p(vals, F64P), m, C.byref(n)))
        return {(int(keys[i, 0]), int(keys[i, 1])): float(vals[i]) for i in range(n.value)}

    def compare_trees_full(self, pairs, capacity=None):
        """compareTreesFull for each pair -> (contacts [n,14], offsets [n_pairs+1], counters)."""
        pairs = np.ascontiguousarray(pairs, dtype=np.int32).reshape(-1, 2)
        return self._query(lambda cap, out, off, cnt: lib().d2g_compare_trees_full(
            self.h, _p(pairs, I32P), len(pairs), _p(out, F64P), cap, _p(off, I32P), _p(cnt, I64P)), len(pairs),
            capacity)

    def find_contacts_bucket_comparison(self, a, b, node_pairs, capacity=None):
        """findContactsBucketComparison: one level of body pair (a, b)'s discrete
        traversal over node_pairs [n, 2] (global node ids) -> (hits [m, 14],
        pair_used [n], the cumulative hit counts)."""
        npairs = np.ascontiguousarray(node_pairs, dtype=np.int32).reshape(-1, 2)
        cap = capacity if capacity is not None else 64 * len(npairs)
        while True:
            out = np.zeros((max(cap, 1), CONTACT_LEN))
            used = np.zeros(max(1, len(npairs)), np.int32)
            rc = lib().d2g_find_contacts_bucket_comparison(self.h, int(a), int(b), _p(npairs, I32P), len(npairs),
                                                           _p(out, F64P), cap, _p(used, I32P))
            total = int(used[len(npairs) - 1]) if len(npairs) else 0
            if rc == 2 and capacity is None:
                cap = total
                continue
            _check(rc)
            return out[:total].copy(), used[:len(npairs)].copy()

    def compare_trees_full_continuous(self, pairs, max_time, capacity=None):
        """compareTreesFullContinuous for each pair over max_time[i]."""
        pairs = np.ascontiguousarray(pairs, dtype=np.int32).reshape(-1, 2)
        mt = np.ascontiguousarray(np.broadcast_to(np.asarray(max_time, dtype=np.float64), (len(pairs),)))
        return self._query(lambda cap, out, off, cnt: lib().d2g_compare_trees_full_continuous(
            self.h, _p(pairs, I32P), _p(mt, F64P), len(pairs), _p(out, F64P), cap, _p(off, I32P), _p(cnt, I64P)),
            len(pairs), capacity)

    def _query(self, call, n_pairs, capacity):
        cap = capacity if capacity is not None else max(4096, 64 * n_pairs)
        while True:
            out = np.zeros((max(cap, 1), CONTACT_LEN))
            off = np.zeros(n_pairs + 1, np.int32)
            cnt = np.zeros(4, np.int64)
            rc = call(cap, out, off, cnt)
            if rc == 2 and capacity is None:
                cap = int(off[-1]) + 16
                continue
            _check(rc)
            return out[:off[-1]].copy(), off, cnt


MLP_PARAMS = 19458


class Mlp:
    """The learned TOI proposal network (d2g_mlp_*): 20-128-128-2, SiLU, BF16
    weights and activations, trained by the library's own kernels."""

    def __init__(self, ctx, seed=0):
        self.ctx = ctx
        self.h = C.c_void_p()
        _check(lib().d2g_mlp_create(ctx.h, C.c_uint64(seed), C.byref(self.h)))

    def close(self):
        if getattr(self, "h", None):
            lib().d2g_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def params(self):
        p = np.zeros(MLP_PARAMS, np.float32)
        _check(lib().d2g_mlp_params(self.h, _p(p, F32P), MLP_PARAMS))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        _check(lib().d2g_mlp_set_params(self.h, _p(p, F32P), MLP_PARAMS))

    def set_normalization(self, mean, std):
        m = np.ascontiguousarray(mean, dtype=np.float32)
        sd = np.ascontiguousarray(std, dtype=np.float32)
        self._norm = (m, sd)
        _check(lib().d2g_mlp_set_normalization(self.h, _p(m, F32P), _p(sd, F32P)))

    def predict(self, feats):
        f = np.ascontiguousarray(feats, dtype=np.float32).reshape(-1, 20)
        out = np.zeros((max(1, len(f)), 2), np.float32)
        _check(lib().d2g_mlp_predict(self.h, _p(f, F32P), len(f), _p(out, F32P)))
        return out[:len(f)]

    def gradient(self, feats, targets):
        f = np.ascontiguousarray(feats, dtype=np.float32).reshape(-1, 20)
        y = np.ascontiguousarray(targets, dtype=np.float32).reshape(-1, 2)
        g = np.zeros(MLP_PARAMS, np.float32)
        loss = C.c_float()
        _check(lib().d2g_mlp_gradient(self.h, _p(f, F32P), _p(y, F32P), len(f), _p(g, F32P), C.byref(loss)))
        return g, loss.value

    def train(self, feats, targets, epochs=1, batch=4096, lr=1e-3, seed=0):
        f = np.ascontiguousarray(feats, dtype=np.float32).reshape(-1, 20)
        y = np.ascontiguousarray(targets, dtype=np.float32).reshape(-1, 2)
        losses = np.zeros(max(1, epochs), np.float32)
        _check(lib().d2g_mlp_train(self.h, _p(f, F32P), _p(y, F32P), len(f), int(epochs), int(batch),
                                   C.c_float(lr), C.c_uint64(seed), _p(losses, F32P)))
        return losses[:epochs]

