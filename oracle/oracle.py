"""ctypes binding of the CPU oracle (test infrastructure only).

Only the test-suite, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` load this module.  It is the checker, never the product path.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

_libs = {}
_kind = "checker"

I32P = C.POINTER(C.c_int32)
F64P = C.POINTER(C.c_double)
F32P = C.POINTER(C.c_float)
U8P = C.POINTER(C.c_uint8)
I64P = C.POINTER(C.c_longlong)


class Trees(C.Structure):
    _fields_ = [("n_meshes", C.c_int32), ("mesh_node_off", I32P), ("nodes", I32P), ("ntris", I32P),
                ("tris", F64P), ("eps", F64P), ("inner_eps", F64P)]


class Bodies(C.Structure):
    _fields_ = [("n", C.c_int32), ("mesh", I32P), ("is_static", U8P), ("geo_eps", F64P), ("mu", F64P),
                ("mass", F64P), ("inv_inertia", F64P), ("last", F64P), ("cur", F64P), ("fut", F64P),
                ("last_dt", F64P), ("sleep_steps", I32P), ("sleeping", U8P), ("bounding_radius", F64P)]


def _p(a, t):
    return a.ctypes.data_as(t)


def select_build(kind):
    """Route every call of this module to one build of the oracle:
    "checker" (the portable -O2 build the tests use, the default) or "fast"
    (the host-tuned -O3 build the benchmark's CPU baselines time).  Both give
    identical results."""
    global _kind
    assert kind in ("checker", "fast")
    _kind = kind


def lib(kind=None):
    kind = kind or _kind
    if kind not in _libs:
        path = _build.build(fast=kind == "fast")
        L = C.CDLL(path)
        for name in ["o_sin", "o_cos", "o_acos", "o_log"]:
            getattr(L, name).restype = C.c_double
            getattr(L, name).argtypes = [C.c_double]
        L.o_sphere_sphere.restype = C.c_double
        L.o_edge_closest.restype = C.c_double
        L.o_world_create.restype = C.c_void_p
        L.o_world_create.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_float, C.c_double]
        for name in ["o_world_destroy", "o_world_set_unstable_filter", "o_world_get_bodies", "o_world_set_bodies",
                     "o_world_step", "o_world_stats", "o_world_broad_phase", "o_world_select_dt", "o_world_solve",
                     "o_world_warm_size", "o_world_warm_get", "o_world_warm_set"]:
            getattr(L, name).argtypes = None
        L.o_world_select_dt.restype = C.c_double
        _libs[kind] = L
    return _libs[kind]


def _d(a):
    return np.ascontiguousarray(a, dtype=np.float64)


# ----------------------------------------------------------- primitives ---
def mass_properties(V, F, surface=False, thickness=0.01):
    """MeshData's volume, centre of mass and unit inertia tensor (oracle/d2o_mass.hpp)."""
    Vf = _d(V).reshape(-1, 3)
    Ff = np.ascontiguousarray(F, dtype=np.int32).reshape(-1, 3)
    out = np.zeros(13)
    lib().o_mass_properties(_p(Vf, F64P), len(Vf), _p(Ff, I32P), len(Ff), int(bool(surface)), C.c_double(thickness),
                            _p(out, F64P))
    return out[0], out[1:4].copy(), out[4:13].reshape(3, 3).copy()


def build_tree(V, F, rng_state):
    """SurrogateTree(V, F, opt) restated (oracle/d2o_tree.hpp) from the PCG32
    stream rng_state = (state, inc) -> (nodes [n,4], ntris, tris [n,8,9], eps,
    inner_eps, rng state after the build); layout as the library's."""
    Vf = _d(V).reshape(-1, 3)
    Ff = np.ascontiguousarray(F, dtype=np.int32).reshape(-1, 3)
    rng = np.array(rng_state, dtype=np.uint64)
    L = lib()
    n = L.o_tree_build(_p(Vf, F64P), len(Vf), _p(Ff, I32P), len(Ff), rng.ctypes.data_as(C.POINTER(C.c_uint64)),
                       None, None, None, None, None, 0)
    assert n > 0, "the reference would throw"
    nodes = np.zeros((n, 4), np.int32)
    ntris = np.zeros(n, np.int32)
    tris = np.zeros((n, 8, 9))
    eps = np.zeros((n, 8))
    ieps = np.zeros((n, 8))
    m = L.o_tree_build(_p(Vf, F64P), len(Vf), _p(Ff, I32P), len(Ff), rng.ctypes.data_as(C.POINTER(C.c_uint64)),
                       _p(nodes, I32P), _p(ntris, I32P), _p(tris, F64P), _p(eps, F64P), _p(ieps, F64P), n)
    assert m == n
    return nodes, ntris, tris, eps, ieps, (int(rng[0]), int(rng[1]))


def sin(x):
    return lib().o_sin(float(x))


def cos(x):
    return lib().o_cos(float(x))


def acos(x):
    return lib().o_acos(float(x))


def log(x):
    return lib().o_log(float(x))


def transformation_euler(euler, pos):
    out = np.zeros(16)
    lib().o_transformation_euler(_p(_d(euler), F64P), _p(_d(pos), F64P), _p(out, F64P))
    return out.reshape(4, 4)


def transformation_quat(q, pos):
    out = np.zeros(16)
    lib().o_transformation_quat(_p(_d(q), F64P), _p(_d(pos), F64P), _p(out, F64P))
    return out.reshape(4, 4)


def mat_inverse(m):
    out = np.zeros(16)
    lib().o_mat_inverse(_p(_d(m).ravel(), F64P), _p(out, F64P))
    return out.reshape(4, 4)


def xform(p, m):
    out = np.zeros(3)
    lib().o_xform(_p(_d(p), F64P), _p(_d(m).ravel(), F64P), _p(out, F64P))
    return out


def tri_xform(tri, m):
    out = np.zeros(9)
    lib().o_tri_xform(_p(_d(tri).ravel(), F64P), _p(_d(m).ravel(), F64P), _p(out, F64P))
    return out.reshape(3, 3)


def bary(tri, p):
    out = np.zeros(3)
    lib().o_bary(_p(_d(tri).ravel(), F64P), _p(_d(p), F64P), _p(out, F64P))
    return out


def intersect_segment(tri, edge):
    pt = np.zeros(3)
    t = C.c_double()
    tinf = C.c_int()
    isint = C.c_int()
    lib().o_intersect_segment(_p(_d(tri).ravel(), F64P), _p(_d(edge).ravel(), F64P), _p(pt, F64P), C.byref(t),
                              C.byref(tinf), C.byref(isint))
    return pt, t.value, bool(tinf.value), bool(isint.value)


def project_to_plane(tri, p):
    out = np.zeros(3)
    inn = C.c_int()
    lib().o_project_to_plane(_p(_d(tri).ravel(), F64P), _p(_d(p), F64P), _p(out, F64P), C.byref(inn))
    return out, bool(inn.value)


def edge_closest(s, e):
    P = np.zeros(3)
    Q = np.zeros(3)
    d = lib().o_edge_closest(_p(_d(s).ravel(), F64P), _p(_d(e).ravel(), F64P), _p(P, F64P), _p(Q, F64P))
    return d, P, Q


def tri_tri_dist(a, b):
    out = np.zeros(7)
    lib().o_tri_tri_dist(_p(_d(a).ravel(), F64P), _p(_d(b).ravel(), F64P), _p(out, F64P))
    return out[0], out[1:4], out[4:7]


def sphere_sphere(ap, av, ar, bp, bv, br):
    return lib().o_sphere_sphere(_p(_d(ap), F64P), _p(_d(av), F64P), C.c_double(ar), _p(_d(bp), F64P),
                                 _p(_d(bv), F64P), C.c_double(br))


def point_tri_ccd(pt, pS, pE, tri, tS, tE):
    out = np.zeros(8)
    lib().o_point_tri_ccd(*[_p(_d(x).ravel(), F64P) for x in (pt, pS, pE, tri, tS, tE)], _p(out, F64P))
    return out[0], out[1:4], out[4:7], out[7]


def edge_edge_ccd(aS, aE, bS, bE):
    out = np.zeros(8)
    lib().o_edge_edge_ccd(*[_p(_d(x).ravel(), F64P) for x in (aS, aE, bS, bE)], _p(out, F64P))
    return out[0], out[1:4], out[4:7], out[7]


def tri_tri_ccd(a, aS, aE, b, bS, bE):
    out = np.zeros(8)
    lib().o_tri_tri_ccd(*[_p(_d(x).ravel(), F64P) for x in (a, aS, aE, b, bS, bE)], _p(out, F64P))
    return out[0], out[1:4], out[4:7], out[7]


def state_extrapolate(s14, t, ii9):
    out = np.zeros(14)
    lib().o_state_extrapolate(_p(_d(s14), F64P), C.c_double(t), _p(_d(ii9).ravel(), F64P), _p(out, F64P))
    return out


# --------------------------------------------------------- scene views ----
class SceneView:
    """Holds numpy arrays alive and exposes Trees / Bodies structs over them.

    ``scene`` is any object with the attributes produced by
    ``delta2_gb300.scene`` (numpy arrays: mesh_node_off, nodes, ntris, tris,
    eps, inner_eps; body arrays mesh, is_static, geo_eps, mu, mass,
    inv_inertia, last, cur, fut, last_dt, sleep_steps, sleeping,
    bounding_radius, local_aabb).
    """

    def __init__(self, scene):
        self.s = scene
        s = scene
        self.trees = Trees(len(s.mesh_node_off) - 1, _p(s.mesh_node_off, I32P), _p(s.nodes, I32P),
                           _p(s.ntris, I32P), _p(s.tris, F64P), _p(s.eps, F64P), _p(s.inner_eps, F64P))
        self.bodies = Bodies(len(s.mesh), _p(s.mesh, I32P), _p(s.is_static, U8P), _p(s.geo_eps, F64P),
                             _p(s.mu, F64P), _p(s.mass, F64P), _p(s.inv_inertia, F64P), _p(s.last, F64P),
                             _p(s.cur, F64P), _p(s.fut, F64P), _p(s.last_dt, F64P), _p(s.sleep_steps, I32P),
                             _p(s.sleeping, U8P), _p(s.bounding_radius, F64P))


def bucket_comparison(scene, ia, ib, node_pairs, cap=4096):
    v = SceneView(scene)
    npairs = np.ascontiguousarray(node_pairs, dtype=np.int32)
    out = np.zeros((cap, 14))
    used = np.zeros(len(npairs), dtype=np.int32)
    n = lib().o_bucket_comparison(C.byref(v.trees), C.byref(v.bodies), ia, ib, _p(npairs, I32P), len(npairs),
                                  _p(out, F64P), cap, _p(used, I32P))
    assert n >= 0
    return out[:n].copy(), used


def bucket_continuous(scene, ia, ib, node_pairs, connected=False, cap=65536):
    v = SceneView(scene)
    npairs = np.ascontiguousarray(node_pairs, dtype=np.int32)
    out = np.zeros((cap, 14))
    used = np.zeros(len(npairs), dtype=np.int32)
    n = lib().o_bucket_continuous(C.byref(v.trees), C.byref(v.bodies), ia, ib, _p(npairs, I32P), len(npairs),
                                  int(connected), _p(out, F64P), cap, _p(used, I32P))
    assert n >= 0
    return out[:n].copy(), used


def filter_contacts(contacts, margin=0.0, unstable=False, continuous=False):
    c = _d(contacts).reshape(-1, 14)
    out = np.zeros_like(c)
    n = lib().o_filter_contacts(_p(c, F64P), len(c), C.c_double(margin), int(unstable), int(continuous),
                                _p(out, F64P))
    return out[:n].copy()


def narrowphase(scene, pairs, cap=1 << 20):
    v = SceneView(scene)
    pr = np.ascontiguousarray(pairs, dtype=np.int32)
    out = np.zeros((cap, 14))
    off = np.zeros(len(pr) + 1, dtype=np.int32)
    cnt = np.zeros(3, dtype=np.int64)
    n = lib().o_narrowphase(C.byref(v.trees), C.byref(v.bodies), _p(pr, I32P), len(pr), _p(out, F64P), cap,
                            _p(off, I32P), _p(cnt, I64P))
    assert n >= 0, "capacity"
    return out[:n].copy(), off, cnt


def ccd(scene, pairs, max_time, cap=1 << 20):
    """compareTreesFullContinuous per pair; writes projected futures back into scene.fut."""
    v = SceneView(scene)
    pr = np.ascontiguousarray(pairs, dtype=np.int32)
    mt = _d(max_time)
    out = np.zeros((cap, 14))
    off = np.zeros(len(pr) + 1, dtype=np.int32)
    mto = np.zeros(len(pr))
    cnt = np.zeros(3, dtype=np.int64)
    n = lib().o_ccd(C.byref(v.trees), C.byref(v.bodies), _p(pr, I32P), _p(mt, F64P), len(pr), _p(out, F64P), cap,
                    _p(off, I32P), _p(mto, F64P), _p(cnt, I64P))
    assert n >= 0, "capacity"
    return out[:n].copy(), off, mto, cnt


class World:
    """The restated adaptive cluster stepper over a copy of a scene."""

    def __init__(self, scene, opt_dt, gravity_z=-9.8):
        self.scene = scene
        self.view = SceneView(scene)
        la = np.ascontiguousarray(scene.local_aabb, dtype=np.float32)
        self.L = lib()  # the build this world lives in
        self.h = self.L.o_world_create(C.byref(self.view.trees), C.byref(self.view.bodies), la.ctypes.data,
                                      C.c_float(opt_dt), C.c_double(gravity_z))

    def __del__(self):
        if getattr(self, "h", None):
            self.L.o_world_destroy(C.c_void_p(self.h))
            self.h = None

    def step(self, n=1):
        return self.L.o_world_step(C.c_void_p(self.h), C.c_int(n))

    def get_bodies(self):
        self.L.o_world_get_bodies(C.c_void_p(self.h), C.byref(self.view.bodies))
        return self.scene

    def set_bodies(self):
        self.L.o_world_set_bodies(C.c_void_p(self.h), C.byref(self.view.bodies))

    def set_unstable_filter(self, u):
        self.L.o_world_set_unstable_filter(C.c_void_p(self.h), C.c_int(int(u)))

    def stats(self):
        out = np.zeros(13, dtype=np.int64)
        self.L.o_world_stats(C.c_void_p(self.h), _p(out, I64P))
        keys = ["ccd_pairs", "ccd_contacts", "np_pairs", "np_contacts", "solves", "failures", "normal_iters",
                "friction_iters", "ccd_node_pairs", "ccd_tri_pairs", "ccd_leaf_pairs", "np_node_pairs",
                "np_tri_pairs"]
        return dict(zip(keys, out.tolist()))

    def broad_phase(self, cap=1 << 20):
        out = np.zeros((cap, 2), dtype=np.int32)
        n = self.L.o_world_broad_phase(C.c_void_p(self.h), _p(out, I32P), C.c_int(cap))
        assert n >= 0
        return out[:n].copy()

    def select_dt(self, particles, interactions):
        p = np.ascontiguousarray(particles, dtype=np.int32)
        it = np.ascontiguousarray(interactions, dtype=np.int32).reshape(-1, 2)
        return self.L.o_world_select_dt(C.c_void_p(self.h), _p(p, I32P), C.c_int(len(p)), _p(it, I32P),
                                       C.c_int(len(it)))

    def solve(self, particles, step_size, contacts):
        p = np.ascontiguousarray(particles, dtype=np.int32)
        c = _d(contacts).reshape(-1, 14)
        iters = np.zeros(2, dtype=np.int32)
        ok = self.L.o_world_solve(C.c_void_p(self.h), _p(p, I32P), C.c_int(len(p)), C.c_double(step_size),
                                 _p(c, F64P), C.c_int(len(c)), _p(iters, I32P))
        return bool(ok), iters

    def warm(self):
        n = self.L.o_world_warm_size(C.c_void_p(self.h))
        keys = np.zeros((max(n, 1), 2), dtype=np.int32)
        vals = np.zeros(max(n, 1))
        m = self.L.o_world_warm_get(C.c_void_p(self.h), _p(keys, I32P), _p(vals, F64P), C.c_int(n))
        return {(int(keys[i, 0]), int(keys[i, 1])): float(vals[i]) for i in range(m)}

    def set_warm(self, warm):
        """Replace the warm-start store by {(body a, body b): impulse}."""
        keys = np.ascontiguousarray([k for k in warm], dtype=np.int32).reshape(-1, 2)
        vals = np.ascontiguousarray([warm[k] for k in warm], dtype=np.float64)
        self.L.o_world_warm_set(C.c_void_p(self.h), _p(keys, I32P), _p(vals, F64P), C.c_int(len(vals)))
