"""Hand-built scenes for the known-answer tests (leaf-only surrogate trees).

A mesh with fewer than 8 triangles is a single leaf bucket in the reference
(model/surrogate_tree.cpp:52-69), so the bucket-level golden cases of
collision_detection/test_comparison.cpp and test_continuous_comparison.cpp
need no tree builder.
"""
import numpy as np

STATE_LEN = 14  # time, qw qx qy qz, L xyz, x xyz, v xyz


def state(x=(0, 0, 0), q=(1, 0, 0, 0), v=(0, 0, 0), L=(0, 0, 0), time=0.0):
    s = np.zeros(STATE_LEN)
    s[0] = time
    s[1:5] = q
    s[5:8] = L
    s[8:11] = x
    s[11:14] = v
    return s


class SmallScene:
    def __init__(self):
        self._meshes = []  # list of (n_nodes arrays)
        self._bodies = []

    def add_leaf_mesh(self, tris):
        tris = np.asarray(tris, dtype=np.float64).reshape(-1, 9)
        assert len(tris) < 8
        self._meshes.append(tris)
        return len(self._meshes) - 1

    def add_body(self, mesh, geo_eps, cur=None, fut=None, last=None, is_static=False, mu=0.5, mass=1.0,
                 inv_inertia=None, last_dt=1.0, bounding_radius=1.0, local_aabb=(-1, -1, -1, 1, 1, 1)):
        self._bodies.append(dict(mesh=mesh, geo_eps=geo_eps, cur=state() if cur is None else cur,
                                 fut=state() if fut is None else fut, last=state() if last is None else last,
                                 is_static=is_static, mu=mu, mass=mass,
                                 ii=np.eye(3) if inv_inertia is None else np.asarray(inv_inertia),
                                 last_dt=last_dt, br=bounding_radius, aabb=local_aabb))
        return len(self._bodies) - 1

    def build(self):
        M = len(self._meshes)
        self.mesh_node_off = np.arange(M + 1, dtype=np.int32)
        self.nodes = np.zeros((M, 4), dtype=np.int32)
        self.nodes[:, 0] = -1
        self.ntris = np.array([len(t) for t in self._meshes], dtype=np.int32)
        self.tris = np.zeros((M, 8, 9))
        for i, t in enumerate(self._meshes):
            self.tris[i, :len(t)] = t
        self.eps = np.zeros((M, 8))
        self.inner_eps = np.zeros((M, 8))
        B = self._bodies
        n = len(B)
        self.mesh = np.array([b["mesh"] for b in B], dtype=np.int32)
        self.is_static = np.array([b["is_static"] for b in B], dtype=np.uint8)
        self.geo_eps = np.array([b["geo_eps"] for b in B], dtype=np.float64)
        self.mu = np.array([b["mu"] for b in B], dtype=np.float64)
        self.mass = np.array([b["mass"] for b in B], dtype=np.float64)
        self.inv_inertia = np.ascontiguousarray(np.stack([b["ii"].reshape(9) for b in B]))
        self.last = np.ascontiguousarray(np.stack([b["last"] for b in B]))
        self.cur = np.ascontiguousarray(np.stack([b["cur"] for b in B]))
        self.fut = np.ascontiguousarray(np.stack([b["fut"] for b in B]))
        self.last_dt = np.array([b["last_dt"] for b in B], dtype=np.float64)
        self.sleep_steps = np.zeros(n, dtype=np.int32)
        self.sleeping = np.zeros(n, dtype=np.uint8)
        self.bounding_radius = np.array([b["br"] for b in B], dtype=np.float64)
        self.local_aabb = np.array([b["aabb"] for b in B], dtype=np.float32)
        self.opt_dt = 0.01
        return self

    def to_product(self):
        """The same arrays as a delta2_gb300.Scene (for the C-ABI entry points)."""
        import delta2_gb300 as D
        s = D.Scene()
        s.__dict__.update({k: v for k, v in self.__dict__.items() if not k.startswith("_")})
        return s


def tris_from(V, F):
    V = np.asarray(V, dtype=np.float64)
    return np.array([np.concatenate([V[f[0]], V[f[1]], V[f[2]]]) for f in F])


# The 4-triangle pyramid surface of the bucket tests (test_comparison.cpp:93-105).
PYRAMID_V = [[1.0, 1.0, 0.0], [-1.0, 1.0, 0.0], [-1.0, -1.0, 0.0], [1.0, -1.0, 0.0], [0.0, 0.0, 0.1]]
PYRAMID_F = [[0, 1, 4], [1, 2, 4], [2, 3, 4], [3, 0, 4]]


def plane_mesh(width):
    """common/primitive_geo.cpp:76-89 plane(width)."""
    h = width / 2.0
    V = [[h, h, 0.0], [h, -h, 0.0], [-h, h, 0.0], [-h, -h, 0.0]]
    F = [[0, 2, 1], [1, 2, 3]]
    return V, F
