"""The surrogate-tree builder (host code of the library, d2g_tree_build)
against the oracle's independent restatement of the reference's builder
(oracle/d2o_tree.hpp: SurrogateTree::buildSurrogateTreeKMean, divideAndFit,
calcEpss, selectSurrogateTriangle, PCG32), node for node and bit for bit,
drawing from the same PCG32 stream: the reference's cube, a 64-point convex
hull, subdivision-2 and noisy subdivision-3 icospheres, a flat grid, and a
degenerate mesh of repeated triangles that takes divideAndFit's last-resort
branch.  Every mesh triangle must land in a leaf (CPU only)."""
import numpy as np
import pytest

import delta2_gb300 as D
from oracle import oracle as O


def cube_mesh(h=0.5):
    V = np.array([[1, 1, 1], [1, 1, -1], [1, -1, 1], [1, -1, -1], [-1, 1, 1], [-1, 1, -1], [-1, -1, 1],
                  [-1, -1, -1]], dtype=np.float64) * h
    F = np.array([[0, 2, 1], [1, 2, 3], [2, 6, 3], [3, 6, 7], [4, 5, 6], [5, 7, 6], [4, 0, 1], [4, 1, 5],
                  [0, 4, 6], [0, 6, 2], [3, 7, 1], [7, 5, 1]], dtype=np.int32)
    return V, F


def icosphere(sub, radius=0.5, noise=0.0, seed=0):
    t = (1.0 + 5 ** 0.5) / 2.0
    V = [[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
         [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]]
    F = [[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2],
         [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5], [2, 4, 11],
         [6, 2, 10], [8, 6, 7], [9, 8, 1]]
    V = [np.array(v, dtype=np.float64) / np.linalg.norm(v) for v in V]
    for _ in range(sub):
        mid = {}

        def m(a, b):
            k = (min(a, b), max(a, b))
            if k not in mid:
                p = V[a] + V[b]
                V.append(p / np.linalg.norm(p))
                mid[k] = len(V) - 1
            return mid[k]

        F = [f for a, b, c in F for f in ([a, m(a, b), m(c, a)], [b, m(b, c), m(a, b)], [c, m(c, a), m(b, c)],
                                          [m(a, b), m(b, c), m(c, a)])]
    V = np.array(V)
    r = radius * (1.0 + noise * np.random.default_rng(seed).uniform(-1, 1, len(V)))
    return V * r[:, None], np.array(F, dtype=np.int32)


def hull_mesh(n=64, radius=0.6, seed=0):
    spatial = pytest.importorskip("scipy.spatial")
    rng = np.random.default_rng(seed)
    p = rng.normal(size=(n, 3))
    p *= (rng.uniform(size=n) ** (1 / 3) / np.linalg.norm(p, axis=1))[:, None]
    h = spatial.ConvexHull(p)
    used = np.unique(h.simplices)
    remap = -np.ones(n, np.int64)
    remap[used] = np.arange(len(used))
    return p[used] * radius, remap[h.simplices].astype(np.int32)


def grid_mesh(k=6):
    xs = np.linspace(-1, 1, k + 1)
    V = np.array([[x, y, 0.0] for y in xs for x in xs])
    F = []
    for j in range(k):
        for i in range(k):
            a = j * (k + 1) + i
            F += [[a, a + 1, a + k + 2], [a, a + k + 2, a + k + 1]]
    return V, np.array(F, dtype=np.int32)


def repeated_mesh(n=9):
    V = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0]])
    return V, np.tile(np.array([[0, 1, 2]], dtype=np.int32), (n, 1))


MESHES = {"cube": cube_mesh, "hull64": hull_mesh, "icosphere2": lambda: icosphere(2),
          "noisy_icosphere3": lambda: icosphere(3, noise=0.2, seed=5), "grid": grid_mesh,
          "repeated9": repeated_mesh, "repeated20": lambda: repeated_mesh(20)}


def _bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.uint64)


@pytest.mark.parametrize("name", sorted(MESHES))
def test_tree_matches_oracle_node_for_node(name):
    V, F = MESHES[name]()
    stream = D.pcg32_seed(42, 54)
    got = D.build_tree(V, F, stream)
    ref = O.build_tree(V, F, stream)
    nodes, ntris, tris, eps, ieps, rng = got
    assert nodes.shape == ref[0].shape, (nodes.shape, ref[0].shape)
    assert np.array_equal(nodes, ref[0]) and np.array_equal(ntris, ref[1])
    for k, what in ((2, "triangles"), (3, "eps"), (4, "inner_eps")):
        assert np.array_equal(_bits(got[k]), _bits(ref[k])), what
    assert rng == ref[5], "the PCG32 stream advanced differently"
    # every mesh triangle lands in a leaf and no leaf holds anything else;
    # copies are possible: when divideAndFit's split of the largest group
    # leaves its first sub-group empty, the largest group keeps its triangles
    # while the other sub-groups take them too (construct_surrogate_tree.h:
    # 99-117), and the reference builds those copies into the tree
    leaf = [tuple(tris[g, i].tolist()) for g in range(len(nodes)) if nodes[g, 2] == 0 for i in range(ntris[g])]
    mesh = [tuple(np.concatenate([V[f[0]], V[f[1]], V[f[2]]]).tolist()) for f in F]
    assert set(leaf) == set(mesh)
    assert len(leaf) >= len(mesh)
    if name in ("cube", "hull64", "icosphere2", "grid"):
        assert sorted(leaf) == sorted(mesh), "each triangle exactly once"


def test_trees_of_many_meshes_continue_one_stream():
    """Meshes built one after another draw from one stream, as the
    reference's Options does: the second tree starts where the first left it."""
    s = D.pcg32_seed(42, 54)
    a = D.build_tree(*cube_mesh(), s)
    b = D.build_tree(*icosphere(2), a[5])
    ra = O.build_tree(*cube_mesh(), s)
    rb = O.build_tree(*icosphere(2), ra[5])
    assert a[5] == ra[5] and b[5] == rb[5]
    assert np.array_equal(_bits(b[2]), _bits(rb[2]))
