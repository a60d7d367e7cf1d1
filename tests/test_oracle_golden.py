"""Pin the CPU oracle to the reference's own known-answer tests.

Each case restates a Catch2 case of the reference (file:line in the test
name's docstring) with the same inputs and the same margins.
"""
import math

import numpy as np
import pytest

from oracle import oracle as O
from tests.small_scenes import PYRAMID_F, PYRAMID_V, SmallScene, plane_mesh, state, tris_from

TRI1 = np.array([[-1, 0, 0], [1, 0, 0], [0, -2, 0]], dtype=np.float64)


def close(a, b, m):
    return np.all(np.abs(np.asarray(a) - np.asarray(b)) < m)


def catch_approx(value, target, eps=1.1920929e-05, margin=0.0):
    # Catch2 v2 Approx: |a-b| <= margin or |a-b| <= eps*(scale + max(|a|,|b|)), scale = 0
    d = abs(value - target)
    return d <= margin or d <= eps * max(abs(value), abs(target))


# ------------------------------------------------ collision_detection/test_comparison.cpp
def test_tri_tri_vert_face():
    """test_comparison.cpp:8-34"""
    A = O.tri_xform(TRI1, O.transformation_euler([0.5235, 0.3491, 0.0], [0.0, 1.0, 1.2651]))
    B = O.tri_xform(TRI1, O.transformation_euler([-0.1745, 0.0, 0.0873], [0, 0, 0]))
    d, P, Q = O.tri_tri_dist(A, B)
    P0 = np.array([-0.342, -0.732, 0.326])
    Q0 = np.array([-0.339, -0.767, 0.129])
    assert close(P, P0, 0.01)
    assert close(Q, Q0, 0.01)
    assert abs(d - np.linalg.norm(P0 - Q0)) <= 0.02


def test_tri_tri_edge_edge():
    """test_comparison.cpp:36-62"""
    A = O.tri_xform(TRI1, O.transformation_euler([1.323341, 0.301492, 0.887539], [-1.0284, -1.0942, 1.1695]))
    B = O.tri_xform(TRI1, O.transformation_euler([-0.1745, 0.0, 0.0873], [0, 0, 0]))
    d, P, Q = O.tri_tri_dist(A, B)
    P0 = np.array([-0.6545, -0.9378, 0.2656])
    Q0 = np.array([-0.5089, -0.8695, 0.1449])
    assert close(P, P0, 0.01)
    assert close(Q, Q0, 0.01)
    assert abs(d - np.linalg.norm(P0 - Q0)) <= 0.02


def test_tri_tri_intersecting():
    """test_comparison.cpp:64-88"""
    A = O.tri_xform(TRI1, O.transformation_euler([1.323341, 0.301492, 0.887539], [0.052572, -0.153374, 1.0443]))
    B = O.tri_xform(TRI1, O.transformation_euler([-0.1745, 0.0, 0.0873], [0, 0, 0]))
    d, P, Q = O.tri_tri_dist(A, B)
    assert abs(d) <= 1e-4


def _pyramid_plane_scene(plane_cur_z, plane_fut_z, pyr_z=1.0):
    s = SmallScene()
    m_pyr = s.add_leaf_mesh(tris_from(PYRAMID_V, PYRAMID_F))
    V, F = plane_mesh(1.0)
    m_pl = s.add_leaf_mesh(tris_from(V, F))
    s.add_body(m_pyr, 0.01, cur=state(x=(0, 0, pyr_z)), fut=state(x=(0, 0, pyr_z)), is_static=True)
    s.add_body(m_pl, 0.01, cur=state(x=(0, 0, plane_cur_z)), fut=state(x=(0, 0, plane_fut_z)))
    return s.build()


def test_bucket_comparison():
    """test_comparison.cpp:90-128: 8 hits, one after filterContacts."""
    sc = _pyramid_plane_scene(1.105, 1.105)
    hits, used = O.bucket_comparison(sc, 0, 1, [[0, 1]])
    assert len(used) == 1 and used[0] == 8
    assert len(O.filter_contacts(hits, 0.0)) == 1
    assert len(O.filter_contacts(hits, 0.0, unstable=True)) == 1


# ----------------------------------------- collision_detection/test_continuous_comparison.cpp
def test_sphere_sphere_first_intersect():
    """test_continuous_comparison.cpp:6-32"""
    assert O.sphere_sphere([0, 0, 0], [1, 0, 0], 1.0, [0, -0.5, 0], [-1, 0, 0], 1.0) == 0.0
    assert O.sphere_sphere([0, 0, 0], [1, 0, 0], 0.5, [0, -1.001, 0], [-1, 0, 0], 0.5) == -1.0
    t = O.sphere_sphere([0, 0, 0], [1, 0, 0], 0.5, [0, -1.001, 0], [1, 0.1, 0], 0.5)
    assert catch_approx(t, 0.01, eps=0.0001)


A_T_START = np.array([[0.9961947202682495, -0.0858316496014595, -0.015134435147047043, 0.0],
                      [0.08715573698282242, 0.981060266494751, 0.17298738658428192, 0.0],
                      [0.0, -0.1736481785774231, 0.9848077297210693, 0.0], [0.0, 0.0, 0.0, 1.0]])


def test_ccd_far():
    """test_continuous_comparison.cpp:34-75"""
    aE = np.eye(4)
    aE[2, 3] = 2.0
    bS = np.array([[0.912834644317627, -0.24342688918113708, -0.32783564925193787, -0.8726963400840759],
                   [0.40832462906837463, 0.548050582408905, 0.7300079464912415, 1.8028504848480225],
                   [0.0019669521134346724, -0.8002399206161499, 0.5996767282485962, 4.524521350860596],
                   [0, 0, 0, 1.0]])
    bE = np.array([[0.9537079334259033, 0.2651883065700531, -0.14183202385902405, 0.0],
                   [-0.05004240944981575, 0.6049837470054626, 0.7946637272834778, 1.0],
                   [0.29654160141944885, -0.7507795095443726, 0.5902484655380249, 3.9175784587860107],
                   [0, 0, 0, 1.0]])
    d, P, Q, toc = O.tri_tri_ccd(TRI1, A_T_START, aE, TRI1, bS, bE)
    P0 = np.array([-0.951562, -0.004578, 2.0])
    Q0 = np.array([-0.954302, 1.05403, 3.62159])
    assert toc == 1.0
    assert close(P, P0, 0.1)
    assert close(Q, Q0, 0.1)
    assert abs(d - np.linalg.norm(P0 - Q0)) <= 0.05


def test_ccd_close():
    """test_continuous_comparison.cpp:77-117"""
    aE = np.eye(4)
    aE[2, 3] = 0.43169140815734863
    bS = np.array([[0.912834644317627, -0.24342688918113708, -0.32783564925193787, 1.958876609802246],
                   [0.40832462906837463, 0.548050582408905, 0.7300079464912415, -0.9190752506256104],
                   [0.0019669521134346724, -0.8002399206161499, 0.5996767282485962, -1.093824863433838],
                   [0, 0, 0, 1.0]])
    bE = np.array([[0.9537079334259033, 0.2651883065700531, -0.14183202385902405, 1.958876609802246],
                   [-0.05004240944981575, 0.6049837470054626, 0.7946637272834778, -0.9190752506256104],
                   [0.29654160141944885, -0.7507795095443726, 0.5902484655380249, 1.0489931106567383],
                   [0, 0, 0, 1.0]])
    d, P, Q, toc = O.tri_tri_ccd(TRI1, A_T_START, aE, TRI1, bS, bE)
    P0 = np.array([0.64, -0.73, 0.38])
    Q0 = np.array([1.0, -0.95, 0.44])
    assert abs(toc - 0.79) <= 0.05
    assert close(P, P0, 0.05)
    assert close(Q, Q0, 0.05)
    assert abs(d - np.linalg.norm(P0 - Q0)) <= 0.05


def test_ccd_intersect():
    """test_continuous_comparison.cpp:119-160"""
    aE = np.eye(4)
    aE[2, 3] = 2.0
    bS = np.array([[0.9396926164627075, 0.1710100769996643, 0.29619812965393066, 0.0],
                   [0.0, 0.8660253882408142, -0.5, 1.0],
                   [-0.3420201241970062, 0.46984633803367615, 0.813797652721405, 1.2651395797729492],
                   [0, 0, 0, 1.0]])
    bE = np.array([[0.9396926164627075, 0.0, 0.3420201241970062, 0.0], [0.0, 1.0, 0.0, 1.0],
                   [-0.3420201241970062, 0.0, 0.9396926164627075, 1.5], [0, 0, 0, 1.0]])
    d, P, Q, toc = O.tri_tri_ccd(TRI1, A_T_START, aE, TRI1, bS, bE)
    P0 = np.array([-0.265017, -0.843225, 0.591865])
    assert abs(toc - 0.24) <= 0.05
    assert close(P, P0, 0.1)
    assert close(Q, P0, 0.1)
    assert d == 0.0


def _deg(x):
    return 2.0 * 3.14159265358979323846 * x / 360.0


TRI_EE = np.array([[1, -1, 0], [-1, 1, 0], [-1, -1, 0]], dtype=np.float64)


def _ee_case(a_end_z, b_end_z):
    ra = [_deg(66.2817), _deg(-45.7037), _deg(-111.169)]
    rb = [_deg(261.326), _deg(52.4147), _deg(-101.34)]
    aS = O.tri_xform(TRI_EE, O.transformation_euler(ra, [0, 0, 0]))
    aE = O.tri_xform(TRI_EE, O.transformation_euler(ra, [0, 0, a_end_z]))
    bS = O.tri_xform(TRI_EE, O.transformation_euler(rb, [0, 0, 1.3]))
    bE = O.tri_xform(TRI_EE, O.transformation_euler(rb, [0, 0, b_end_z]))
    return O.edge_edge_ccd(aS[:2], aE[:2], bS[:2], bE[:2])


def test_edge_edge_intersect():
    """test_continuous_comparison.cpp:163-190"""
    d, P, Q, toc = _ee_case(0.7, 0.5)
    assert abs(toc - 0.87) <= 0.01
    assert close(P, [0, 0, 0.6], 0.01)
    assert close(Q, [0, 0, 0.6], 0.01)
    assert abs(d) <= 0.01


def test_edge_edge_no_intersect():
    """test_continuous_comparison.cpp:192-219"""
    d, P, Q, toc = _ee_case(0.5, 0.7)
    assert abs(toc - 1.0) <= 0.02
    assert close(P, [0, 0, 0.5], 0.1)
    assert close(Q, [-0.01, -0.11, 0.68], 0.1)
    assert abs(d - 0.2) <= 0.05


def test_continuous_bucket():
    """test_continuous_comparison.cpp:222-263: one filtered hit, toc == Approx(0.9)."""
    sc = _pyramid_plane_scene(2.0, 1.0)
    hits, used = O.bucket_continuous(sc, 0, 1, [[0, 1]])
    f = O.filter_contacts(hits, 0.0, continuous=True)
    assert len(f) == 1
    assert catch_approx(f[0, 10], 0.9)


def test_point_tri_segment_error_case():
    """test_continuous_comparison.cpp:265-275"""
    tri = np.array([[50, 50, 0], [-50, 50, 0], [50, -50, 0]], dtype=np.float64)
    _, t, tinf, isint = O.intersect_segment(tri, [[2, -1, 0.29], [2, -1, -0.81]])
    assert isint


# ----------------------------------------------------------- common/test_*.cpp
def test_barycentric_vertices():
    """common/test_triangle.cpp:57-82"""
    tri = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], dtype=np.float64)
    assert list(O.bary(tri, tri[0])) == [1.0, 0.0, 0.0]
    assert list(O.bary(tri, tri[1])) == [0.0, 1.0, 0.0]
    assert list(O.bary(tri, tri[2])) == [0.0, 0.0, 1.0]


def test_triangle_interaction():
    """common/test_triangle.cpp:84-103"""
    b = [1.0, 0.0, 0.0]
    d = [-1.0, 1.0, 0.0]
    e = [-1.0, -1.0, 0.0]
    tri2 = np.array([b, d, e])
    pt, t, tinf, isint = O.intersect_segment(tri2, [[-1.0, 1.0, 1.0], [1.0, -1.0, -1.0]])
    assert isint
    assert close(pt, [0, 0, 0], 1e-3)
    proj, inside = O.project_to_plane(tri2, [2.0, 2.0, 1.0])
    assert not inside
    assert close(proj, [2.0, 2.0, 0.0], 1e-3)


def test_edge_closest():
    """common/test_edge.cpp:22-73"""
    ab = [[0.0, 1.0, 0.0], [0.0, -1.0, 0.0]]
    cd = [[1.0, 0.0, 1.0], [1.0, 0.0, -1.0]]
    ef = [[0.0, 0.0, 1.0], [0.0, 0.0, 0.0]]
    assert catch_approx(O.edge_closest(ab, cd)[0], 1.0)
    assert O.edge_closest(ab, ef)[0] <= 1e-12
    assert catch_approx(O.edge_closest(ef, cd)[0], 1.0)
    d, P, Q = O.edge_closest(ab, cd)
    d2, P2, Q2 = O.edge_closest(cd, ab)
    assert close(P, [0, 0, 0], 1e-3) and close(Q, [1, 0, 0], 1e-3)
    assert close(P, Q2, 1e-3) and close(Q, P2, 1e-3)
    d, P, Q = O.edge_closest(ef, cd)
    assert abs(P[0]) < 1e-9 and abs(P[1]) < 1e-9 and -1e-9 <= P[2] <= 1 + 1e-9
    assert abs(Q[0] - 1) < 1e-9 and abs(Q[1]) < 1e-9


def test_transformation_matrix():
    """common/test_utils.cpp:36-91 (MatrixEqual default margin 1e-3)."""
    t = O.transformation_euler([0.0, 0.0, 3.14159 / 2.0], [0, 0, 0])
    ref = np.array([[0, -1, 0, 0], [1, 0, 0, 0], [0, 0, 1, 0], [0, 0, 0, 1.0]])
    assert close(t, ref, 1e-3)
    assert close(O.xform([1, 0, 0], t), [0, 1, 0], 1e-3)
    t = O.transformation_euler([0.5235, 0.3491, 0.0], [0.0, 1.0, 1.2651])
    ref = np.array([[0.9396926164627075, 0.1710100769996643, 0.29619812965393066, 0.0],
                    [0.0, 0.8660253882408142, -0.5, 1.0],
                    [-0.3420201241970062, 0.46984633803367615, 0.813797652721405, 1.2651395797729492],
                    [0, 0, 0, 1.0]])
    assert close(t, ref, 1e-3)
    assert close(O.xform([1, 0, 0], t), [0.9397, 1.0, 0.923], 1e-3)


def test_inverse_of_rigid_transform():
    t = O.transformation_euler([0.3, -1.2, 2.0], [1.0, -2.0, 0.5])
    assert np.allclose(O.mat_inverse(t) @ t, np.eye(4), atol=1e-14)


# ------------------------------------------------------------ model/test_mesh_data.cpp
def _reference_sphere(r, res):
    """common/primitive_geo.cpp:33-75 sphere(r, res, V, F) (UV sphere)."""
    V = [[0.0, 0.0, r]]
    for j in range(1, res - 1):
        z = r * math.cos(math.pi * j / (res - 1))
        for k in range(res):
            s = r * math.sin(math.pi * j / (res - 1))
            V.append([s * math.cos(2 * math.pi * k / res), s * math.sin(2 * math.pi * k / res), z])
    V.append([0.0, 0.0, -r])
    F = [[0, j + 1, (j + 1) % res + 1] for j in range(res)]
    for j in range(1, res - 2):
        for k in range(res):
            v1, v2 = (j - 1) * res + k + 1, j * res + k + 1
            v3, v4 = (j - 1) * res + 1 + (k + 1) % res, j * res + 1 + (k + 1) % res
            F += [[v1, v4, v3], [v1, v2, v4]]
    vo = 1 + (res - 3) * res
    F += [[vo + res, vo + (j + 1) % res, vo + j] for j in range(res)]
    return np.array(V), np.array(F, dtype=np.int32)


CUBE2_V = np.array([[1, 1, 1], [1, 1, -1], [1, -1, 1], [1, -1, -1], [-1, 1, 1], [-1, 1, -1], [-1, -1, 1],
                    [-1, -1, -1]], dtype=np.float64)
CUBE2_F = np.array([[0, 2, 1], [1, 2, 3], [2, 6, 3], [3, 6, 7], [4, 5, 6], [5, 7, 6], [4, 0, 1], [4, 1, 5],
                    [0, 4, 6], [0, 6, 2], [3, 7, 1], [7, 5, 1]], dtype=np.int32)


def test_inertia_matrix():
    """model/test_mesh_data.cpp:6-51: the side-2 cube's unit inertia is
    V * 4/6 * I (to 1e-3), a solid sphere(1, 10) V * 2/5 * I and a hollow
    sphere(1, 8) (surface model) V * 2/3 * I, both to 0.15."""
    vol, com, I = O.mass_properties(CUBE2_V, CUBE2_F)
    assert abs(vol - 8.0) < 1e-12 and np.abs(com).max() < 1e-12
    assert np.abs(I - vol * (4.0 / 6.0) * np.eye(3)).max() <= 1e-3
    V, F = _reference_sphere(1.0, 10)
    vol, com, I = O.mass_properties(V, F)
    assert np.abs(I - vol * 0.4 * np.eye(3)).max() <= 0.15
    V, F = _reference_sphere(1.0, 8)
    vol, com, I = O.mass_properties(V, F, surface=True, thickness=0.01)
    assert np.abs(I - vol * (2.0 / 3.0) * np.eye(3)).max() <= 0.15
