"""GPU parity: the CUDA narrow phase and CCD against the CPU oracle, through
the C ABI, from identical states.  Contact records (points, eps, toc, body
ids), their per-pair order, the traversal counters and the future states
left on the bodies must match bit for bit."""
import numpy as np
import pytest

import delta2_gb300 as D
from oracle import oracle as O
from tests.small_scenes import PYRAMID_F, PYRAMID_V, SmallScene, plane_mesh, state, tris_from

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(gpu_required):
    from delta2_gb300 import build as B
    B.build()
    c = D.Context(0)
    yield c
    c.close()


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.uint64)


def assert_bits_equal(got, ref, what):
    g, r = bits(got), bits(ref)
    if g.shape != r.shape:
        raise AssertionError(f"{what}: shape {got.shape} != {ref.shape}")
    bad = np.argwhere(g != r)
    if len(bad):
        i = tuple(bad[0])
        raise AssertionError(f"{what}: {len(bad)} mismatches, first at {i}: {got[i]!r} != {ref[i]!r}")


def project_futures(scene):
    """fut = extrapolate(cur, last_dt) for every body, as the outer step does
    (broad_phase_embree_cluster.cpp:126-132)."""
    for i in range(scene.n_bodies):
        scene.fut[i] = O.state_extrapolate(scene.cur[i], scene.last_dt[i], scene.inv_inertia[i])
    return scene


def broad_pairs(scene):
    w = O.World(scene.copy(), scene.opt_dt)
    return w.broad_phase()


def ccd_parity(ctx, scene, pairs, max_time):
    ref = scene.copy()
    c_ref, off_ref, _, cnt_ref = O.ccd(ref, pairs, max_time)
    gs = scene.copy()
    ctx.set_scene(gs)
    c, off, cnt = ctx.compare_trees_full_continuous(pairs, max_time)
    assert np.array_equal(off, off_ref), "per-pair contact counts differ"
    assert_bits_equal(c, c_ref, "continuous contacts")
    assert cnt[:3].tolist() == cnt_ref.tolist(), (cnt, cnt_ref)
    ctx.get_bodies(gs)
    touched = np.unique(np.asarray(pairs).ravel())
    assert_bits_equal(gs.fut[touched], ref.fut[touched], "projected future states")
    return len(c), cnt


def np_parity(ctx, scene, pairs):
    c_ref, off_ref, cnt_ref = O.narrowphase(scene.copy(), pairs)
    ctx.set_scene(scene.copy())
    c, off, cnt = ctx.compare_trees_full(pairs)
    assert np.array_equal(off, off_ref), "per-pair contact counts differ"
    assert_bits_equal(c, c_ref, "discrete contacts")
    assert cnt[:2].tolist() == cnt_ref[:2].tolist(), (cnt, cnt_ref)
    return len(c)


def test_bucket_golden_on_gpu(ctx):
    """test_comparison.cpp:90-128 and test_continuous_comparison.cpp:222-263 through the GPU."""
    s = SmallScene()
    m_pyr = s.add_leaf_mesh(tris_from(PYRAMID_V, PYRAMID_F))
    V, F = plane_mesh(1.0)
    m_pl = s.add_leaf_mesh(tris_from(V, F))
    s.add_body(m_pyr, 0.01, cur=state(x=(0, 0, 1.0)), fut=state(x=(0, 0, 1.0)), is_static=True)
    s.add_body(m_pl, 0.01, cur=state(x=(0, 0, 1.105)), fut=state(x=(0, 0, 1.105)))
    sc = s.build().to_product()
    ctx.set_scene(sc)
    c, off, _ = ctx.compare_trees_full([[0, 1]])
    assert off.tolist() == [0, 8]
    assert len(O.filter_contacts(c, 0.0)) == 1
    assert np_parity(ctx, sc, [[0, 1]]) == 8
    # continuous: plane from z=2 to z=1 over max_time 1 with velocity -1 (toc 0.9)
    sc.cur[1] = state(x=(0, 0, 2.0), v=(0, 0, -1.0))
    n, _ = ccd_parity(ctx, sc, [[0, 1]], [1.0])
    assert n >= 1
    ctx.set_scene(sc.copy())
    c, off, _ = ctx.compare_trees_full_continuous([[0, 1]], [1.0])
    f = O.filter_contacts(c, 0.0, continuous=True)
    assert len(f) == 1 and abs(f[0, 10] - 0.9) <= 0.9 * 1.1920929e-05


def _next_level(nodes, level, used):
    """compareTreesFull's expansion of one level (full_tree_comparison.h:26-64):
    node pairs with new hits that are not leaf-leaf put the shallower inner
    side's children (b on ties) into the next level, in order."""
    nxt, last = [], 0
    for (na, nb), u in zip(level, used):
        if u > last:
            a_in, b_in = nodes[na, 2] != 0, nodes[nb, 2] != 0
            if a_in or b_in:
                adv_a = a_in and (not b_in or nodes[na, 3] < nodes[nb, 3])
                if adv_a:
                    nxt += [(nodes[na, 0] + c, nb) for c in range(nodes[na, 1])]
                else:
                    nxt += [(na, nodes[nb, 0] + c) for c in range(nodes[nb, 1])]
        last = u
    return nxt


def test_find_contacts_bucket_comparison_matches_oracle(ctx):
    """The per-level strategy entry (ContactDetectionStrategy::
    findContactsBucketComparison) against the oracle bit for bit: the
    reference's pyramid/plane case (test_comparison.cpp:90-128: 8 hits, one
    after filterContacts), then every level of two close hulls' traversal,
    driven from the host the way compareTreesFull drives it."""
    s = SmallScene()
    m_pyr = s.add_leaf_mesh(tris_from(PYRAMID_V, PYRAMID_F))
    V, F = plane_mesh(1.0)
    m_pl = s.add_leaf_mesh(tris_from(V, F))
    s.add_body(m_pyr, 0.01, cur=state(x=(0, 0, 1.0)), fut=state(x=(0, 0, 1.0)), is_static=True)
    s.add_body(m_pl, 0.01, cur=state(x=(0, 0, 1.105)), fut=state(x=(0, 0, 1.105)))
    sc = s.build().to_product()
    ctx.set_scene(sc)
    hits, used = ctx.find_contacts_bucket_comparison(0, 1, [[0, 1]])
    ref, ref_used = O.bucket_comparison(sc, 0, 1, [[0, 1]])
    assert used.tolist() == ref_used.tolist() == [8]
    assert_bits_equal(hits, ref, "golden bucket hits")
    assert len(O.filter_contacts(hits, 0.0)) == 1

    hull = project_futures(D.make_scene(2, nx=2, ny=1, nz=1, spacing=1.02, speed_sigma=1.0, seed=4))
    ctx.set_scene(hull.copy())
    a, b = 1, 2
    level = [(int(hull.mesh_node_off[hull.mesh[a]]), int(hull.mesh_node_off[hull.mesh[b]]))]
    total, levels = 0, 0
    while level:
        hits, used = ctx.find_contacts_bucket_comparison(a, b, level)
        ref, ref_used = O.bucket_comparison(hull, a, b, level)
        assert used.tolist() == ref_used.tolist(), levels
        assert_bits_equal(hits, ref, f"hull bucket hits, level {levels}")
        total += len(hits)
        levels += 1
        level = _next_level(hull.nodes, level, used)
    assert levels >= 3 and total > 0
    # an empty level, an out-of-range node and a too-small buffer
    hits, used = ctx.find_contacts_bucket_comparison(a, b, np.zeros((0, 2), np.int32))
    assert len(hits) == 0 and len(used) == 0
    with pytest.raises(D.D2GError, match="outside"):
        ctx.find_contacts_bucket_comparison(a, b, [[0, len(hull.nodes)]])
    first = [(int(hull.mesh_node_off[hull.mesh[a]]), int(hull.mesh_node_off[hull.mesh[b]]))]
    n_first = len(ctx.find_contacts_bucket_comparison(a, b, first)[0])
    if n_first > 1:
        with pytest.raises(D.CapacityError):
            ctx.find_contacts_bucket_comparison(a, b, first, capacity=1)


def test_empty_and_invalid_pairs(ctx):
    s = D.make_scene(1, nx=2, ny=1, nz=1)
    ctx.set_scene(s)
    c, off, _ = ctx.compare_trees_full_continuous(np.zeros((0, 2), np.int32), [])
    assert len(c) == 0 and off.tolist() == [0]
    with pytest.raises(D.D2GError):
        ctx.compare_trees_full_continuous([[0, 99]], [0.01])
    with pytest.raises(D.D2GError):
        ctx.compare_trees_full([[-1, 1]])


def test_capacity_reported(ctx):
    s = D.make_scene(1, nx=2, ny=1, nz=1, spacing=1.05)
    s = project_futures(s)
    ctx.set_scene(s)
    c, off, _ = ctx.compare_trees_full([[1, 2]])
    assert len(c) > 1
    with pytest.raises(D.CapacityError):
        ctx.compare_trees_full([[1, 2]], capacity=1)


def test_ccd_parity_cubes_full_scene(ctx):
    s = D.make_scene(1)
    pairs = broad_pairs(s)
    mt = np.minimum(s.last_dt[pairs[:, 0]], s.last_dt[pairs[:, 1]])
    ccd_parity(ctx, s, pairs, mt)


def test_ccd_parity_cubes_close_fast(ctx):
    """Cubes nearly touching, fast, long horizon: hits at every level and stage."""
    s = D.make_scene(1, spacing=1.12, speed_sigma=3.0, seed=7)
    pairs = broad_pairs(s)
    mt = np.full(len(pairs), 0.05)
    n, cnt = ccd_parity(ctx, s, pairs, mt)
    assert n > 100 and cnt[2] > 0


def test_ccd_parity_hulls_close(ctx):
    s = D.make_scene(2, nx=4, ny=4, nz=3, spacing=1.2, speed_sigma=2.0, seed=3)
    pairs = broad_pairs(s)
    mt = np.full(len(pairs), 0.04)
    n, cnt = ccd_parity(ctx, s, pairs, mt)
    assert n > 50 and cnt[2] > 0


def test_ccd_parity_hulls_benchmark_scene(ctx):
    """The benchmark workload itself: every broad-phase pair of the 1,024-hull scene."""
    s = D.make_scene(2)
    pairs = broad_pairs(s)
    mt = np.minimum(s.last_dt[pairs[:, 0]], s.last_dt[pairs[:, 1]])
    ccd_parity(ctx, s, pairs, mt)


def test_ccd_and_narrowphase_parity_noisy_icospheres(ctx):
    """Non-convex bodies (1,280-triangle noisy icospheres, deep trees) in the
    open box: a 2 x 2 x 2 block close together, moving fast."""
    s = project_futures(D.make_scene(5, nx=2, ny=2, nz=2, spacing=1.15, speed_sigma=2.0, seed=4))
    pairs = broad_pairs(s)
    assert len(pairs) >= 8
    mt = np.full(len(pairs), 0.01)
    n, cnt = ccd_parity(ctx, s, pairs, mt)
    assert n > 0 and cnt[2] > 0
    assert np_parity(ctx, s, pairs) > 0


def test_narrowphase_parity_cubes(ctx):
    s = project_futures(D.make_scene(1, spacing=1.12, speed_sigma=3.0, seed=5))
    pairs = broad_pairs(s)
    assert np_parity(ctx, s, pairs) > 0


def test_narrowphase_parity_hulls(ctx):
    s = project_futures(D.make_scene(2, nx=5, ny=5, nz=3, spacing=1.22, seed=11))
    pairs = broad_pairs(s)
    assert np_parity(ctx, s, pairs) > 0


def test_repeated_calls_are_identical(ctx):
    s = D.make_scene(1, spacing=1.12, speed_sigma=3.0, seed=9)
    pairs = broad_pairs(s)
    ctx.set_scene(s.copy())
    a = ctx.compare_trees_full_continuous(pairs, 0.05)[0]
    ctx.set_scene(s.copy())
    b = ctx.compare_trees_full_continuous(pairs, 0.05)[0]
    assert_bits_equal(a, b, "repeat")


WORK_SAVING_CASES = {
    # the benchmark workload: every broad-phase pair of the 1,024-hull scene
    "benchmark_hulls": lambda: (lambda s: (s, broad_pairs(s), None))(D.make_scene(2)),
    # non-convex noisy icospheres in the open box, close together and fast
    "noisy_icospheres": lambda: (lambda s: (s, broad_pairs(s), 0.01))(
        project_futures(D.make_scene(5, nx=2, ny=2, nz=2, spacing=1.15, speed_sigma=2.0, seed=4))),
    # the cube configuration, close and fast
    "cubes": lambda: (lambda s: (s, broad_pairs(s), 0.05))(D.make_scene(1, spacing=1.12, speed_sigma=3.0, seed=5)),
}


@pytest.mark.parametrize("case", sorted(WORK_SAVING_CASES))
def test_work_saving_modes_keep_the_ccd_exact(ctx, case):
    """Every work-saving mode at once, at its most aggressive: the root
    certificate on every query (the proposal at threshold 1, so the network's
    prediction does not matter) and separation witnesses, over two calls (the
    second skips node pairs the first one witnessed).  Contacts, per-pair
    offsets and projected futures equal the oracle's bit for bit."""
    s, pairs, mt = WORK_SAVING_CASES[case]()
    if mt is None:
        mt = np.minimum(s.last_dt[pairs[:, 0]], s.last_dt[pairs[:, 1]])
    mt = np.broadcast_to(np.asarray(mt, dtype=np.float64), (len(pairs),)).copy()
    ref_s = s.copy()
    ref, ref_off, _, _ = O.ccd(ref_s, pairs, mt)
    touched = np.unique(pairs.ravel())
    net = D.Mlp(ctx, seed=1)
    stats = []
    try:
        ctx.set_ccd_proposal(net, 1.0)
        ctx.set_ccd_witnesses(True)
        ctx.ccd_stats(reset=True)
        for call in range(2):
            gs = s.copy()
            ctx.set_scene(gs)
            c, off, _ = ctx.compare_trees_full_continuous(pairs, mt, capacity=1 << 22)
            stats.append(ctx.ccd_stats(reset=True))
            assert np.array_equal(off, ref_off), (case, call)
            assert_bits_equal(c, ref, f"{case}: contacts, call {call}")
            ctx.get_bodies(gs)
            assert_bits_equal(gs.fut[touched], ref_s.fut[touched], f"{case}: futures, call {call}")
    finally:
        ctx.set_ccd_proposal(None)
        ctx.set_ccd_witnesses(False)
        net.close()
    assert len(ref) > 0
    assert stats[0]["pairs_seen"] == len(pairs)
    print(case, stats)
