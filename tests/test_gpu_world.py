"""The GPU contact filter, sequential-impulse solve and adaptive cluster
stepper against the oracle, bit for bit: every body state after every outer
step, the statistics and the warm-start store."""
import numpy as np
import pytest

import delta2_gb300 as D
from oracle import oracle as O
from tests.clusters import separate

pytestmark = pytest.mark.gpu

BODY_FIELDS = ["last", "cur", "fut", "last_dt", "sleep_steps", "sleeping"]


@pytest.fixture(scope="module")
def ctx(gpu_required):
    from delta2_gb300 import build as B
    B.build()
    c = D.Context(0)
    yield c
    c.close()


def bits(a):
    a = np.ascontiguousarray(a)
    return a.view(np.uint64) if a.dtype == np.float64 else a


def assert_bodies_equal(got, ref, where):
    for f in BODY_FIELDS:
        g, r = bits(getattr(got, f)), bits(getattr(ref, f))
        if not np.array_equal(g, r):
            bad = np.nonzero((g != r).reshape(len(g), -1).any(axis=1))[0]
            raise AssertionError(f"{where}: field {f} differs for bodies {bad[:10].tolist()}: "
                                 f"gpu {getattr(got, f)[bad[0]]} oracle {getattr(ref, f)[bad[0]]}")


def run_world(ctx, scene, steps, skip_stats=()):
    ref = O.World(scene.copy(), scene.opt_dt, scene.gravity_z)
    gs = scene.copy()
    ctx.set_scene(gs)
    ctx.world_configure(gs)
    for i in range(steps):
        assert ref.step(1) == 0
        ctx.world_step(1)
        assert_bodies_equal(ctx.get_bodies(gs), ref.get_bodies(), f"after step {i + 1}")
    ref_stats = {k: v for k, v in ref.stats().items() if k not in skip_stats}
    got_stats = {k: v for k, v in ctx.world_stats().items() if k not in skip_stats}
    assert got_stats == ref_stats
    assert {k: np.float64(v).view(np.uint64) for k, v in ctx.world_warm().items()} == \
        {k: np.float64(v).view(np.uint64) for k, v in ref.warm().items()}
    return got_stats


def test_world_cubes_with_rollbacks(ctx):
    # 8 cubes falling onto the ground and each other; the solver rejects
    # steps (rollback and step halving in stepRecursive) from about step 90
    s = D.make_scene(1, nx=2, ny=2, nz=2)
    st = run_world(ctx, s, 140)
    assert st["np_contacts"] > 0 and st["failures"] > 0


def test_world_hulls(ctx):
    s = D.make_scene(2, nx=2, ny=2, nz=1)
    st = run_world(ctx, s, 110)
    assert st["np_contacts"] > 0


def test_world_sleeping_clusters_share_the_ground(ctx):
    # Weightless, motionless cubes hovering 0.4 m over the ground: each is a
    # cluster with the ground (broad-phase pair, no contact), and after 20
    # stationary steps every cluster sleeps, so the ground's clock advances
    # once per sleeping cluster.
    s = D.make_scene(1, nx=2, ny=2, nz=1, spacing=3.0, speed_sigma=0.0, gravity_z=0.0)
    for arr in (s.last, s.cur, s.fut):
        arr[1:, 1:5] = [1.0, 0.0, 0.0, 0.0]
        arr[1:, 10] = 0.9
        arr[1:, 11:14] = 0.0
        arr[1:, 5:8] = 0.0
    st = run_world(ctx, s, 30)
    got = ctx.get_bodies(s.copy())
    assert got.sleeping[1:].all()
    assert st["np_contacts"] == 0


def test_filter_matches_oracle(ctx):
    s = D.make_scene(2, nx=3, ny=3, nz=1, spacing=1.25, speed_sigma=0.0)
    pairs = D.broad_phase(s)
    ctx.set_scene(s.copy())
    con, off, _ = ctx.compare_trees_full(pairs)
    assert len(con) > 0
    kept, koff = ctx.filter_contacts(con, off)
    for p in range(len(pairs)):
        ref = O.filter_contacts(con[off[p]:off[p + 1]])
        got = kept[koff[p]:koff[p + 1]]
        assert np.array_equal(bits(got), bits(np.asarray(ref).reshape(-1, 14))), p


def solve_against_oracle(ctx, base, s, min_contacts=1):
    """Solve every cluster of state `base` (contacts from the oracle's narrow
    phase and filter) on the GPU in one call and with the oracle cluster by
    cluster; compare statuses, iterations, future states and the warm store."""
    pairs = D.broad_phase(base)
    clusters = separate(pairs, base.is_static, base.n_bodies)
    flat = np.array([p for _, inter in clusters for p in inter], dtype=np.int32).reshape(-1, 2)
    raw, off = O.narrowphase(base, flat)[:2]
    hits, k = [], 0
    for parts, inter in clusters:
        cl = []
        for _ in inter:
            f = np.asarray(O.filter_contacts(raw[off[k]:off[k + 1]])).reshape(-1, 14)
            cl.append(f)
            k += 1
        hits.append(np.concatenate(cl) if cl else np.zeros((0, 14)))
    assert sum(len(h) for h in hits) >= min_contacts
    step = float(np.float32(s.opt_dt))
    # oracle: one cluster after another, its warm store empty
    ref_world = O.World(base.copy(), s.opt_dt, s.gravity_z)
    ref_res = [ref_world.solve(parts, step, h) for (parts, _), h in zip(clusters, hits)]
    ref_b = ref_world.get_bodies()
    # GPU: all clusters in one call
    gs = base.copy()
    ctx.set_scene(gs)
    inputs = []
    for (parts, _), h in zip(clusters, hits):
        keys = [tuple(sorted((int(r[11]), int(r[12])))) for r in h]
        cnt = [keys.count(kk) for kk in keys]
        inputs.append((parts, step, h, cnt, np.full(len(h), np.nan)))
    status, iters, imps, abs_ = ctx.solve_clusters(inputs, s.gravity_z)
    got = ctx.get_bodies(gs)
    for i, (ok, it) in enumerate(ref_res):
        assert status[i] == (0 if ok else 1)
        if ok:
            assert tuple(iters[i]) == tuple(it)
    assert np.array_equal(bits(got.fut), bits(ref_b.fut))
    # the warm-start store: last contact of each pair in sorted order
    warm = {}
    for imp, ab, ok in zip(imps, abs_, status):
        if ok != 0:
            continue
        seen = {}
        for x, (a, b) in zip(imp, ab):
            key = (min(a, b), max(a, b))
            seen[key] = (x if key in seen else 0.0 + x)
        warm.update(seen)
    ref_warm = ref_world.warm()
    assert {k: np.float64(v).view(np.uint64) for k, v in warm.items()} == \
        {k: np.float64(v).view(np.uint64) for k, v in ref_warm.items()}
    return clusters, hits


@pytest.mark.parametrize("lanes", [0, 4, 16])
def test_solve_matches_oracle(ctx, lanes):
    # a state with many contacts: the cube scene after 120 oracle steps; the
    # normal-impulse waves on four or sixteen lanes per contact, or chosen by
    # wave width
    s = D.make_scene(1, nx=2, ny=2, nz=2)
    w = O.World(s.copy(), s.opt_dt, s.gravity_z)
    w.step(120)
    ctx.set_tuning(D.TUNE_SOLVE_LANES, lanes)
    try:
        solve_against_oracle(ctx, w.get_bodies().copy(), s)
    finally:
        ctx.set_tuning(D.TUNE_SOLVE_LANES, 0)


@pytest.mark.parametrize("grid_min_parts, solve_cluster, lanes", [
    (128, 0, 4), (128, 0, 16), (1000000, 16, 4), (1000000, 16, 16), (1000000, 2, 0), (1000000, 1, 0)],
    ids=["grid-4", "grid-16", "cluster16-4", "cluster16-16", "cluster2", "block"])
def test_solve_wide_cluster_matches_oracle(ctx, grid_min_parts, solve_cluster, lanes):
    # 144 axis-aligned unit cubes 1 cm apart and 1 cm above the ground, falling
    # at 0.5 m/s: one cluster of 144 moving bodies with hundreds of contacts,
    # solved by the cooperative grid (part threshold below 145), by a
    # thread-block cluster of 16 or 2 blocks, or by one block, with four or
    # sixteen lanes per contact (0: by wave width)
    defaults = {k: ctx.get_tuning(k) for k in (D.TUNE_GRID_MIN_PARTS, D.TUNE_SOLVE_CLUSTER, D.TUNE_SOLVE_LANES)}
    ctx.set_tuning(D.TUNE_GRID_MIN_PARTS, grid_min_parts)
    ctx.set_tuning(D.TUNE_SOLVE_CLUSTER, solve_cluster)
    ctx.set_tuning(D.TUNE_SOLVE_LANES, lanes)
    s = _wide_cluster_scene()
    try:
        clusters, hits = solve_against_oracle(ctx, s.copy(), s, min_contacts=128)
        layout = ctx.solve_layout()
    finally:
        for k, v in defaults.items():
            ctx.set_tuning(k, v)
    # the cluster took the layout the settings ask for
    if grid_min_parts == 128:
        assert layout["grid"] == 1, layout
    elif solve_cluster == 1:
        assert layout["block"] == 1, layout
    else:
        assert layout["thread_block_cluster"] == 1 and layout["cluster_size"] == solve_cluster, layout
    assert max(len(parts) for parts, _ in clusters) > 128
    assert max(len(h) for h in hits) >= 128


def test_solve_several_thread_block_clusters_in_one_launch(ctx):
    """Two piles of 72 touching cubes, 4 m apart: two clusters of hundreds of
    contacts solved by one launch of 16-block thread-block clusters (fixed
    size, then the automatic choice), bit for bit against the oracle."""
    s = _wide_cluster_scene()
    far = s.cur[:, 9] > 0.0  # the cubes of the upper half in y (index 0 is the ground)
    far[0] = False
    for arr in (s.cur, s.fut, s.last):
        arr[far, 9] += 4.0
    defaults = {k: ctx.get_tuning(k) for k in (D.TUNE_GRID_MIN_PARTS, D.TUNE_SOLVE_CLUSTER)}
    try:
        for size in (16, 0):
            ctx.set_tuning(D.TUNE_GRID_MIN_PARTS, 1000000)
            ctx.set_tuning(D.TUNE_SOLVE_CLUSTER, size)
            clusters, hits = solve_against_oracle(ctx, s.copy(), s, min_contacts=256)
            layout = ctx.solve_layout()
            big = sum(1 for h in hits if len(h) >= 32)
            assert big == 2, [len(h) for h in hits]
            assert layout["thread_block_cluster"] == 2 and layout["cluster_size"] >= 2, layout
            if size:
                assert layout["cluster_size"] == size, layout
    finally:
        for k, v in defaults.items():
            ctx.set_tuning(k, v)


def _wide_cluster_scene():
    # 144 axis-aligned unit cubes 1 cm apart and 1 cm above the ground, falling at 0.5 m/s
    s = D.make_scene(1, nx=12, ny=12, nz=1, spacing=1.01, speed_sigma=0.0)
    s.cur[1:, 1:5] = [1.0, 0.0, 0.0, 0.0]
    s.cur[1:, 10] = 0.51
    s.cur[1:, 11:14] = [0.0, 0.0, -0.5]
    s.fut[1:] = s.cur[1:]
    s.last[1:] = s.cur[1:]
    return s


def test_grid_barrier_wait_runs_out_then_the_context_recovers(ctx):
    """The cooperative-grid solve's barrier waits are bounded.  With a limit
    of one poll a block gives up at some barrier of the wide cluster's solve
    (all blocks still arrive, so every wait ends): the call returns
    D2G_SPIN_LIMIT.  The next solve on the same context, with the default
    limit and the states uploaded again, matches the oracle bit for bit."""
    s = _wide_cluster_scene()
    pairs = D.broad_phase(s)
    clusters = separate(pairs, s.is_static, s.n_bodies)
    flat = np.array([p for _, inter in clusters for p in inter], dtype=np.int32).reshape(-1, 2)
    raw, off = O.narrowphase(s, flat)[:2]
    inputs, k = [], 0
    for parts, inter in clusters:
        h = np.concatenate([np.asarray(O.filter_contacts(raw[off[k + i]:off[k + i + 1]])).reshape(-1, 14)
                            for i in range(len(inter))])
        k += len(inter)
        keys = [tuple(sorted((int(r[11]), int(r[12])))) for r in h]
        inputs.append((parts, float(np.float32(s.opt_dt)), h, [keys.count(kk) for kk in keys],
                       np.full(len(h), np.nan)))
    assert max(len(h) for _, _, h, _, _ in inputs) >= 128
    default = ctx.get_tuning(D.TUNE_SPIN_LIMIT)
    assert default == 1 << 25
    parts_default = ctx.get_tuning(D.TUNE_GRID_MIN_PARTS)
    ctx.set_scene(s.copy())
    ctx.set_tuning(D.TUNE_GRID_MIN_PARTS, 64)  # the 145-part cluster takes the grid
    ctx.set_tuning(D.TUNE_SPIN_LIMIT, 1)
    try:
        with pytest.raises(D.D2GError, match="grid barrier") as e:
            ctx.solve_clusters(inputs, s.gravity_z)
        assert e.value.code == 3  # D2G_SPIN_LIMIT
    finally:
        ctx.set_tuning(D.TUNE_SPIN_LIMIT, default)
    try:
        solve_against_oracle(ctx, s.copy(), s, min_contacts=128)
    finally:
        ctx.set_tuning(D.TUNE_GRID_MIN_PARTS, parts_default)


def test_ee_first_iters_do_not_change_results(ctx):
    # the edge-edge split point is a launch-shape setting: every value gives
    # the same contacts, bit for bit
    s = D.make_scene(2, nx=4, ny=4, nz=4, speed_sigma=2.0, seed=9)
    pairs = D.broad_phase(s)
    mt = np.full(len(pairs), np.float64(np.float32(s.opt_dt)) * 4)
    outs = []
    try:
        for v in (0, 1, 2, 3, 10):
            ctx.set_scene(s.copy())
            ctx.set_tuning(D.TUNE_EE_FIRST_ITERS, v)
            outs.append(ctx.compare_trees_full_continuous(pairs, mt))
    finally:
        ctx.set_tuning(D.TUNE_EE_FIRST_ITERS, 2)
    assert len(outs[0][0]) > 0
    for o in outs[1:]:
        for a, b in zip(outs[0], o):
            assert np.array_equal(bits(np.asarray(a)), bits(np.asarray(b)))


def test_ccd_certificates_do_not_change_results(ctx):
    """The conservative-advancement cut-off of edge-edge CCD tests gives the
    same contacts, bit for bit, as running every test to its end, and as the
    oracle; it does cut tests on a hull scene in motion."""
    s = D.make_scene(2, nx=4, ny=4, nz=4, spacing=1.3, speed_sigma=2.0, seed=9)
    pairs = D.broad_phase(s)
    mt = np.full(len(pairs), np.float64(np.float32(s.opt_dt)) * 4)
    ref = O.ccd(s.copy(), pairs, mt)
    out = {}
    try:
        for mode in (True, False):
            ctx.set_scene(s.copy())
            ctx.set_ccd_certificates(mode)
            ctx.ccd_stats(reset=True)
            out[mode] = ctx.compare_trees_full_continuous(pairs, mt, capacity=1 << 20)
            out[(mode, "stats")] = ctx.ccd_stats(reset=True)
    finally:
        ctx.set_ccd_certificates(True)
    for mode in (True, False):
        c, off, cnt = out[mode]
        assert np.array_equal(off, ref[1])
        assert np.array_equal(bits(c), bits(ref[0]))
    assert len(ref[0]) > 0
    assert out[(True, "stats")]["ee_tests_cut"] > 0 and out[(True, "stats")]["newton_iters_saved"] > 0
    assert out[(False, "stats")]["ee_tests_cut"] == 0


def test_separation_witnesses_keep_the_stepper_exact(ctx):
    """Separation witnesses on: the stepper over 100 outer steps of a hull
    scene equals the oracle in every body state after every step, and in its
    statistics and warm-start store; the witnesses do skip node pairs (their
    counters), and a repeated CCD call skips node pairs the first one
    witnessed while giving the same contacts."""
    s = D.make_scene(2, nx=3, ny=2, nz=2, spacing=1.3, speed_sigma=1.0, seed=21)
    ctx.set_ccd_witnesses(True)
    try:
        ctx.ccd_stats(reset=True)
        # (skipped node pairs test no primitive pairs: only that counter may differ)
        run_world(ctx, s, 100, skip_stats=("ccd_tri_pairs",))
        st = ctx.ccd_stats(reset=True)
        assert st["witnesses_written"] > 0 and st["node_pairs_witnessed"] > 0
        pairs = D.broad_phase(s)
        mt = np.full(len(pairs), np.float64(np.float32(s.opt_dt)) * 2)
        ref = O.ccd(s.copy(), pairs, mt)
        first, second = [], []
        for out in (first, second):
            ctx.set_scene(s.copy())
            ctx.ccd_stats(reset=True)
            out.append(ctx.compare_trees_full_continuous(pairs, mt, capacity=1 << 20))
            out.append(ctx.ccd_stats(reset=True))
        for c, off, _ in (first[0], second[0]):
            assert np.array_equal(off, ref[1])
            assert np.array_equal(bits(c), bits(ref[0]))
        assert second[1]["node_pairs_witnessed"] > 0
    finally:
        ctx.set_ccd_witnesses(False)


def test_fp32_bounds_do_not_change_results(ctx):
    # the FP64-exact mode (every primitive test in FP64) and the default FP32
    # candidate bounds give the same contacts, bit for bit
    s = D.make_scene(2, nx=4, ny=4, nz=4, speed_sigma=2.0, seed=9)
    pairs = D.broad_phase(s)
    mt = np.full(len(pairs), np.float64(np.float32(s.opt_dt)) * 4)
    out = {}
    for mode in (True, False):
        ctx.set_scene(s.copy())
        ctx.set_fp32_bounds(mode)
        c1, o1, k1 = ctx.compare_trees_full_continuous(pairs, mt)
        c2, o2, k2 = ctx.compare_trees_full(pairs)
        out[mode] = (c1, o1, k1, c2, o2, k2)
    ctx.set_fp32_bounds(True)
    for a, b in zip(out[True], out[False]):
        assert np.array_equal(bits(np.asarray(a)), bits(np.asarray(b)))
    assert len(out[True][0]) > 0 and len(out[True][3]) > 0


def test_world_noisy_icospheres_in_open_box(ctx):
    # The noisy-icosphere configuration at small size: four non-convex bodies
    # (icospheres of 1,280 triangles with radial noise) in the static open
    # box; two start beside opposite walls moving towards them, two beside
    # each other, all just above the floor.
    s = D.make_scene(5, nx=2, ny=2, nz=1)
    assert s.n_bodies == 5 and s.is_static[0] == 1 and s.ntris[s.mesh_node_off[1]:].max() <= 8
    br = s.bounding_radius
    s.cur[1, 8], s.cur[1, 11] = -20.0 + br[1] + 0.05, -0.5
    s.cur[2, 8], s.cur[2, 11] = 20.0 - br[2] - 0.05, 0.5
    st = run_world(ctx, s, 60)
    assert st["np_contacts"] > 0
    got = ctx.get_bodies(s.copy())
    assert np.isfinite(got.cur).all()


def test_world_cube_pile(ctx):
    # the 64-cube configuration: the bodies land and pile into one cluster
    # with hundreds of contacts (65 parts: the cooperative grid solves it,
    # above the default part threshold of 64)
    s = D.make_scene(1)
    st = run_world(ctx, s, 100)
    assert st["np_contacts"] > 0


def test_chunked_traversals_match_unchunked(ctx):
    # a level budget far below the calls' needs makes both traversals run in
    # pair chunks (abandoned and halved until a level fits); the contacts are
    # the same bits as one unchunked call
    s = D.make_scene(2, nx=4, ny=4, nz=4, speed_sigma=2.0, seed=9)
    pairs = D.broad_phase(s)
    mt = np.full(len(pairs), np.float64(np.float32(s.opt_dt)) * 4)
    out = {}
    try:
        for budget in (0, 200_000):
            ctx.set_level_budget(budget)
            ctx.set_scene(s.copy())
            c1, o1, k1 = ctx.compare_trees_full_continuous(pairs, mt)
            c2, o2, k2 = ctx.compare_trees_full(pairs)
            out[budget] = (c1, o1, c2, o2)
    finally:
        ctx.set_level_budget(0)
    assert len(out[0][0]) > 0 and len(out[0][2]) > 0
    for a, b in zip(out[0], out[200_000]):
        assert np.array_equal(bits(np.asarray(a)), bits(np.asarray(b)))


def test_world_chunked_matches_oracle(ctx):
    s = D.make_scene(1, nx=2, ny=2, nz=2)
    try:
        ctx.set_level_budget(100_000)
        st = run_world(ctx, s, 100)
    finally:
        ctx.set_level_budget(0)
    assert st["np_contacts"] > 0


def test_world_obj_scene_matches_oracle(ctx, tmp_path):
    # a scene of the caller's meshes: three OBJ cubes dropped onto an OBJ plane
    from tests.test_host_setup import CUBE_F, CUBE_V, _write_obj

    _write_obj(tmp_path / "cube.obj", [[0.4 * c for c in v] for v in CUBE_V], CUBE_F)
    _write_obj(tmp_path / "plane.obj", [[20, 20, 0], [20, -20, 0], [-20, 20, 0], [-20, -20, 0]],
               [[0, 2, 1], [1, 2, 3]])
    b = D.SceneBuilder(dt=1 / 120)
    plane, _ = b.add_mesh(*D.load_obj(tmp_path / "plane.obj"), surface=True)
    cube, _ = b.add_mesh(*D.load_obj(tmp_path / "cube.obj"))
    b.add_body(plane, static=True, geo_eps=0.1)
    s2 = np.sqrt(0.5)
    for k, (x, z) in enumerate([(0.0, 0.6), (0.5, 1.6), (-0.4, 2.7)]):
        b.add_body(cube, position=(x, 0.1 * k, z), quaternion=(s2, s2, 0, 0) if k == 1 else (1, 0, 0, 0),
                   velocity=(0, 0, -0.5), geo_eps=0.1)
    s = b.finish()
    st = run_world(ctx, s, 80)
    assert st["np_contacts"] > 0
