"""GPU time-step selection against the oracle (bit for bit): the clamped step
of every cluster and the future states the CCD queries leave on the bodies."""
import numpy as np
import pytest

import delta2_gb300 as D
from oracle import oracle as O
from tests.clusters import separate

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(gpu_required):
    from delta2_gb300 import build as B
    B.build()
    c = D.Context(0)
    yield c
    c.close()


def run_case(ctx, scene, last_dt):
    scene.last_dt[:] = last_dt
    pairs = D.broad_phase(scene)
    clusters = separate(pairs, scene.is_static, scene.n_bodies)
    assert clusters
    ref_scene = scene.copy()
    w = O.World(ref_scene, scene.opt_dt)
    ref_steps = [w.select_dt(parts, inter) for parts, inter in clusters]
    w.get_bodies()
    flat = np.array([p for _, inter in clusters for p in inter], dtype=np.int32).reshape(-1, 2)
    gs = scene.copy()
    ctx.set_scene(gs)
    steps, cnt = ctx.select_time_steps(flat, [(parts, len(inter)) for parts, inter in clusters], scene.opt_dt)
    ctx.get_bodies(gs)
    assert np.array_equal(steps.view(np.uint64), np.array(ref_steps).view(np.uint64)), (steps, ref_steps)
    touched = np.unique(flat.ravel())
    assert np.array_equal(gs.fut[touched].view(np.uint64), ref_scene.fut[touched].view(np.uint64))
    return steps, len(clusters)


def test_select_steps_cubes_one_cluster(ctx):
    s = D.make_scene(1, spacing=1.12, speed_sigma=3.0, seed=2)
    steps, nc = run_case(ctx, s, np.float64(np.float32(s.opt_dt)))
    assert nc >= 1


def test_select_steps_many_clusters_long_horizon(ctx):
    # widely spaced hulls: many small clusters, long horizon so contacts restrict steps
    s = D.make_scene(2, nx=6, ny=6, nz=2, spacing=1.6, speed_sigma=4.0, seed=4, dt=0.05)
    steps, nc = run_case(ctx, s, 0.05)
    assert nc > 3
    assert np.any(steps < s.opt_dt)  # some cluster's step is cut by its contacts


def test_select_steps_benchmark_scene(ctx):
    s = D.make_scene(2)
    run_case(ctx, s, np.float64(np.float32(s.opt_dt)))
