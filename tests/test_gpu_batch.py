"""Batched scenes: independent scenes stepped in one context, each bit for
bit equal to the oracle stepping that scene alone."""
import numpy as np
import pytest

import delta2_gb300 as D
from oracle import oracle as O

pytestmark = pytest.mark.gpu

FIELDS = ["last", "cur", "fut", "last_dt", "sleep_steps", "sleeping"]


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


def test_batched_broad_phase_is_the_union_of_the_scenes(ctx):
    batch, scene_of, scenes = D.make_batch(5, seed=2, min_bodies=8, max_bodies=40)
    ctx.set_scene(batch)
    ctx.set_scenes(scene_of)
    got = ctx.broad_phase_device(batch)
    base = np.concatenate([[0], np.cumsum([s.n_bodies for s in scenes])])
    ref = np.concatenate([D.broad_phase(s) + base[k] for k, s in enumerate(scenes)])
    assert len(ref) > 0
    assert np.array_equal(got, ref)


def test_batched_world_matches_each_scene_alone(ctx):
    batch, scene_of, scenes = D.make_batch(3, seed=1, min_bodies=8, max_bodies=24)
    ctx.set_scene(batch.copy())
    ctx.set_scenes(scene_of)
    ctx.world_configure(batch)
    refs = [O.World(s.copy(), s.opt_dt, s.gravity_z) for s in scenes]
    got = batch.copy()
    for step in range(60):
        ctx.world_step(1)
        for w in refs:
            assert w.step(1) == 0
        if step % 5 == 4 or step == 59:
            ctx.get_bodies(got)
            for k, w in enumerate(refs):
                part = D.split_bodies(got, scene_of, k)
                ref = w.get_bodies()
                for f in FIELDS:
                    assert np.array_equal(bits(getattr(part, f)), bits(getattr(ref, f))), (step, k, f)
    total = {}
    for w in refs:
        for key, v in w.stats().items():
            total[key] = total.get(key, 0) + v
    assert ctx.world_stats() == total
    assert total["np_contacts"] > 0
