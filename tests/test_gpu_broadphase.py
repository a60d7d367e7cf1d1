"""The GPU broad phase and cluster separation against the oracle and the
Python restatement: identical pair sets (ascending), clusters, particle and
interaction order, minimum times and steps."""
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


def advanced(kw, steps):
    """A scene advanced by the oracle stepper, so clusters sit at different
    times and the swept-sphere test interpolates."""
    s = D.make_scene(**kw)
    if steps:
        w = O.World(s.copy(), s.opt_dt, s.gravity_z)
        assert w.step(steps) == 0
        s = w.get_bodies().copy()
    return s


CASES = [
    ("cubes", dict(config=1, nx=3, ny=3, nz=2), 60),
    ("hulls", dict(config=2, nx=3, ny=3, nz=2, spacing=1.6, speed_sigma=2.0, seed=5), 25),
    ("mixed", dict(config=3, nx=3, ny=3, nz=2), 8),
    ("benchmark", dict(config=2), 0),
]


@pytest.mark.parametrize("name,kw,steps", CASES, ids=[c[0] for c in CASES])
def test_broad_phase_matches_oracle(ctx, name, kw, steps):
    s = advanced(kw, steps)
    ctx.set_scene(s.copy())
    got = ctx.broad_phase_device(s)
    ref = O.World(s.copy(), s.opt_dt, s.gravity_z).broad_phase()
    assert len(ref) > 0
    assert np.array_equal(got, ref)
    assert np.array_equal(got, D.broad_phase(s))
    if steps:
        moving = s.is_static == 0
        assert len(np.unique(s.cur[moving, 0])) >= 1


@pytest.mark.parametrize("name,kw,steps", CASES, ids=[c[0] for c in CASES])
def test_clusters_match_restatement(ctx, name, kw, steps):
    s = advanced(kw, steps)
    ctx.set_scene(s.copy())
    pairs = D.broad_phase(s)
    got = ctx.separate_clusters(pairs)
    ref = separate(pairs, s.is_static, s.n_bodies)
    assert len(got) == len(ref)
    for (gp, gi, mct, step, sl), (rp, ri) in zip(got, ref):
        assert gp == [int(x) for x in rp]
        assert [tuple(x) for x in gi.tolist()] == [tuple(map(int, x)) for x in ri]
        dyn = [p for p in rp if not s.is_static[p]]
        assert mct == min(s.cur[p, 0] for p in dyn)
        assert step == min(s.last_dt[p] for p in dyn)
        assert sl == all(bool(s.sleeping[p]) for p in dyn)
