"""The benchmark's CPU arms (CPU only, no GPU).

bench.py times the oracle restatement as the reference's CPU path: on one
core (`cpu_baseline`) and on every host core (`--impl reference`).  These
tests check what those timed regions contain: the host-tuned build of the
oracle gives the same contacts, bit for bit, as the portable checker build,
and no scene is copied inside the timed chunk loops (every CCD query
re-projects the futures from the current states, so one resident scene
serves every call).  The late-window stepper baseline restarts the oracle
from a state and warm-start store taken from another run: stepping from that
snapshot must continue the run exactly.
"""
import numpy as np

import bench
import delta2_gb300 as D
from oracle import oracle as O


def _sample():
    scene, pairs, mt = bench.build_workload(0)
    idx = np.arange(0, len(pairs), 9)  # a strided sample of the benchmark step with contact-bearing pairs
    return scene, pairs[idx], mt[idx]


def test_fast_build_matches_checker_bitwise_on_bench_workload():
    scene, pairs, mt = _sample()
    O.select_build("checker")
    ref, off, _, cnt = O.ccd(scene.copy(), pairs, mt)
    try:
        O.select_build("fast")
        got, off2, _, cnt2 = O.ccd(scene.copy(), pairs, mt)
    finally:
        O.select_build("checker")
    assert len(ref) > 1000
    assert np.array_equal(off, off2) and np.array_equal(cnt, cnt2)
    assert np.array_equal(ref.view(np.uint64), got.view(np.uint64))


def test_repeated_queries_on_one_scene_match_fresh_copies():
    """The reason the timed loops need no copy: a query leaves the scene so
    that the same query again gives the same contacts."""
    scene, pairs, mt = _sample()
    sc = scene.copy()
    first = O.ccd(sc, pairs, mt)[0]
    again = O.ccd(sc, pairs, mt)[0]
    fresh = O.ccd(scene.copy(), pairs, mt)[0]
    assert np.array_equal(first.view(np.uint64), again.view(np.uint64))
    assert np.array_equal(first.view(np.uint64), fresh.view(np.uint64))


def test_timed_cpu_loops_copy_no_scene(monkeypatch):
    scene, pairs, mt = _sample()
    copies = []
    orig = D.Scene.copy

    def counting_copy(self):
        copies.append(1)
        return orig(self)

    monkeypatch.setattr(D.Scene, "copy", counting_copy)
    cpu = bench.cpu_baseline(scene, pairs, mt, budget_s=0.5)
    assert cpu["value"] > 0 and cpu["sample"].startswith(f"{int(cpu['sample'].split()[0])} pair-queries")
    assert len(copies) == 1  # the one resident scene, made before the timed loop

    copies.clear()
    bench._worker_init(scene, pairs, mt)
    n = len(pairs)
    done = sum(bench._worker_run(np.arange(k, n, 16)) for k in range(16))
    assert done == n
    assert copies == []


def test_stepper_restarts_exactly_from_a_snapshot():
    """Two oracle worlds: one steps 4 times; the other starts from the
    first's bodies and warm-start store after 2 steps and steps 2 times."""
    s = D.make_scene(1, nx=2, ny=2, nz=1, spacing=1.12, speed_sigma=1.0, seed=3)
    w = O.World(s.copy(), s.opt_dt, s.gravity_z)
    assert w.step(2) == 0
    snap = w.get_bodies().copy()
    warm = w.warm()
    assert warm, "the snapshot should carry warm-start impulses"
    assert w.step(2) == 0
    end = w.get_bodies()
    w2 = O.World(snap, snap.opt_dt, snap.gravity_z)
    w2.set_warm(warm)
    assert w2.warm() == warm
    assert w2.step(2) == 0
    end2 = w2.get_bodies()
    for k in ["last", "cur", "fut", "last_dt"]:
        assert np.array_equal(getattr(end, k).view(np.uint64), getattr(end2, k).view(np.uint64)), k
