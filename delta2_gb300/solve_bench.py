"""Solve benchmark: SequentialImpulses::solve
(strategies/contact_force/sequential_impulses.cpp:104-638) of the largest
contact cluster of a 1,024-hull state (configuration 2 after N outer steps of
the GPU stepper), timed for each way the library can spread a cluster over
the GPU: a cooperative grid, a thread-block cluster of 16 or 8 blocks, one
block, and the library's default choice.  Every layout must give the same
statuses, iteration counts, impulses and future states, bit for bit; the tool
checks that.

  python -m delta2_gb300.solve_bench --steps 480 --save c2_480.npz
  python -m delta2_gb300.solve_bench --load c2_480.npz

The cluster's inputs are built as the stepper builds them: broad phase,
cluster separation, discrete narrow phase and filterContacts on the GPU, the
per-pair contact counts, no warm start, the scene's optimal time step.
"""
import argparse
import json
import time

import numpy as np

import delta2_gb300 as D

LAYOUTS = {
    "default": {},
    "grid": {D.TUNE_GRID_MIN_PARTS: 0},
    "cluster16": {D.TUNE_GRID_MIN_PARTS: 1 << 30, D.TUNE_SOLVE_CLUSTER: 16},
    "cluster8": {D.TUNE_GRID_MIN_PARTS: 1 << 30, D.TUNE_SOLVE_CLUSTER: 8},
    "block": {D.TUNE_GRID_MIN_PARTS: 1 << 30, D.TUNE_SOLVE_CLUSTER: 1},
}
STATE_FIELDS = ["cur", "fut", "last", "last_dt", "sleep_steps", "sleeping"]


def late_state(steps, seed=0, load=None, save=None):
    """The configuration-2 scene after `steps` GPU outer steps (or loaded)."""
    base = D.make_scene(2, seed=seed)
    if load:
        z = np.load(load)
        for k in STATE_FIELDS:
            getattr(base, k)[...] = z[k]
        return base
    ctx = D.Context(0)
    try:
        ctx.set_scene(base.copy())
        ctx.world_configure(base)
        ctx.world_step(steps)
        state = ctx.get_bodies(base.copy())
    finally:
        ctx.close()
    if save:
        np.savez(save, **{k: getattr(state, k) for k in STATE_FIELDS})
    return state


def largest_cluster(ctx, base):
    """(particles, step, contacts, pair counts, warm) of the cluster with the
    most contacts after the narrow phase and filter."""
    ctx.set_scene(base.copy())
    pairs = ctx.broad_phase_device(base)
    clusters = ctx.separate_clusters(pairs)
    ctx.set_scene(base.copy())  # the separation rolls the device states back
    flat = np.concatenate([c[1] for c in clusters]).reshape(-1, 2) if clusters else np.zeros((0, 2), np.int32)
    raw, off, _ = ctx.compare_trees_full(flat)
    kept, koff = ctx.filter_contacts(raw, off)
    step = float(np.float32(base.opt_dt))
    best, k = None, 0
    for parts, inter, _, _, _ in clusters:
        h = kept[koff[k]:koff[k + len(inter)]]
        k += len(inter)
        if best is None or len(h) > len(best[2]):
            keys = [tuple(sorted((int(r[11]), int(r[12])))) for r in h]
            counts = {}
            for kk in keys:
                counts[kk] = counts.get(kk, 0) + 1
            best = (parts, step, h, [counts[kk] for kk in keys], np.full(len(h), np.nan))
    return best


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--steps", type=int, default=480, help="GPU outer steps before the solve")
    p.add_argument("--seed", type=int, default=0)
    p.add_argument("--load", help="state file written by --save (skips the stepping)")
    p.add_argument("--save", help="write the state after the stepping to this .npz file")
    p.add_argument("--layouts", default="default,grid,cluster16,cluster8,block")
    p.add_argument("--reps", type=int, default=3)
    a = p.parse_args()
    from delta2_gb300 import build as B

    B.build()
    base = late_state(a.steps, a.seed, a.load, a.save)
    ctx = D.Context(0)
    try:
        cluster = largest_cluster(ctx, base)
        parts, _, con, _, _ = cluster
        ref = None
        for name in a.layouts.split(","):
            saved = {key: ctx.get_tuning(key) for key in LAYOUTS[name]}
            for key, v in LAYOUTS[name].items():
                ctx.set_tuning(key, v)
            ms = []
            for _ in range(a.reps):
                ctx.set_scene(base.copy())
                t0 = time.perf_counter()
                status, iters, imps, _ = ctx.solve_clusters([cluster], base.gravity_z)
                ms.append((time.perf_counter() - t0) * 1e3)
            fut = ctx.get_bodies(base.copy()).fut
            got = (int(status[0]), tuple(int(x) for x in iters[0]), np.ascontiguousarray(imps[0]).view(np.uint64),
                   np.ascontiguousarray(fut).view(np.uint64))
            if ref is None:
                ref = got
            elif not (got[0] == ref[0] and got[1] == ref[1] and np.array_equal(got[2], ref[2]) and
                      np.array_equal(got[3], ref[3])):
                raise SystemExit(f"layout {name} changed the solve's results")
            for key, v in saved.items():
                ctx.set_tuning(key, v)
            print(json.dumps({"layout": name, "ms": [round(x, 2) for x in ms], "parts": len(parts),
                              "contacts": int(len(con)), "iterations": list(got[1]), "status": got[0],
                              "solved_by": ctx.solve_layout()}), flush=True)
    finally:
        ctx.close()


if __name__ == "__main__":
    main()
