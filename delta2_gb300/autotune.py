"""Launch-shape autotuner: measures the context settings that change only
how the work is spread over the GPU (``d2g_ctx_set_tuning``) on a workload,
checks that every candidate gives bit-identical results, and writes the
fastest settings to a JSON file that ``Context.apply_tuning`` (and bench.py)
applies.

  python -m delta2_gb300.autotune --out delta2_gb300/tuning/gb300.json

Settings and their workloads:
  ee_first_iters   Newton iterations an edge-edge CCD test runs on one lane
                   before the tests still running continue on four lanes;
                   timed on the CCD step of the 1,024-hull scene (every
                   broad-phase pair, max_time = min(last_dt)), L2 flushed
                   before each timed step, CUDA events on the context stream.
  grid_min_parts   part count above which a large cluster is solved by a
                   cooperative grid over all SMs instead of a thread-block
                   cluster (or one block); timed on outer steps of three
                   piles: the 64-cube scene after its bodies have landed (one
                   65-part cluster), and 144 and 400 cubes resting side by
                   side (one 145- and one 401-part cluster).
"""
import argparse
import json
import os
import time

import numpy as np

import delta2_gb300 as D

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_OUT = os.path.join(HERE, "tuning", "gb300.json")


def _ccd_workload(seed=0):
    s = D.make_scene(2, seed=seed)
    pairs = D.broad_phase(s)
    mt = np.minimum(s.last_dt[pairs[:, 0]], s.last_dt[pairs[:, 1]])
    return s, pairs, mt


def time_ccd(values, steps=10, warmup=3):
    """ms per CCD step for each ee_first_iters value, and the contact digests."""
    import torch

    s, pairs, mt = _ccd_workload()
    ctx = D.Context(0)
    ctx.set_scene(s.copy())
    d_pairs = torch.from_numpy(pairs).cuda()
    d_mt = torch.from_numpy(mt).cuda()
    stream = torch.cuda.ExternalStream(ctx.stream())
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    out = {}
    digests = {}
    for v in values:
        ctx.set_tuning(D.TUNE_EE_FIRST_ITERS, v)
        for _ in range(warmup):
            ctx.compare_trees_full_continuous_device(d_pairs.data_ptr(), d_mt.data_ptr(), len(pairs))
        tot = 0.0
        for _ in range(steps):
            with torch.cuda.stream(stream):
                flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            ctx.compare_trees_full_continuous_device(d_pairs.data_ptr(), d_mt.data_ptr(), len(pairs))
            e1.record(stream)
            e1.synchronize()
            tot += e0.elapsed_time(e1)
        out[v] = tot / steps
        con, off, _ = ctx.compare_trees_full_continuous(pairs, mt)
        digests[v] = (len(con), int(np.ascontiguousarray(con).view(np.uint64).sum()),
                      int(np.ascontiguousarray(off).astype(np.int64).sum()))
    ctx.close()
    return out, digests


def _pile(kind):
    if kind == "cubes64":
        s = D.make_scene(1)
        return s, 100, 20
    side, timed = (12, 10) if kind == "cubes144" else (20, 3)
    s = D.make_scene(1, nx=side, ny=side, nz=1, spacing=1.01, speed_sigma=0.0)
    s.cur[1:, 1:5] = [1.0, 0.0, 0.0, 0.0]
    s.cur[1:, 10] = 0.51
    s.cur[1:, 11:14] = [0.0, 0.0, -0.5]
    s.fut[1:] = s.cur[1:]
    s.last[1:] = s.cur[1:]
    return s, 0, timed


def time_world(values, kinds=("cubes64", "cubes144", "cubes400")):
    """Seconds for the timed outer steps of each pile under each
    grid_min_parts value (fresh context per run; the untimed steps bring the
    pile to the same state), and digests of the final states."""
    out, digests = {}, {}
    for kind in kinds:
        for v in values:
            s, skip, timed = _pile(kind)
            ctx = D.Context(0)
            ctx.set_tuning(D.TUNE_GRID_MIN_PARTS, v)
            gs = s.copy()
            ctx.set_scene(gs)
            ctx.world_configure(gs)
            if skip:
                ctx.world_step(skip)
            t0 = time.perf_counter()
            ctx.world_step(timed)
            out[(kind, v)] = time.perf_counter() - t0
            b = ctx.get_bodies(gs)
            digests[(kind, v)] = int(np.ascontiguousarray(b.cur).view(np.uint64).sum())
            ctx.close()
    return out, digests


def choose_grid_threshold(totals):
    """The smallest part threshold whose total time is within 1% of the
    fastest: the piles measured stop at 401 parts, and larger clusters gain
    from the grid, so a tie goes to the value that lets them take it."""
    best = min(totals.values())
    return min(v for v, t in totals.items() if t <= 1.01 * best)


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--out", default=DEFAULT_OUT)
    p.add_argument("--ee-values", default="0,1,2,3,4")
    p.add_argument("--grid-values", default="64,512,1000000")
    a = p.parse_args()
    from delta2_gb300 import build as B

    B.build()
    ee_values = [int(x) for x in a.ee_values.split(",")]
    grid_values = [int(x) for x in a.grid_values.split(",")]
    ccd_ms, ccd_dig = time_ccd(ee_values)
    world_s, world_dig = time_world(grid_values)
    if len(set(ccd_dig.values())) != 1:
        raise SystemExit(f"ee_first_iters changed the CCD results: {ccd_dig}")
    for kind in {k for k, _ in world_dig}:
        if len({d for (k, _), d in world_dig.items() if k == kind}) != 1:
            raise SystemExit(f"grid_min_parts changed the {kind} states: {world_dig}")
    best_ee = min(ccd_ms, key=ccd_ms.get)
    totals = {v: sum(world_s[(k, v)] for k, vv in world_s if vv == v) for v in grid_values}
    best_grid = choose_grid_threshold(totals)
    import torch

    res = {"gpu": torch.cuda.get_device_name(0),
           "settings": {"ee_first_iters": best_ee, "grid_min_parts": best_grid},
           "measurements": {
               "ccd_ms_per_step_by_ee_first_iters": {str(k): round(v, 4) for k, v in ccd_ms.items()},
               "pile_seconds_by_grid_min_parts": {f"{k}/{v}": round(t, 4) for (k, v), t in world_s.items()},
               "identical_results": True}}
    os.makedirs(os.path.dirname(os.path.abspath(a.out)), exist_ok=True)
    with open(a.out, "w") as f:
        json.dump(res, f, indent=1)
    print(json.dumps(res))


def load(path=DEFAULT_OUT):
    """The settings of a tuning file, or {} when there is none."""
    if not os.path.exists(path):
        return {}
    with open(path) as f:
        return json.load(f).get("settings", {})


if __name__ == "__main__":
    main()
