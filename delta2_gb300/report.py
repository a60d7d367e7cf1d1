"""Full-run statistics of the GPU stepper: energy and contact penetration
per outer step, optionally compared step by step with the oracle stepper.

  python -m delta2_gb300.report --config 1 --steps 240 --oracle
  python -m delta2_gb300.report --batch 256 --steps 300   # the batched configuration

Energy of the moving bodies: translational 1/2 m |v|^2, rotational
1/2 L . w with w = R I^-1 R^T L, and potential m |g| z.  Penetration: the
discrete narrow phase (compareTreesFull) over the broad-phase pairs of the
current future states; the smallest contact distance |A - B| and the number
of contacts closer than 1e-6 m (touching or interpenetrating surfaces)."""
import argparse
import json
import time

import numpy as np

import delta2_gb300 as D
from delta2_gb300.learned import qmat


def energy(scene, gravity):
    moving = scene.is_static == 0
    st = scene.cur[moving]
    m = scene.mass[moving]
    R = qmat(st[:, 1:5])
    ii = np.asarray(scene.inv_inertia[moving]).reshape(-1, 3, 3)
    L = st[:, 5:8]
    w = np.einsum("nij,njk,nlk,nl->ni", R, ii, R, L)
    kin = 0.5 * np.sum(m * np.sum(st[:, 11:14] ** 2, axis=1)) + 0.5 * np.sum(np.sum(L * w, axis=1))
    pot = np.sum(m * abs(gravity) * st[:, 10])
    return float(kin), float(pot)


def run(config, steps, seed=0, oracle=False, every=1, batch=0):
    """batch > 0: the batched configuration of that many scenes (config 3's
    mixed shapes) in one context; the broad phase of the penetration check
    then pairs bodies of the same scene only."""
    scene_of = None
    if batch > 0:
        s, scene_of, _ = D.make_batch(batch, seed=seed)
        config = 3
    else:
        s = D.make_scene(config, seed=seed)
    ctx = D.Context(0)
    ctx.set_scene(s.copy())
    if scene_of is not None:
        ctx.set_scenes(scene_of)
    ctx.world_configure(s)
    ref = None
    if oracle:
        from oracle import oracle as O
        ref = O.World(s.copy(), s.opt_dt, s.gravity_z)
    rows, identical, t_gpu = [], True, 0.0
    cur = s.copy()
    for i in range(steps):
        t0 = time.perf_counter()
        ctx.world_step(1)
        t_gpu += time.perf_counter() - t0
        ctx.get_bodies(cur)
        if ref is not None:
            assert ref.step(1) == 0
            rb = ref.get_bodies()
            for f in ["last", "cur", "fut", "last_dt", "sleep_steps", "sleeping"]:
                a, b = np.ascontiguousarray(getattr(cur, f)), np.ascontiguousarray(getattr(rb, f))
                if a.dtype == np.float64:
                    a, b = a.view(np.uint64), b.view(np.uint64)
                identical = identical and np.array_equal(a, b)
        if i % every and i != steps - 1:
            continue
        kin, pot = energy(cur, s.gravity_z)
        pairs = ctx.broad_phase_device(cur) if scene_of is not None else D.broad_phase(cur)
        con, off, _ = ctx.compare_trees_full(pairs)
        d = np.linalg.norm(con[:, 0:3] - con[:, 3:6], axis=1) if len(con) else np.zeros(0)
        moving = cur.is_static == 0
        rows.append({"step": i + 1, "time": float(cur.cur[moving, 0].min()), "kinetic": kin, "potential": pot,
                     "contacts": int(len(con)), "min_contact_distance": float(d.min()) if len(d) else None,
                     "penetrating": int(np.sum(d < 1e-6)), "finite": bool(np.isfinite(cur.cur).all())})
    ctx.close()
    e = np.array([r["kinetic"] + r["potential"] for r in rows])
    out = {"config": config, "batch_scenes": batch, "steps": steps, "bodies": int(s.n_bodies), "gpu_stepper_s": t_gpu,
           "sim_seconds": rows[-1]["time"], "energy_start": float(e[0]), "energy_end": float(e[-1]),
           "energy_max_rise": float(np.max(e - e[0])), "max_penetrating": max(r["penetrating"] for r in rows),
           "min_contact_distance": min((r["min_contact_distance"] for r in rows
                                        if r["min_contact_distance"] is not None), default=None),
           "all_finite": all(r["finite"] for r in rows)}
    if ref is not None:
        out["identical_to_oracle_every_step"] = bool(identical)
        out["oracle_stats"] = ref.stats()
    return out, rows


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--config", type=int, default=1)
    p.add_argument("--steps", type=int, default=240)
    p.add_argument("--seed", type=int, default=0)
    p.add_argument("--oracle", action="store_true")
    p.add_argument("--every", type=int, default=10)
    p.add_argument("--batch", type=int, default=0, help="scenes of the batched configuration (0: one scene)")
    a = p.parse_args()
    out, rows = run(a.config, a.steps, a.seed, a.oracle, a.every, a.batch)
    out["samples"] = rows
    print(json.dumps(out))


if __name__ == "__main__":
    main()
