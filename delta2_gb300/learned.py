"""Data for the learned time-of-impact proposal: pair-query features and
CCD-derived targets.

A CCD pair query is one compareTreesFullContinuous call
(collision_detection/full_tree_comparison.h:69-219) over [0, max_time].  Its
20 features, from the bodies' current states (model/state.h):
  * B's pose in A's frame: R_a^T R_b (9, row major) and R_a^T (x_b - x_a) (3);
  * the relative motion over the query's horizon, in A's frame:
    R_a^T (v_b - v_a) * max_time (3) and R_a^T (w_b - w_a) * max_time (3),
    with w = R I^-1 R^T L the world angular velocity;
  * the two bodies' bounding radii (2).
Targets: the normalised time of impact (the smallest toc of the query's
contacts, 1 when it has none) and the hit flag (any contact)."""
import numpy as np

import delta2_gb300 as D


def qmat(q):
    """Rotation matrices [n,3,3] of unit quaternions [n,4] (w, x, y, z)."""
    w, x, y, z = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    return np.stack([
        np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)], -1),
        np.stack([2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)], -1),
        np.stack([2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)], -1)], -2)


def pair_features(scene, pairs, max_time):
    """[n_pairs, 20] float32 features of the queries (a, b, max_time)."""
    pairs = np.asarray(pairs, dtype=np.int64).reshape(-1, 2)
    a, b = pairs[:, 0], pairs[:, 1]
    st = scene.cur
    R = qmat(st[:, 1:5])
    ii = np.asarray(scene.inv_inertia).reshape(-1, 3, 3)
    omega = np.einsum("nij,njk,nlk,nl->ni", R, ii, R, st[:, 5:8])
    Ra_t = np.transpose(R[a], (0, 2, 1))
    rel_R = Ra_t @ R[b]
    rel_t = np.einsum("nij,nj->ni", Ra_t, st[b, 8:11] - st[a, 8:11])
    mt = np.asarray(max_time, dtype=np.float64).reshape(-1)[:, None]
    rel_v = np.einsum("nij,nj->ni", Ra_t, st[b, 11:14] - st[a, 11:14]) * mt
    rel_w = np.einsum("nij,nj->ni", Ra_t, omega[b] - omega[a]) * mt
    rad = np.stack([scene.bounding_radius[a], scene.bounding_radius[b]], -1)
    return np.concatenate([rel_R.reshape(-1, 9), rel_t, rel_v, rel_w, rad], -1).astype(np.float32)


def ccd_targets(contacts, offsets):
    """[n_pairs, 2] float32: smallest toc (1 when no contact), hit flag."""
    n = len(offsets) - 1
    toi = np.ones(n, np.float64)
    cnt = np.diff(offsets)
    hit = cnt > 0
    if len(contacts):
        pair_of = np.repeat(np.arange(n), cnt)
        np.minimum.at(toi, pair_of, contacts[:, 10])
    return np.stack([toi, hit.astype(np.float64)], -1).astype(np.float32)


def cube_queries(ctx, seed, nx=8, ny=8, nz=8, speed=3.0, horizon=1.0 / 30.0):
    """CCD queries of one cube scene (the 1 m cubes of the small
    configuration, on a grid of the given size) with every broad-phase pair
    over `horizon`: (features, targets, pairs, max_time)."""
    s = D.make_scene(1, nx=nx, ny=ny, nz=nz, spacing=1.6, speed_sigma=speed, seed=seed, dt=horizon)
    s.last_dt[:] = np.float64(np.float32(horizon))
    s.fut[:, 8:11] = s.cur[:, 8:11] + s.last_dt[:, None] * s.cur[:, 11:14]
    pairs = D.broad_phase(s)
    mt = np.minimum(s.last_dt[pairs[:, 0]], s.last_dt[pairs[:, 1]])
    ctx.set_scene(s)
    con, off, _ = ctx.compare_trees_full_continuous(pairs, mt)
    return pair_features(s, pairs, mt), ccd_targets(con, off), pairs, mt


def dataset(ctx, n_queries, seed=0, **kw):
    """At least n_queries CCD queries from cube scenes of successive seeds."""
    feats, targs = [], []
    total, k = 0, 0
    while total < n_queries:
        f, t, _, _ = cube_queries(ctx, seed * 1000003 + k, **kw)
        feats.append(f)
        targs.append(t)
        total += len(f)
        k += 1
    return np.concatenate(feats)[:n_queries], np.concatenate(targs)[:n_queries]


def report(ctx, n_train=1_800_000, n_test=200_000, epochs=8, batch=4096, lr=2e-3, seed=0):
    """Train on n_train queries (cube scenes of one seed range), evaluate on
    n_test queries of other seeds; returns a dict of the figures."""
    import time

    t0 = time.perf_counter()
    f_tr, y_tr = dataset(ctx, n_train, seed=2 * seed + 1)
    f_te, y_te = dataset(ctx, n_test, seed=2 * seed + 2)
    gen_s = time.perf_counter() - t0
    net = D.Mlp(ctx, seed=seed)
    net.set_normalization(f_tr.mean(0), f_tr.std(0))
    t0 = time.perf_counter()
    losses = net.train(f_tr, y_tr, epochs=epochs, batch=batch, lr=lr, seed=seed)
    train_s = time.perf_counter() - t0
    net.predict(f_te[:4096])
    t0 = time.perf_counter()
    out = net.predict(f_te)
    pred_s = time.perf_counter() - t0
    hit = y_te[:, 1] > 0.5
    ph = out[:, 1] > 0
    toi_err = np.abs(np.clip(out[hit, 0], 0, 1) - y_te[hit, 0])
    return {
        "train_queries": int(len(f_tr)), "test_queries": int(len(f_te)), "hit_rate": float(hit.mean()),
        "epochs": epochs, "loss_per_epoch": [float(x) for x in losses],
        "hit_accuracy": float(np.mean(ph == hit)), "hit_recall": float(np.mean(ph[hit])) if hit.any() else None,
        "miss_rate": float(np.mean(~ph[hit])) if hit.any() else None,
        "false_alarm_rate": float(np.mean(ph[~hit])) if (~hit).any() else None,
        "toi_mae_on_hits": float(toi_err.mean()) if hit.any() else None,
        "toi_p90_err_on_hits": float(np.quantile(toi_err, 0.9)) if hit.any() else None,
        "train_samples_per_s": len(f_tr) * epochs / train_s, "predict_samples_per_s_e2e": len(f_te) / pred_s,
        "data_generation_s": gen_s,
    }


if __name__ == "__main__":
    import json
    import sys

    ctx = D.Context(0)
    kw = {}
    if len(sys.argv) > 1:
        kw["n_train"] = int(sys.argv[1])
        kw["n_test"] = max(1000, int(sys.argv[1]) // 9)
    print(json.dumps(report(ctx, **kw)))
