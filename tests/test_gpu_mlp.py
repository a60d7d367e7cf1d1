"""The learned TOI proposal network: tensor-core forward pass and gradient
against a CPU FP64 restatement with the same BF16 rounding points, and a
short training run on CCD queries generated by the exact GPU path."""
import numpy as np
import pytest

import delta2_gb300 as D
from tests import mlp_ref as R

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(gpu_required):
    from delta2_gb300 import build as B
    B.build()
    c = D.Context(0)
    yield c
    c.close()


def random_problem(n, seed):
    rng = np.random.default_rng(seed)
    feats = rng.normal(0.0, 1.5, size=(n, 20)).astype(np.float32)
    targets = np.stack([rng.uniform(0, 1, n), rng.integers(0, 2, n)], -1).astype(np.float32)
    params = (rng.normal(0.0, 0.12, size=D.MLP_PARAMS)).astype(np.float32)
    mean = rng.normal(0.0, 0.3, 20).astype(np.float32)
    std = rng.uniform(0.5, 2.0, 20).astype(np.float32)
    return feats, targets, params, mean, std


def test_forward_matches_restatement(ctx):
    feats, targets, params, mean, std = random_problem(1000, 1)  # not a multiple of the 64-row tile
    net = D.Mlp(ctx, seed=3)
    net.set_params(params)
    net.set_normalization(mean, std)
    out = net.predict(feats)
    _, _, ref = R.loss_and_grad(params, feats, targets, mean, std)
    # tolerance: BF16 rounding of activations can land on the other side of a tie
    assert np.allclose(out, ref, rtol=1e-2, atol=2e-2), np.abs(out - ref).max()
    assert np.mean(np.abs(out - ref)) < 2e-3


def test_gradient_matches_restatement(ctx):
    feats, targets, params, mean, std = random_problem(777, 2)
    net = D.Mlp(ctx, seed=3)
    net.set_params(params)
    net.set_normalization(mean, std)
    g, loss = net.gradient(feats, targets)
    ref_loss, ref_g, _ = R.loss_and_grad(params, feats, targets, mean, std)
    assert abs(loss - ref_loss) <= 1e-3 * abs(ref_loss)
    o = 0
    for name, shape in R.SIZES:
        k = int(np.prod(shape))
        a, b = g[o:o + k].astype(np.float64), ref_g[o:o + k]
        rel = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-12)
        assert rel < 2e-2, (name, rel)
        o += k


def test_training_learns_the_exact_ccd(ctx):
    from delta2_gb300 import learned as L

    f_tr, y_tr = L.dataset(ctx, 60000, seed=1, nx=6, ny=6, nz=6)
    f_te, y_te = L.dataset(ctx, 8000, seed=2, nx=6, ny=6, nz=6)
    assert 0.05 < y_tr[:, 1].mean() < 0.95  # both classes present
    net = D.Mlp(ctx, seed=7)
    net.set_normalization(f_tr.mean(0), f_tr.std(0))
    before = net.predict(f_te)
    losses = net.train(f_tr, y_tr, epochs=6, batch=2048, lr=2e-3, seed=5)
    assert losses[-1] < losses[0]
    after = net.predict(f_te)
    hit = y_te[:, 1] > 0.5
    acc = np.mean((after[:, 1] > 0) == hit)
    majority = max(hit.mean(), 1 - hit.mean())
    assert acc > majority
    # the proposal's TOI error on hits shrinks with training
    err_before = np.mean(np.abs(np.clip(before[hit, 0], 0, 1) - y_te[hit, 0]))
    err_after = np.mean(np.abs(np.clip(after[hit, 0], 0, 1) - y_te[hit, 0]))
    assert err_after < err_before


def _cube_query_scene(seed, n=6, horizon=1.0 / 30.0):
    """A cube scene of the network's training distribution (delta2_gb300.learned
    cube_queries) and its CCD queries over the horizon."""
    s = D.make_scene(1, nx=n, ny=n, nz=n, spacing=1.6, speed_sigma=3.0, seed=seed, dt=horizon)
    s.last_dt[:] = np.float64(np.float32(horizon))
    s.fut[:, 8:11] = s.cur[:, 8:11] + s.last_dt[:, None] * s.cur[:, 11:14]
    pairs = D.broad_phase(s)
    return s, pairs, np.minimum(s.last_dt[pairs[:, 0]], s.last_dt[pairs[:, 1]])


def test_device_features_match_the_training_features(ctx):
    """The CCD computes the proposal's features on the device; they must be
    the features the network was trained on (delta2_gb300.learned)."""
    from delta2_gb300 import learned as L

    s, pairs, mt = _cube_query_scene(77)
    ctx.set_scene(s.copy())
    got = ctx.ccd_features(pairs, mt)
    ref = L.pair_features(s, pairs, mt)
    assert np.allclose(got, ref, rtol=1e-5, atol=1e-6), np.abs(got - ref).max()


def test_learned_proposal_in_the_ccd(ctx):
    """The learned proposal inside compareTreesFullContinuous: queries the
    network predicts contact-free go to the root certificate, and the proven
    ones are skipped.  Contacts, per-pair offsets and projected futures stay
    identical to the oracle's, with the network, without it (threshold 1:
    every query goes to the certificate) and with the proposal off, on a
    cube scene of other seeds than the training data and on a hull scene.
    The network's gain over the certificate alone: it sends far fewer queries
    to the certificate and keeps most of the skips."""
    from delta2_gb300 import learned as L
    from oracle import oracle as O

    f_tr, y_tr = L.dataset(ctx, 60000, seed=1, nx=6, ny=6, nz=6)
    net = D.Mlp(ctx, seed=7)
    net.set_normalization(f_tr.mean(0), f_tr.std(0))
    net.train(f_tr, y_tr, epochs=6, batch=2048, lr=2e-3, seed=5)
    hull = D.make_scene(2, nx=4, ny=4, nz=4, spacing=1.3, speed_sigma=2.0, seed=9)
    hp = D.broad_phase(hull)
    cases = {"cubes": _cube_query_scene(4242), "hulls": (hull, hp, np.full(len(hp), np.float64(np.float32(
        hull.opt_dt)) * 4))}
    stats = {}
    try:
        for case, (s, pairs, mt) in cases.items():
            ref_s = s.copy()
            ref, ref_off, _, _ = O.ccd(ref_s, pairs, mt)
            touched = np.unique(pairs.ravel())
            for mode, (mlp, th) in {"off": (None, 0.5), "network": (net, 0.5), "certificate_only": (net, 1.0)}.items():
                gs = s.copy()
                ctx.set_scene(gs)
                ctx.set_ccd_proposal(mlp, th)
                ctx.ccd_stats(reset=True)
                c, off, _ = ctx.compare_trees_full_continuous(pairs, mt, capacity=1 << 20)  # one call
                stats[(case, mode)] = ctx.ccd_stats(reset=True)
                assert np.array_equal(off, ref_off), (case, mode)
                assert np.array_equal(c.view(np.uint64), ref.view(np.uint64)), (case, mode)
                ctx.get_bodies(gs)
                assert np.array_equal(gs.fut[touched].view(np.uint64), ref_s.fut[touched].view(np.uint64))
            assert stats[(case, "off")]["pairs_seen"] == 0
            allq = stats[(case, "certificate_only")]
            assert allq["pairs_predicted_clear"] == allq["pairs_seen"] == len(pairs)
            assert allq["pairs_certified"] + allq["pairs_missed"] == len(pairs)
    finally:
        ctx.set_ccd_proposal(None)
    cn, ca = stats[("cubes", "network")], stats[("cubes", "certificate_only")]
    assert ca["pairs_certified"] > 0
    assert cn["pairs_predicted_clear"] < ca["pairs_predicted_clear"]
    assert cn["pairs_certified"] >= 0.5 * ca["pairs_certified"]
    print({f"{k[0]}/{k[1]}": v for k, v in stats.items()})


def test_network_outlives_its_context(gpu_required):
    """Destroying a context before its network: the network's calls report
    the lost context (D2G_ERR_STATE) and destroying it afterwards is safe."""
    c = D.Context(0)
    net = D.Mlp(c, seed=1)
    feats = np.zeros((8, 20), np.float32)
    assert net.predict(feats).shape == (8, 2)
    c.close()
    with pytest.raises(D.D2GError) as e:
        net.predict(feats)
    assert e.value.code == -4
    net.close()
