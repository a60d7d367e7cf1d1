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
