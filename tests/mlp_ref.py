"""CPU FP64 restatement of the learned proposal network's forward pass, loss
and gradient, with the GPU kernels' BF16 rounding points (inputs, weights,
activations, and dZ2 where it feeds the tensor cores), for the gradient
check.  Parameter layout: W1 [128][20], b1 [128], W2 [128][128], b2 [128],
W3 [2][128], b3 [2]."""
import numpy as np

SIZES = [("W1", (128, 20)), ("b1", (128,)), ("W2", (128, 128)), ("b2", (128,)), ("W3", (2, 128)), ("b3", (2,))]


def unpack(p):
    out, o = {}, 0
    for name, shape in SIZES:
        n = int(np.prod(shape))
        out[name] = np.asarray(p[o:o + n], dtype=np.float32).reshape(shape)
        o += n
    return out


def pack(d):
    return np.concatenate([d[name].reshape(-1) for name, _ in SIZES]).astype(np.float64)


def bf16(x):
    """Round float32 values to BF16 (nearest, ties to even), as float64."""
    b = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def silu(z):
    return z / (1.0 + np.exp(-z))


def silu_grad(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def loss_and_grad(params, feats, targets, mean, std):
    W = unpack(params)
    f = np.asarray(feats, np.float32)
    inv = np.where(np.asarray(std, np.float32) > 0, np.float32(1.0) / np.asarray(std, np.float32), np.float32(1.0))
    X = bf16((f - np.asarray(mean, np.float32)) * inv)
    W1, W2, W3 = bf16(W["W1"]), bf16(W["W2"]), bf16(W["W3"])
    b1, b2, b3 = (W[k].astype(np.float64) for k in ("b1", "b2", "b3"))
    Z1 = X @ W1.T + b1
    H1 = bf16(silu(Z1).astype(np.float32))
    Z2 = H1 @ W2.T + b2
    H2 = bf16(silu(Z2).astype(np.float32))
    out = H2 @ W3.T + b3
    y = np.asarray(targets, np.float64)
    n = len(f)
    e = out[:, 0] - y[:, 0]
    p = 1.0 / (1.0 + np.exp(-out[:, 1]))
    bce = np.log1p(np.exp(-np.abs(out[:, 1]))) + np.maximum(out[:, 1], 0.0) - out[:, 1] * y[:, 1]
    loss = np.mean(e * e + bce)
    dout = np.stack([2.0 * e, p - y[:, 1]], -1) / n
    dZ2 = (dout @ W3) * silu_grad(Z2)
    dH1 = bf16(dZ2.astype(np.float32)) @ W2
    dZ1 = dH1 * silu_grad(Z1)
    g = {"W1": dZ1.T @ X[:, :20], "b1": dZ1.sum(0), "W2": dZ2.T @ H1, "b2": dZ2.sum(0), "W3": dout.T @ H2,
         "b3": dout.sum(0)}
    return loss, pack(g), out
