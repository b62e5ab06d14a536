"""FP64 reference of the warm-start network -- TEST INFRASTRUCTURE ONLY.

The per-node MLP 24 -> 64 -> 64 -> 64 -> 3 with GELU (tanh form) on the three
hidden layers, mean-squared-error loss, and the Adam update, written with
plain numpy in float64.  The GPU kernels (phybs_gb300/csrc/warmstart.cu) are
checked against it: forward outputs, parameter gradients and one Adam step.

Parameter vector layout (10,115 floats): W1 (64x24, row = output), b1 (64),
W2 (64x64), b2 (64), W3 (64x64), b3 (64), W4 (3x64), b4 (3).
"""
from __future__ import annotations

import numpy as np

SIZES = [(64, 24), (64, 64), (64, 64), (3, 64)]
N_PARAMS = sum(o * i + o for o, i in SIZES)
GELU_C = np.sqrt(2.0 / np.pi)


def unpack(theta):
    theta = np.asarray(theta, np.float64)
    out, off = [], 0
    for o, i in SIZES:
        W = theta[off:off + o * i].reshape(o, i)
        off += o * i
        b = theta[off:off + o]
        off += o
        out.append((W, b))
    assert off == theta.size == N_PARAMS
    return out


def pack(layers):
    return np.concatenate([np.concatenate([W.ravel(), b]) for W, b in layers])


def gelu(z):
    return 0.5 * z * (1.0 + np.tanh(GELU_C * (z + 0.044715 * z ** 3)))


def gelu_grad(z):
    u = GELU_C * (z + 0.044715 * z ** 3)
    t = np.tanh(u)
    return 0.5 * (1.0 + t) + 0.5 * z * (1.0 - t * t) * GELU_C * (1.0 + 3 * 0.044715 * z * z)


def bf16(a):
    """Round to bfloat16 (nearest even), returned as float64."""
    a = np.asarray(a, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def forward(theta, X, round_bf16=False):
    """Returns the output and the per-layer (input, pre-activation) cache.
    With round_bf16 the weights and every layer input are rounded to BF16 the
    way the tensor-core kernels feed them, accumulation staying exact."""
    layers = unpack(theta)
    h = np.asarray(X, np.float64)
    cache = []
    for li, (W, b) in enumerate(layers):
        hin = bf16(h) if round_bf16 else h
        Wq = bf16(W) if round_bf16 else W
        z = hin @ Wq.T + b
        cache.append((hin, z))
        h = gelu(z) if li < 3 else z
    return h, cache


def loss_and_grad(theta, X, Y, round_bf16=False, W=None):
    """Mean over rows of the squared error summed over the 3 outputs (each row
    weighted by W when given), and its gradient with respect to theta."""
    layers = unpack(theta)
    out, cache = forward(theta, X, round_bf16)
    n = X.shape[0]
    diff = out - np.asarray(Y, np.float64)
    w = np.ones((n, 1)) if W is None else np.asarray(W, np.float64).reshape(n, 1)
    loss = float((w * diff ** 2).sum() / n)
    delta = 2.0 * w * diff / n
    grads = [None] * 4
    for li in range(3, -1, -1):
        hin, z = cache[li]
        W, _ = layers[li]
        Wq = bf16(W) if round_bf16 else W
        if li < 3:
            delta = delta * gelu_grad(z)
        grads[li] = (delta.T @ hin, delta.sum(0))
        delta = delta @ Wq
    return loss, pack(grads)


def adam(theta, m, v, g, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** step)
    vh = v / (1 - b2 ** step)
    return theta - lr * mh / (np.sqrt(vh) + eps), m, v


def init_params(seed=0):
    rng = np.random.default_rng(seed)
    layers = []
    for o, i in SIZES:
        W = rng.normal(0.0, np.sqrt(2.0 / i), (o, i))
        layers.append((W, np.zeros(o)))
    return pack(layers)
