"""CPU restatement of the learned absorbing layer's network and its training
gradient -- test infrastructure only (the checker of the CUDA kernels in
distributed-cube-average_gb300/csrc/dc_learned.cu); the product never calls
it.

The reference has no learned boundary (it absorbs with the random velocity
boundary of src/boundary.c:7-104), so there is no reference output to pin
this to: it is pinned instead by finite differences (tests/test_learned_cpu.py)
and the CUDA kernels are checked against it.

Network: 32 features x -> r = rms(x); x^ = bf16(x / r);
h1 = bf16(gelu(W1 x^ + b1[depth])); h2 = bf16(gelu(W2 h1 + b2)), GELU in its
tanh form a/2 (1 + tanh(sqrt(2/pi) (a + 0.044715 a^3))) (the GPU evaluates
tanh with its hardware approximation, relative error ~2^-11);
y = W3 h2 + b3; correction = r * y.  Weights W1, W2, W3 are rounded to BF16,
biases stay FP32.  Loss over samples: sum_i |r_i y_i - t_i|^2, with sum r_i^2
reported beside it; gradients pass the BF16 roundings unchanged.
"""
from __future__ import annotations

import math

import numpy as np

IN, HID, OUT, DEPTHS = 32, 32, 2, 16
OFF_W1 = 0
OFF_B1 = OFF_W1 + HID * IN
OFF_W2 = OFF_B1 + DEPTHS * HID
OFF_B2 = OFF_W2 + HID * HID
OFF_W3 = OFF_B2 + HID
OFF_B3 = OFF_W3 + OUT * HID
NPARAMS = OFF_B3 + OUT
STRIDE = IN + 1


def bf16(a, enabled: bool = True) -> np.ndarray:
    """Round to bfloat16 (nearest, ties to even) and back to float64."""
    if not enabled:
        return np.asarray(a, np.float64)
    f = np.asarray(a, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


C0, C1 = math.sqrt(2.0 / math.pi), 0.044715


def gelu(a):
    return 0.5 * a * (1.0 + np.tanh(C0 * (a + C1 * a ** 3)))


def gelu_grad(a):
    th = np.tanh(C0 * (a + C1 * a ** 3))
    return 0.5 * (1.0 + th) + 0.5 * a * (1.0 - th * th) * C0 * (1.0 + 3.0 * C1 * a * a)


def unpack(p, rounding: bool = True):
    p = np.asarray(p, np.float64)
    W1 = bf16(p[OFF_W1:OFF_B1], rounding).reshape(HID, IN)
    b1 = p[OFF_B1:OFF_W2].reshape(DEPTHS, HID)
    W2 = bf16(p[OFF_W2:OFF_B2], rounding).reshape(HID, HID)
    b2 = p[OFF_B2:OFF_W3]
    W3 = bf16(p[OFF_W3:OFF_B3], rounding).reshape(OUT, HID)
    b3 = p[OFF_B3:NPARAMS]
    return W1, b1, W2, b2, W3, b3


def _forward(p, samples, rounding=True):
    s = np.asarray(samples, np.float64).reshape(-1, STRIDE)
    x = s[:, :IN]
    depth = np.clip(s[:, IN].astype(np.int64), 0, DEPTHS - 1)
    r = np.sqrt(np.mean(x * x, axis=1))
    live = r > 0
    rs = np.where(live, r, 1.0)
    W1, b1, W2, b2, W3, b3 = unpack(p, rounding)
    xh = bf16(x / rs[:, None], rounding)
    a1 = xh @ W1.T + b1[depth]
    h1 = bf16(gelu(a1), rounding)
    a2 = h1 @ W2.T + b2
    h2 = bf16(gelu(a2), rounding)
    y = h2 @ W3.T + b3
    return dict(x=x, depth=depth, r=r, live=live, xh=xh, a1=a1, h1=h1, a2=a2, h2=h2, y=y,
                W=(W1, W2, W3))


def forward(p, samples, rounding=True) -> np.ndarray:
    """Corrections r * y, [n][2]."""
    f = _forward(p, samples, rounding)
    return np.where(f["live"][:, None], f["r"][:, None] * f["y"], 0.0)


def loss(p, samples, targets, rounding=True):
    f = _forward(p, samples, rounding)
    t = np.asarray(targets, np.float64).reshape(-1, OUT)
    e = f["r"][:, None] * f["y"] - t
    e = np.where(f["live"][:, None], e, 0.0)
    return float(np.sum(e * e)), float(np.sum(np.where(f["live"], f["r"] ** 2, 0.0)))


def gradient(p, samples, targets, rounding=True):
    """(grad of sum |r y - t|^2 w.r.t. the FP32 master parameters, loss
    sum, sum r^2)."""
    f = _forward(p, samples, rounding)
    t = np.asarray(targets, np.float64).reshape(-1, OUT)
    live = f["live"]
    r = f["r"]
    e = np.where(live[:, None], r[:, None] * f["y"] - t, 0.0)
    dy = 2.0 * r[:, None] * e
    W1, W2, W3 = f["W"]
    g = np.zeros(NPARAMS, np.float64)
    g[OFF_W3:OFF_B3] = (dy.T @ f["h2"]).reshape(-1)
    g[OFF_B3:NPARAMS] = dy.sum(axis=0)
    d2 = (dy @ W3) * gelu_grad(f["a2"])
    d2 = np.where(live[:, None], d2, 0.0)
    g[OFF_W2:OFF_B2] = (d2.T @ f["h1"]).reshape(-1)
    g[OFF_B2:OFF_W3] = d2.sum(axis=0)
    d1 = (d2 @ W2) * gelu_grad(f["a1"])
    d1 = np.where(live[:, None], d1, 0.0)
    g[OFF_W1:OFF_B1] = (d1.T @ f["xh"]).reshape(-1)
    gb1 = np.zeros((DEPTHS, HID))
    np.add.at(gb1, f["depth"], d1)
    g[OFF_B1:OFF_W2] = gb1.reshape(-1)
    return g, float(np.sum(e * e)), float(np.sum(np.where(live, r * r, 0.0)))


def init_params(seed: int) -> np.ndarray:
    """A seeded parameter vector for tests (not the library's own init)."""
    rng = np.random.default_rng(seed)
    p = np.zeros(NPARAMS, np.float64)
    p[OFF_W1:OFF_B1] = rng.normal(0, 1 / math.sqrt(IN), HID * IN)
    p[OFF_B1:OFF_W2] = rng.normal(0, 0.1, DEPTHS * HID)
    p[OFF_W2:OFF_B2] = rng.normal(0, 1 / math.sqrt(HID), HID * HID)
    p[OFF_B2:OFF_W3] = rng.normal(0, 0.1, HID)
    p[OFF_W3:OFF_B3] = rng.normal(0, 1 / math.sqrt(HID), OUT * HID)
    p[OFF_B3:NPARAMS] = rng.normal(0, 0.1, OUT)
    return p.astype(np.float32)


def random_samples(n: int, seed: int, depths: int = 8):
    rng = np.random.default_rng(seed)
    s = np.zeros((n, STRIDE), np.float32)
    scale = np.exp(rng.normal(0, 2, n)).astype(np.float32)[:, None]
    s[:, :IN] = rng.normal(0, 1, (n, IN)).astype(np.float32) * scale
    s[:, IN] = rng.integers(0, depths, n)
    s[:5, :IN] = 0.0  # silent samples contribute nothing
    return s
