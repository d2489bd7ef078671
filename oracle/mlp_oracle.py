"""CPU oracle of the learned capillary closure (test infrastructure only).

A plain numpy restatement of what the library's network kernels compute
(gpucode_gb300/csrc/capnet.cu, capnet.cuh): the standardisation of the raw
features and targets, the 4 -> 64 -> 64 -> 2 SiLU forward pass, the loss (mean
over samples of the squared error of the standardised outputs) and its
analytic gradient, and the BF16 tensor-core forward (weights and activations
rounded to BF16 where the tiles round them, FP32 accumulation).  The plain
capillary formula the network stands in for is restated from the reference's
fCap (kernel.cu:65-81) and rupture distance (kernel.cu:518).

The gradient is pinned against central finite differences of the loss in
FP64 (tests/test_capnet_oracle.py).
"""
from __future__ import annotations

import numpy as np

N_PARAMS = 4610
PI_REF = 3.1415926  # heydem.h:15


def unpack(p: np.ndarray):
    p = np.asarray(p, np.float64)
    return (p[0:256].reshape(64, 4), p[256:320], p[320:4416].reshape(64, 64), p[4416:4480],
            p[4480:4608].reshape(2, 64), p[4608:4610])


def pack(W1, b1, W2, b2, W3, b3) -> np.ndarray:
    return np.concatenate([W1.ravel(), b1, W2.ravel(), b2, W3.ravel(), b3])


def std_inputs(xraw: np.ndarray, norm: np.ndarray) -> np.ndarray:
    x = np.asarray(xraw, np.float64)
    f = np.column_stack([np.log(x[:, 0]), np.log(x[:, 1]), x[:, 2], x[:, 3]])
    return (f - norm[0:4]) / norm[4:8]


def std_targets(yraw: np.ndarray, norm: np.ndarray) -> np.ndarray:
    return (np.asarray(yraw, np.float64) - norm[8:10]) / norm[10:12]


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(p, xs):
    """standardised inputs -> standardised outputs (FP64)"""
    W1, b1, W2, b2, W3, b3 = unpack(p)
    z1 = xs @ W1.T + b1
    h1 = silu(z1)
    z2 = h1 @ W2.T + b2
    h2 = silu(z2)
    return h2 @ W3.T + b3, (z1, h1, z2, h2)


def loss_and_grad(p, xraw, yraw, norm):
    xs, ts = std_inputs(xraw, norm), std_targets(yraw, norm)
    W1, b1, W2, b2, W3, b3 = unpack(p)
    y, (z1, h1, z2, h2) = forward(p, xs)
    n = len(xs)
    e = y - ts
    loss = float((e ** 2).sum() / n)
    dy = 2.0 * e / n
    gW3, gb3 = dy.T @ h2, dy.sum(0)
    dz2 = (dy @ W3) * dsilu(z2)
    gW2, gb2 = dz2.T @ h1, dz2.sum(0)
    dz1 = (dz2 @ W2) * dsilu(z1)
    gW1, gb1 = dz1.T @ xs, dz1.sum(0)
    return loss, pack(gW1, gb1, gW2, gb2, gW3, gb3)


def loss_only(p, xraw, yraw, norm) -> float:
    y, _ = forward(p, std_inputs(xraw, norm))
    e = y - std_targets(yraw, norm)
    return float((e ** 2).sum() / len(e))


def bf16(a: np.ndarray) -> np.ndarray:
    """round FP32 values to the nearest BF16 (ties to even), returned as FP32"""
    u = np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.uint64)
    r = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return r.astype(np.uint32).view(np.float32)


def forward_bf16(p, xraw, norm) -> np.ndarray:
    """raw features -> raw outputs as the tensor-core tiles compute them"""
    W1, b1, W2, b2, W3, b3 = (np.asarray(w, np.float32) for w in unpack(p))
    xs = bf16(std_inputs(xraw, norm).astype(np.float32)).astype(np.float64)
    W1b, W2b, W3b = (bf16(w).astype(np.float64) for w in (W1, W2, W3))
    h1 = bf16(silu(xs @ W1b.T + b1).astype(np.float32)).astype(np.float64)
    h2 = bf16(silu(h1 @ W2b.T + b2).astype(np.float32)).astype(np.float64)
    y = h2 @ W3b.T + b3
    return y * norm[10:12] + norm[8:10]


def formula(xraw: np.ndarray) -> np.ndarray:
    """the plain closure on raw features: kernel.cu:65-81 divided by
    2 pi R_eff gamma, and 0.99 (V / 8)^0.33 (kernel.cu:518), FP64"""
    x = np.asarray(xraw, np.float64)
    sp, v = x[:, 0] / np.sqrt(x[:, 1]), x[:, 1]
    lv = np.log(v)
    f1 = -0.44507 - 0.1119 * lv - 0.012101 * lv ** 2 - 0.0005 * lv ** 3
    f2 = 1.9222 - 0.0668 * lv - 0.0013375 * lv ** 2
    f3 = 1.268 + 0.198 * lv + 0.02232 * lv ** 2 + 0.0008585 * lv ** 3
    f4 = -0.010703 + 0.03345 * lv + 0.0018574 * lv ** 2
    ls = np.log(sp)
    force = np.exp(f1 - f2 * np.exp(f3 * ls + f4 * ls ** 2))
    return np.column_stack([force, 0.99 * (v / 8.0) ** 0.33])


def init_params(seed: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    parts = []
    for count, fan in ((256, 4), (64, 4), (4096, 64), (64, 64), (128, 64), (2, 64)):
        b = 1.0 / np.sqrt(fan)
        parts.append(rng.uniform(-b, b, count))
    return np.concatenate(parts)
