"""CPU oracle of the surrogate MLP (test infrastructure only).

The network of include/emt6ro_surrogate.h: 100 -> 512 -> 512 -> 512 -> 1,
exact-erf GELU on the hidden layers, mean-squared-error loss, Adam.

Two restatements:

* `exact_*`   float64 throughout; its gradients are pinned against central
              finite differences (tests/test_surrogate.py), so it is the
              mathematical reference.
* `mixed_*`   the same arithmetic with the tensor-core kernels' rounding
              points: BF16 inputs, weights, pre-activations, activations and
              hidden-layer gradients (round to nearest even), products summed
              in float64 (the GPU sums them in FP32; the difference is the
              tolerance the GPU tests allow), FP32 output layer and Adam.

The surrogate has no counterpart in the reference; its correctness is the
agreement of the GPU kernels with these restatements.
"""
from __future__ import annotations

import numpy as np
from scipy.special import erf

IN, IN_PAD, H = 100, 128, 512
SQRT1_2 = 0.70710678118654752
INV_SQRT_2PI = 0.39894228040143268


def bf16(x) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest even), returned as float32."""
    a = np.ascontiguousarray(x, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).reshape(a.shape)


def gelu(z):
    return 0.5 * z * (1.0 + erf(z * SQRT1_2))


def gelu_grad(z):
    return 0.5 * (1.0 + erf(z * SQRT1_2)) + z * INV_SQRT_2PI * np.exp(-0.5 * z * z)


def init_params(seed: int = 0) -> list[np.ndarray]:
    """He-normal weights (W1's padding columns zero), zero biases."""
    rng = np.random.default_rng(seed)
    w1 = np.zeros((H, IN_PAD), np.float32)
    w1[:, :IN] = rng.normal(0, np.sqrt(2.0 / IN), (H, IN))
    w2 = rng.normal(0, np.sqrt(2.0 / H), (H, H)).astype(np.float32)
    w3 = rng.normal(0, np.sqrt(2.0 / H), (H, H)).astype(np.float32)
    w4 = rng.normal(0, np.sqrt(2.0 / H), H).astype(np.float32)
    z = np.zeros(H, np.float32)
    return [w1, z.copy(), w2, z.copy(), w3, z.copy(), w4, np.zeros(1, np.float32)]


def _pad(x):
    xp = np.zeros((x.shape[0], IN_PAD), np.float64)
    xp[:, :IN] = x
    return xp


# ---- float64 reference -------------------------------------------------------
def exact_forward(params, x):
    w1, b1, w2, b2, w3, b3, w4, b4 = [np.asarray(p, np.float64) for p in params]
    a0 = _pad(np.asarray(x, np.float64))
    z1 = a0 @ w1.T + b1
    a1 = gelu(z1)
    z2 = a1 @ w2.T + b2
    a2 = gelu(z2)
    z3 = a2 @ w3.T + b3
    a3 = gelu(z3)
    y = a3 @ w4 + b4[0]
    return y, (a0, z1, a1, z2, a2, z3, a3)


def exact_loss(params, x, t):
    y, _ = exact_forward(params, x)
    return float(np.mean((y - np.asarray(t, np.float64)) ** 2))


def exact_gradients(params, x, t):
    w1, b1, w2, b2, w3, b3, w4, b4 = [np.asarray(p, np.float64) for p in params]
    y, (a0, z1, a1, z2, a2, z3, a3) = exact_forward(params, x)
    B = len(y)
    dy = 2.0 * (y - np.asarray(t, np.float64)) / B
    gw4 = a3.T @ dy
    gb4 = np.array([dy.sum()])
    dz3 = np.outer(dy, w4) * gelu_grad(z3)
    gw3, gb3 = dz3.T @ a2, dz3.sum(0)
    dz2 = (dz3 @ w3) * gelu_grad(z2)
    gw2, gb2 = dz2.T @ a1, dz2.sum(0)
    dz1 = (dz2 @ w2) * gelu_grad(z1)
    gw1, gb1 = dz1.T @ a0, dz1.sum(0)
    return [gw1, gb1, gw2, gb2, gw3, gb3, gw4, gb4]


# ---- the kernels' rounding points ----------------------------------------------
def mixed_forward(params, x):
    w1, b1, w2, b2, w3, b3, w4, b4 = params
    a = bf16(np.pad(np.asarray(x, np.float32), ((0, 0), (0, IN_PAD - IN)))).astype(np.float64)
    cache = [a]
    for w, b in ((w1, b1), (w2, b2), (w3, b3)):
        acc = (a @ bf16(w).astype(np.float64).T).astype(np.float32)
        z = (acc + np.asarray(b, np.float32)).astype(np.float32)
        zb = bf16(z)
        a = bf16(gelu(z.astype(np.float64)).astype(np.float32)).astype(np.float64)
        cache += [zb, a]
    y = (a @ np.asarray(w4, np.float64)).astype(np.float32) + np.float32(b4[0])
    return y.astype(np.float32), cache


def mixed_gradients(params, x, t):
    w1, b1, w2, b2, w3, b3, w4, b4 = params
    y, (a0, z1, a1, z2, a2, z3, a3) = mixed_forward(params, x)
    B = len(y)
    dy = (np.float32(2.0) * (y - np.asarray(t, np.float32)) / np.float32(B)).astype(np.float32)
    gw4 = a3.T @ dy.astype(np.float64)
    gb4 = np.array([dy.astype(np.float64).sum()])
    dz3 = bf16((np.outer(dy, np.asarray(w4, np.float32)) *
                gelu_grad(z3.astype(np.float64))).astype(np.float32)).astype(np.float64)
    gw3, gb3 = dz3.T @ a2, dz3.sum(0)
    da2 = (dz3 @ bf16(w3).astype(np.float64)).astype(np.float32)
    dz2 = bf16((da2 * gelu_grad(z2.astype(np.float64))).astype(np.float32)).astype(np.float64)
    gw2, gb2 = dz2.T @ a1, dz2.sum(0)
    da1 = (dz2 @ bf16(w2).astype(np.float64)).astype(np.float32)
    dz1 = bf16((da1 * gelu_grad(z1.astype(np.float64))).astype(np.float32)).astype(np.float64)
    gw1, gb1 = dz1.T @ a0, dz1.sum(0)
    loss = float(np.mean((y.astype(np.float64) - np.asarray(t, np.float64)) ** 2))
    return [gw1, gb1, gw2, gb2, gw3, gb3, gw4, gb4], loss


def adam(params, grads, m, v, step, lr, beta1=0.9, beta2=0.999, eps=1e-8):
    """One Adam step (FP32 state), returns new (params, m, v)."""
    bc1 = np.float32(1.0 - beta1 ** step)
    bc2 = np.float32(1.0 - beta2 ** step)
    out_p, out_m, out_v = [], [], []
    for p, g, mm, vv in zip(params, grads, m, v):
        g = np.asarray(g, np.float32)
        mm = np.float32(beta1) * mm + np.float32(1 - beta1) * g
        vv = np.float32(beta2) * vv + np.float32(1 - beta2) * g * g
        p = p - np.float32(lr) * (mm / bc1) / (np.sqrt(vv / bc2) + np.float32(eps))
        out_p.append(p.astype(np.float32))
        out_m.append(mm.astype(np.float32))
        out_v.append(vv.astype(np.float32))
    return out_p, out_m, out_v
