"""ORACLE - test infrastructure, not the product.

FP64 numpy restatement of the surrogate MLP that the GPU trains and evaluates
(8 inputs: 7 features and a zero pad -> 4 x 256 SiLU -> 2 outputs: the price
target and the error head).  The reference project has no learned part, so this
restatement is the oracle for the GPU forward pass, the gradients and the Adam
step; it is itself checked by central finite differences (tests/test_mlp_oracle.py).

Layout matches the GPU kernels: W_l is [fan_in, fan_out] row-major, y = x W + b.
The GPU computes layers 0 and 4 in fp32 (layer 0 from fp32 features, layer 4 from
layer 3's fp32 activations), feeds layer 1 its input as a bf16 hi / lo pair, and keeps
bf16 copies of the weights of layers 1-3 and bf16 activations between layers 1-3 with
fp32 accumulation; `forward(..., bf16=True)`
rounds the same tensors the same way so the comparison isolates accumulation-order
and activation-approximation differences.

Loss: 0.5 mean((o0 - y)^2) + err_weight * 0.5 mean((o1 - log(|o0 - y| + eps))^2),
the error head's target held constant (no gradient flows through it).
"""
from __future__ import annotations

import numpy as np

DIMS = (8, 256, 256, 256, 256, 2)
ERR_EPS = 1e-3


def bf16_round(x: np.ndarray) -> np.ndarray:
    """Round-to-nearest-even to bfloat16, returned as float64."""
    f = np.asarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    rounding = ((u >> 16) & 1) + 0x7FFF
    u = ((u + rounding) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def init_params(seed: int = 0, dims=DIMS):
    """He-style init: W ~ N(0, 1/fan_in) scaled for SiLU, b = 0."""
    rng = np.random.default_rng(seed)
    params = []
    for fi, fo in zip(dims[:-1], dims[1:]):
        W = rng.standard_normal((fi, fo)) * np.sqrt(2.0 / fi)
        if fo == 1:
            W *= 0.1
        params.append((W, np.zeros(fo)))
    return params


def forward(params, x, bf16: bool = False):
    """Returns (outputs [n, fan_out of the last layer], cache of pre-activations and
    layer inputs)."""
    h = np.asarray(x, dtype=np.float64)
    inputs, pre = [], []
    last = len(params) - 1
    for li, (W, b) in enumerate(params):
        Wq = bf16_round(W) if (bf16 and 0 < li < last) else W
        inputs.append(h)
        z = h @ Wq + b
        pre.append(z)
        if li < last:
            h = silu(z)
            # the last layer reads fp32 activations and layer 1 a bf16 hi / lo pair
            # (about 16 bits), taken as exact here
            if bf16 and 0 < li < last - 1:
                h = bf16_round(h)
        else:
            h = z
    return h, {"inputs": inputs, "pre": pre}


def loss_and_grads(params, x, y, bf16: bool = False, err_weight: float = 0.0, eps: float = ERR_EPS):
    """Loss (module docstring) and its gradients; a one-output network has only the
    squared-error term."""
    out, cache = forward(params, x, bf16)
    n = x.shape[0]
    r = out[:, 0] - y
    loss = 0.5 * float(np.mean(r * r))
    g = np.zeros_like(out)
    g[:, 0] = r / n
    if out.shape[1] > 1:
        r1 = out[:, 1] - np.log(np.abs(r) + eps)
        loss += err_weight * 0.5 * float(np.mean(r1 * r1))
        g[:, 1] = err_weight * r1 / n
    grads = [None] * len(params)
    last = len(params) - 1
    for li in range(last, -1, -1):
        W, _ = params[li]
        Wq = bf16_round(W) if (bf16 and 0 < li < last) else W
        if li < last:
            g = g * dsilu(cache["pre"][li])
        a = cache["inputs"][li]
        grads[li] = (a.T @ g, g.sum(axis=0))
        g = g @ Wq.T
    return loss, grads


def adam_step(params, grads, state, lr, beta1=0.9, beta2=0.999, eps=1e-8):
    """One Adam update (bias-corrected), in place on params; returns state."""
    t = state.get("t", 0) + 1
    state["t"] = t
    m = state.setdefault("m", [(np.zeros_like(W), np.zeros_like(b)) for W, b in params])
    v = state.setdefault("v", [(np.zeros_like(W), np.zeros_like(b)) for W, b in params])
    c1 = 1.0 - beta1 ** t
    c2 = 1.0 - beta2 ** t
    for i, ((W, b), (gW, gb)) in enumerate(zip(params, grads)):
        mW, mb = m[i]
        vW, vb = v[i]
        mW[:] = beta1 * mW + (1 - beta1) * gW
        mb[:] = beta1 * mb + (1 - beta1) * gb
        vW[:] = beta2 * vW + (1 - beta2) * gW * gW
        vb[:] = beta2 * vb + (1 - beta2) * gb * gb
        W -= lr * (mW / c1) / (np.sqrt(vW / c2) + eps)
        b -= lr * (mb / c1) / (np.sqrt(vb / c2) + eps)
    return state


def cosine_lr(step: int, total: int, lr0: float = 1e-3, lr_min: float = 0.0) -> float:
    return lr_min + 0.5 * (lr0 - lr_min) * (1.0 + np.cos(np.pi * min(step, total) / max(total, 1)))
