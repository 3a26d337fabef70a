"""The surrogate's FP64 CPU oracle checked by central finite differences (it is
the reference for the GPU gradients)."""
import os
import sys

import numpy as np

from conftest import ROOT

sys.path.insert(0, os.path.join(ROOT, "oracle"))
import mlp_oracle as mo  # noqa: E402


def test_gradients_match_finite_differences():
    dims = (7, 16, 16, 1)
    params = mo.init_params(3, dims)
    rng = np.random.default_rng(0)
    x = rng.standard_normal((32, 7))
    y = rng.standard_normal(32) * 0.1
    _, grads = mo.loss_and_grads(params, x, y)
    eps = 1e-6
    for li, (W, b) in enumerate(params):
        for (i, j) in ((0, 0), (W.shape[0] - 1, W.shape[1] - 1), (W.shape[0] // 2, W.shape[1] // 2)):
            old = W[i, j]
            W[i, j] = old + eps
            lp, _ = mo.loss_and_grads(params, x, y)
            W[i, j] = old - eps
            lm, _ = mo.loss_and_grads(params, x, y)
            W[i, j] = old
            fd = (lp - lm) / (2 * eps)
            assert abs(fd - grads[li][0][i, j]) <= 1e-6 * max(1.0, abs(fd)), (li, i, j, fd, grads[li][0][i, j])
        old = b[0]
        b[0] = old + eps
        lp, _ = mo.loss_and_grads(params, x, y)
        b[0] = old - eps
        lm, _ = mo.loss_and_grads(params, x, y)
        b[0] = old
        assert abs((lp - lm) / (2 * eps) - grads[li][1][0]) <= 1e-6


def test_bf16_rounding():
    # spacing at 1 is 2^-7; halfway cases go to the even mantissa
    v = np.array([1.0, 1.00390625, 1.001953125, -3.14159, 0.0, 1.01171875])
    r = mo.bf16_round(v)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 and r[5] == 1.015625
    assert abs(r[3] + 3.140625) < 1e-12


def test_adam_decreases_loss():
    dims = (7, 32, 32, 1)
    params = mo.init_params(1, dims)
    rng = np.random.default_rng(2)
    x = rng.standard_normal((256, 7))
    y = np.sin(x[:, 0]) * 0.1
    state = {}
    l0, _ = mo.loss_and_grads(params, x, y)
    for step in range(200):
        _, g = mo.loss_and_grads(params, x, y)
        mo.adam_step(params, g, state, mo.cosine_lr(step, 200, 3e-3))
    l1, _ = mo.loss_and_grads(params, x, y)
    assert l1 < 0.2 * l0


def test_error_head_gradients_match_finite_differences():
    """Two outputs: the error head's target log(|o0 - y| + eps) is held constant, so
    the analytic gradients equal finite differences of the loss with that target
    frozen at the unperturbed parameters."""
    dims = (8, 12, 12, 2)
    params = mo.init_params(5, dims)
    rng = np.random.default_rng(4)
    x = rng.standard_normal((24, 8))
    y = rng.standard_normal(24) * 0.1
    w = 0.3
    out0, _ = mo.forward(params, x)
    target = np.log(np.abs(out0[:, 0] - y) + mo.ERR_EPS)

    def frozen_loss():
        o, _ = mo.forward(params, x)
        r = o[:, 0] - y
        r1 = o[:, 1] - target
        return 0.5 * np.mean(r * r) + w * 0.5 * np.mean(r1 * r1)

    loss, grads = mo.loss_and_grads(params, x, y, err_weight=w)
    assert abs(loss - frozen_loss()) <= 1e-12
    eps = 1e-6
    for li, (W, b) in enumerate(params):
        for (i, j) in ((0, 0), (W.shape[0] - 1, W.shape[1] - 1)):
            old = W[i, j]
            W[i, j] = old + eps
            lp = frozen_loss()
            W[i, j] = old - eps
            lm = frozen_loss()
            W[i, j] = old
            fd = (lp - lm) / (2 * eps)
            assert abs(fd - grads[li][0][i, j]) <= 1e-6 * max(1.0, abs(fd)), (li, i, j, fd, grads[li][0][i, j])
