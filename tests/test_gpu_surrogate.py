"""Surrogate MLP on the GPU: tensor-core forward and backward against the FP64
CPU oracle (oracle/mlp_oracle.py), training, box routing and the tree judge."""
import os
import sys

import numpy as np
import pytest

from conftest import ROOT, load_set

sys.path.insert(0, os.path.join(ROOT, "oracle"))
import mlp_oracle as mo  # noqa: E402

pytestmark = pytest.mark.gpu

DIMS = (8, 256, 256, 256, 256, 1)


def _oracle_params(seed):
    p = mo.init_params(seed, DIMS)
    p[0][0][7, :] = 0.0  # the pad row of the first layer
    return p


@pytest.fixture(scope="module")
def sur(pkg, pricer):
    s = pkg.Surrogate(pricer, seed=5)
    yield s
    s.close()


def test_forward_matches_oracle(sur):
    params = _oracle_params(1)
    sur.set_params(params)
    rng = np.random.default_rng(0)
    x = rng.standard_normal((777, 7))
    got = sur.forward(x)
    ref, _ = mo.forward(params, np.hstack([x, np.zeros((len(x), 1))]), bf16=True)
    scale = np.std(ref) + np.mean(np.abs(ref))
    err = np.abs(got - ref)
    # bf16 activations: a rounding tie can flip one hidden unit by one bf16 ulp
    assert np.max(err) <= 2e-2 * scale, np.max(err) / scale
    assert np.mean(err) <= 2e-3 * scale


def test_gradients_match_oracle(sur):
    params = _oracle_params(2)
    sur.set_params(params)
    rng = np.random.default_rng(1)
    x = rng.standard_normal((2048, 7))
    y = rng.standard_normal(2048) * 0.5
    loss, grads = sur.loss_grads(x, y)
    rl, rg = mo.loss_and_grads(params, np.hstack([x, np.zeros((len(x), 1))]), y, bf16=True)
    assert abs(loss - rl) <= 1e-2 * abs(rl)
    for li, ((gw, gb), (rw, rb)) in enumerate(zip(grads, rg)):
        if li == 0:
            gw, rw = gw[:7], rw[:7]
        for a, b in ((gw, rw), (gb, rb)):
            rel = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)
            assert rel <= 5e-2, (li, rel)


def test_train_route_judge_and_checkpoint(pkg, pricer, orc, tmp_path):
    wl = pkg.workloads
    rates, days = wl.yield_curve()
    y = pkg.Yield(rates, days)
    s = pkg.Surrogate(pricer, seed=3)
    train = pkg.Options.from_batch(wl.surrogate_training_batch(65536, seed=21))
    st = s.train(train, y, epochs=3, batch=8192, lr=1e-3)
    assert st["steps"] == 3 * (65536 // 8192) and np.isfinite(st["final_loss"])
    q = wl.surrogate_query_batch(4000, seed=22, outside_fraction=0.1)
    opts = pkg.Options.from_batch(q)
    got = s.price(opts, y, judge_fraction=0.05, seed=9, tree_mode=pkg.BATCHED_FP64)
    stats = s.stats.as_dict()
    ref = orc.price(opts, y, "f64")
    out = q["outside"]
    assert stats["n_routed"] == int(out.sum())
    # out-of-box options come back from the FP64 tree
    assert np.max(np.abs(got[out] - ref[out])) <= 1e-10 * np.max(np.abs(ref)) + 1e-12
    assert 100 <= stats["n_judged"] <= 300
    assert np.isfinite(got).all()
    # a short training run already lands within a few percent of forward on average
    inb = ~out
    fwd = wl.forward_bond_price(q["option_maturity"], q["bond_maturity"])
    assert np.mean(np.abs(got[inb] - ref[inb]) / fwd[inb]) < 5e-2
    # a judge tolerance the short-trained network cannot meet sends the batch to the tree
    fb = s.price(opts, y, judge_fraction=0.05, seed=9, tree_mode=pkg.BATCHED_FP64, judge_tolerance=1e-9)
    assert s.stats.as_dict()["fell_back"] == 1
    assert np.max(np.abs(fb - ref)) <= 1e-10 * np.max(np.abs(ref)) + 1e-12
    # checkpoint round trip: same network output after loading into a fresh model
    path = str(tmp_path / "sur.bin")
    s.save(path)
    s2 = pkg.Surrogate(pricer, seed=99)
    s2.load(path)
    x = np.random.default_rng(3).standard_normal((64, 7))
    assert np.array_equal(s.forward(x), s2.forward(x))
    s.close()
    s2.close()


def test_bounded_wait_reports_timeout_and_context_survives(pkg, sur):
    """Failure path of the tensor-core GEMM without a GPU fault: with the stall
    injected, every GEMM's mbarrier wait runs out (a phase nothing completes), the
    call returns HWT_ETIMEOUT, and the next call on the same surrogate works."""
    params = _oracle_params(2)
    sur.set_params(params)
    x = np.random.default_rng(1).standard_normal((300, 7))
    ok = sur.forward(x)
    sur.inject_stall(True)
    try:
        with pytest.raises(pkg.HwtError) as e:
            sur.forward(x)
        assert e.value.code == pkg.HWT_ETIMEOUT
    finally:
        sur.inject_stall(False)
    assert np.array_equal(sur.forward(x), ok)
