"""Host logic of the surrogate's single-tree routing, without a GPU: the kink
finder on prices of the 1,000-option book's tree from the oracle, and the
per-point routing distances against a numpy restatement of their definition."""
import numpy as np
import pytest


def test_route_distances_cover_every_sample_above_the_tolerance(pkg):
    rng = np.random.default_rng(5)
    points = np.sort(rng.uniform(0.0, 1.0, 12))
    x = rng.uniform(-0.1, 1.1, 20_000)
    err = np.abs(rng.normal(0.0, 4e-5, x.size))
    err[rng.integers(0, x.size, 40)] = 3e-4  # scattered large errors
    tol = 1e-4
    delta, answered = pkg.route_distances(points, x, err, tol)
    near = np.argmin(np.abs(x[:, None] - points[None, :]), axis=1)
    dist = np.abs(x - points[near])
    want = np.full(points.size, -1.0)
    for k in range(points.size):
        sel = (near == k) & (err > tol)
        if sel.any():
            want[k] = dist[sel].max()
    assert np.array_equal(delta, want)
    covered = (np.abs(x[:, None] - points[None, :]) <= delta[None, :]).any(axis=1)
    assert np.all(covered[err > tol])          # every sample above tol goes to the tree
    assert np.all(err[~covered] <= tol)        # what the network keeps is within tol
    assert answered == pytest.approx(np.mean(~covered), abs=0.0)
    # nothing above the tolerance: no distances, everything answered
    d0, a0 = pkg.route_distances(points, x, np.zeros_like(x), tol)
    assert np.all(d0 == -1.0) and a0 == 1.0
    d1, a1 = pkg.route_distances(points, np.zeros(0), np.zeros(0), tol)
    assert np.all(d1 == -1.0) and a1 == 1.0


def test_find_kinks_on_the_book_tree(pkg, orc):
    """The book's tree (t = 5 y, T = 10 y, 12 steps/year, a = 0.10, sigma = 0.01):
    its price is piecewise linear in the strike, with 12 kinks between strikes 75 and
    95; between two found kinks the oracle's prices lie on a line."""
    wl = pkg.workloads
    rates, days = wl.yield_curve()
    y = pkg.Yield(rates, days)
    strikes = np.linspace(75.0, 95.0, 20001)
    b = wl.uniform_book(2 * strikes.size, seed=0)
    b["strike"] = np.concatenate([strikes, strikes])
    b["type"] = np.concatenate([np.zeros(strikes.size), np.ones(strikes.size)]).astype(np.int8)
    price = orc.price(pkg.Options.from_batch(b), y, "f64")
    fwd = wl.forward_bond_price(5.0, 10.0)
    x = b["strike"] / fwd
    kinks = pkg.find_kinks(x, price, b["type"])
    assert kinks.size == 12, kinks
    assert np.all(np.diff(kinks) > 0)
    # linear between kinks: second differences of the price vanish away from them
    step = x[1] - x[0]
    for t in (0, 1):
        xs, ps = x[b["type"] == t], price[b["type"] == t]
        d2 = ps[2:] - 2.0 * ps[1:-1] + ps[:-2]
        far = np.min(np.abs(xs[1:-1, None] - kinks[None, :]), axis=1) > 2.5 * step
        assert np.max(np.abs(d2[far])) < 1e-9, np.max(np.abs(d2[far]))
    # more kinks than the caller's room: not one tree
    with pytest.raises(ValueError):
        pkg.find_kinks(x, price, b["type"], cap=4)
