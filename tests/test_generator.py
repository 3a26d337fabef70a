"""The seven benchmark distributions of the reference's data generator
(data-generator/RandomDataGenerator.cpp:114-257) against the reference's own data
files (65,536-option sets thinned to every 64th option, tests/golden/reference/)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, FP64_ABS, FP64_REL

REF = os.path.join(GOLDEN, "reference")


def _shape(pkg, opts):
    s = pkg.shape(opts)
    return 2 * s["jmax"] + 1, opts.Maturities


def test_width_formula_inverse(pkg):
    """reversion_rate_for_width gives every odd width 5..4095 under the reference's
    width formula (common/OptionConstants.hpp:45-52), at 12 and at 48 steps/year."""
    wl = pkg.workloads
    w = np.arange(5, 4097, 2)
    for steps in (12, 48):
        a = wl.reversion_rate_for_width(w, steps)
        n = len(w)
        o = pkg.Options.from_batch(wl._batch(np.full(n, 63.0), np.full(n, 300.0), np.full(n, 3.0),
                                             np.full(n, steps), a, np.full(n, 0.01), np.ones(n)))
        assert np.array_equal(2 * pkg.shape(o)["jmax"] + 1, w)
    with pytest.raises(ValueError):
        wl.reversion_rate_for_width([6])


@pytest.mark.parametrize("kind", range(7))
def test_distribution_matches_reference_file(pkg, kind):
    stats = pytest.importorskip("scipy.stats")
    wl = pkg.workloads
    name = wl.THESIS_DATASETS[kind]
    ref = pkg.Options.from_file(os.path.join(REF, f"{name}_every64.in"))
    gen = pkg.Options.from_batch(wl.thesis_dataset(kind, 8192, seed=11))
    # the fields the generator fixes (RandomDataGenerator.cpp:93-104)
    for field in ("StrikePrices", "Lengths", "TermUnits", "TermStepCounts", "Volatilities", "Types"):
        r, g = getattr(ref, field), getattr(gen, field)
        assert np.all(r == r[0]) and np.all(g == r[0]), field
    wr, tr = _shape(pkg, ref)
    wg, tg = _shape(pkg, gen)
    assert np.all(wg % 2 == 1)
    # same support, same distribution (two-sample Kolmogorov-Smirnov, 1,024 vs 8,192)
    for r, g, what in ((wr, wg, "width"), (tr, tg, "bond maturity")):
        if np.all(r == r[0]):
            assert np.all(g == r[0]), what
            continue
        assert stats.ks_2samp(r, g).pvalue > 1e-3, what
    lo, hi = {0: (47, 47), 1: (7, 511), 2: (7, 511), 3: (47, 47), 4: (7, 511), 5: (7, 107), 6: (7, 511)}[kind]
    assert wg.min() >= lo and wg.max() <= hi


def test_skew_share(pkg):
    wl = pkg.workloads
    b = wl.thesis_dataset(4, 10000, skew_percent=5, seed=1)
    assert np.sum(b["bond_maturity"] >= 70) >= 500  # ceil(5% x 10,000) skewed, T in 70..100
    b6 = wl.thesis_dataset(6, 1000, seed=2)
    o = pkg.Options.from_batch(b6)
    w = 2 * pkg.shape(o)["jmax"] + 1
    assert np.sum(w >= 509) == 10 and len(np.unique(w[w >= 509])) == 1  # one skewed width


def test_generated_set_priced_by_oracle_like_reference_file(pkg, orc):
    """A generated 2_RANDCONSTHEIGHT sample and the reference's file price through
    the same oracle into the same range of values (same option family)."""
    wl = pkg.workloads
    y = pkg.Yield.from_file(os.path.join(REF, "yield.in"))
    gen = pkg.Options.from_batch(wl.thesis_dataset(2, 256, seed=3))
    p = orc.price(gen, y, "f64")
    with open(os.path.join(REF, "2_RANDCONSTHEIGHT_every64.out64")) as f:
        gold = np.array(pkg.read_arrays(f.read())[0], dtype=np.float64)
    assert np.all(np.isfinite(p))
    assert gold.min() - 0.5 <= np.median(p) <= gold.max() + 0.5


def test_single_tree_workloads(pkg):
    """The surrogate's single-tree box and batches (configs[4] as written): training
    samples drawn as the 1,000-option book (only strike and type vary), queries with
    exactly 10% outside the box, each flagged one outside it in one parameter."""
    import numpy as np
    wl = pkg.workloads
    box = wl.single_tree_box()
    tr = wl.single_tree_training_batch(50_000, seed=3)
    for k in ("bond_maturity", "option_maturity", "a", "sigma", "term_steps"):
        assert np.unique(tr[k]).size == 1, k
    assert set(np.unique(tr["type"])) == {0, 1}
    q = wl.single_tree_query_batch(100_000, seed=4)
    assert q["outside"].sum() == 10_000
    fwd = wl.forward_bond_price(q["option_maturity"], q["bond_maturity"])
    mny = q["strike"] / fwd
    span = q["bond_maturity"] - q["option_maturity"]
    inside = ((q["option_maturity"] >= box["t_min"]) & (q["option_maturity"] <= box["t_max"])
              & (span >= box["span_min"]) & (span <= box["span_max"])
              & (mny >= box["moneyness_min"]) & (mny <= box["moneyness_max"])
              & (q["a"] >= box["a_min"]) & (q["a"] <= box["a_max"])
              & (q["sigma"] >= box["sigma_min"]) & (q["sigma"] <= box["sigma_max"])
              & (q["term_steps"] >= box["steps_min"]) & (q["term_steps"] <= box["steps_max"]))
    assert np.array_equal(inside, ~q["outside"])
