"""Seeded synthetic option batches with the shapes of the benchmark configurations.

No public data set exists for these workloads; every batch is generated here from a
fixed numpy seed so the GPU path, the oracle and the CPU baseline see identical
inputs.  Records use the reference's SoA option fields (common/Options.hpp:48-58):
strike, bond maturity (Maturities), option maturity (Lengths), term unit, term steps
per year, mean reversion a, volatility sigma, type (0 = CALL, 1 = PUT).

The yield curve is 11 nodes at 0.25/0.5/1/2/3/5/7/10/15/20/30 years, held as whole
days (common/Yield.hpp:17-18 stores int32 days), with continuously compounded zero
rates rising linearly in maturity from 1.0% to 4.0%.
"""
from __future__ import annotations

import numpy as np

CURVE_YEARS = (0.25, 0.5, 1.0, 2.0, 3.0, 5.0, 7.0, 10.0, 15.0, 20.0, 30.0)


def yield_curve():
    """(rates float64[11], days int32[11]) of the synthetic curve."""
    years = np.array(CURVE_YEARS)
    days = np.array([int(y * 365 + 0.5) for y in CURVE_YEARS], dtype=np.int32)
    rates = 0.01 + 0.03 * (years - years[0]) / (years[-1] - years[0])
    return rates.astype(np.float64), days


def _curve_rate(t_years, rates, days, term_unit=365):
    """Zero rate at t the way common/Domain.hpp:11-46 interpolates it (whole days)."""
    t_days = np.floor(np.asarray(t_years, dtype=np.float64) * term_unit + 0.5).astype(np.int64)
    days = np.asarray(days, dtype=np.int64)
    rates = np.asarray(rates, dtype=np.float64)
    s = np.clip(np.searchsorted(days, t_days, side="left"), 1, len(days) - 1)
    f = s - 1
    inner = rates[f] + (t_days - days[f]) / (days[s] - days[f]).astype(np.float64) * (rates[s] - rates[f])
    return np.where(t_days <= days[0], rates[0], np.where(t_days > days[-1], rates[-1], inner))


def forward_bond_price(option_maturity, bond_maturity, rates=None, days=None):
    """100 * P(0,T) / P(0,t) from the curve's zero rates."""
    if rates is None:
        rates, days = yield_curve()
    t = np.asarray(option_maturity, dtype=np.float64)
    T = np.asarray(bond_maturity, dtype=np.float64)
    pt = np.exp(-_curve_rate(t, rates, days) * t)
    pT = np.exp(-_curve_rate(T, rates, days) * T)
    return 100.0 * pT / pt


def _batch(strike, T, t, steps, a, sigma, typ):
    n = len(strike)
    return dict(
        strike=np.asarray(strike, dtype=np.float64),
        bond_maturity=np.asarray(T, dtype=np.float64),
        option_maturity=np.asarray(t, dtype=np.float64),
        term_unit=np.full(n, 365, dtype=np.uint16),
        term_steps=np.asarray(steps, dtype=np.uint16),
        a=np.asarray(a, dtype=np.float64),
        sigma=np.asarray(sigma, dtype=np.float64),
        type=np.asarray(typ, dtype=np.int8),
    )


def uniform_book(n=1000, seed=0):
    """1,000 options: t=5y, T=10y, 12 steps/year (jmax 23, width 47, height 120),
    a=0.10, sigma=0.01, strike U[75,95], call/put 50/50."""
    rng = np.random.default_rng(seed)
    return _batch(rng.uniform(75.0, 95.0, n), np.full(n, 10.0), np.full(n, 5.0), np.full(n, 12),
                  np.full(n, 0.10), np.full(n, 0.01), rng.integers(0, 2, n))


def uneven_batch(n=30000, seed=1):
    """30,000 uneven options: t U{1..10}, T = t + U{1..10}, steps/year U{6..48},
    a U[0.02,0.20], sigma U[0.005,0.02], strike = forward bond price x U[0.9,1.1]."""
    rng = np.random.default_rng(seed)
    t = rng.integers(1, 11, n).astype(np.float64)
    T = t + rng.integers(1, 11, n)
    steps = rng.integers(6, 49, n)
    a = rng.uniform(0.02, 0.20, n)
    sigma = rng.uniform(0.005, 0.02, n)
    strike = forward_bond_price(t, T) * rng.uniform(0.9, 1.1, n)
    return _batch(strike, T, t, steps, a, sigma, rng.integers(0, 2, n))


def skewed_batch(n=100000, seed=2, heavy_fraction=0.01):
    """100,000 options, 1% heavy.  Light: a U[0.10,0.20], 12 steps/year, t U{1..5},
    T U{t+1..10}.  Heavy: a U[0.01,0.02], steps/year U{48..96}, t U{10..20},
    T U{t+1..30}.  sigma=0.01, strike U[75,95], call/put 50/50 for both."""
    rng = np.random.default_rng(seed)
    heavy = np.zeros(n, dtype=bool)
    heavy[rng.permutation(n)[: int(round(n * heavy_fraction))]] = True
    t = np.where(heavy, rng.integers(10, 21, n), rng.integers(1, 6, n)).astype(np.float64)
    span = np.where(heavy, 30.0 - t, 10.0 - t)
    T = t + 1.0 + np.floor(rng.uniform(0.0, 1.0, n) * span)
    steps = np.where(heavy, rng.integers(48, 97, n), 12)
    a = np.where(heavy, rng.uniform(0.01, 0.02, n), rng.uniform(0.10, 0.20, n))
    return _batch(rng.uniform(75.0, 95.0, n), T, t, steps, a, np.full(n, 0.01), rng.integers(0, 2, n))


def book_batch(count=100):
    """The reference's 'Book options' unit-test batch (test/TestCuda.cu:20-31):
    t=3, T=9, strike 63, term unit 365, steps 1..count, a=0.1, sigma=0.01, PUT."""
    k = np.arange(1, count + 1)
    return _batch(np.full(count, 63.0), np.full(count, 9.0), np.full(count, 3.0), k,
                  np.full(count, 0.1), np.full(count, 0.01), np.ones(count))


# ---------------------------------------------------------------------------
# The reference's seven benchmark distributions
# ---------------------------------------------------------------------------
# data-generator/RandomDataGenerator.cpp:114-257 writes the seven data/*.in sets
# the thesis benchmarks (65,536 options each): every option is a PUT on a bond,
# option maturity 3 y, strike 63, term unit 365, 12 steps per year, sigma 0.01;
# what varies is the bond maturity T (tree height 12 T + 1) and the tree width,
# which the generator sets through the mean reversion a.  It draws widths from a
# table of odd widths 7..1023 with a 5-decimal `a` for each; here `a` is computed
# for any odd width from the width formula itself (reversion_rate_for_width), and
# the draws come from numpy's generator instead of C rand(), so the sets have the
# reference's distributions, not its exact records.

THESIS_DATASETS = ("0_UNIFORM", "1_RAND", "2_RANDCONSTHEIGHT", "3_RANDCONSTWIDTH", "4_SKEWED",
                   "5_SKEWEDCONSTHEIGHT", "6_SKEWEDCONSTWIDTH")


def reversion_rate_for_width(width, steps_per_year=12):
    """Mean reversion a for which the reference's width formula
    (common/OptionConstants.hpp:45-52: jmax = (int)(-0.184 / (exp(-a dt) - 1)) + 1,
    width = 2 jmax + 1, dt = 1 / steps_per_year at term unit 365) gives `width`
    (odd, >= 5): the midpoint of the interval of a that truncates to that jmax."""
    w = np.asarray(width, dtype=np.int64)
    if np.any(w % 2 == 0) or np.any(w < 5):
        raise ValueError("widths are odd and at least 5")
    jmax = (w - 1) // 2
    dt = 1.0 / steps_per_year
    # -0.184 / (exp(-a dt) - 1) in [jmax - 1, jmax)  <=>  a in (a_lo, a_hi]
    a_lo = -np.log1p(-0.184 / jmax) / dt
    a_hi = -np.log1p(-0.184 / (jmax - 1)) / dt
    return 0.5 * (a_lo + a_hi)


def _odd_widths(rng, lo, hi, n):
    """Uniform draws from the odd widths in [lo, hi]."""
    first = lo if lo % 2 else lo + 1
    count = (hi - first) // 2 + 1
    return first + 2 * rng.integers(0, count, n)


def thesis_dataset(kind, n=65536, skew_percent=1, seed=0):
    """One of the reference's seven benchmark distributions (kind 0..6 or its name),
    n options, shuffled:
      0 UNIFORM            T = 9, a = 0.1 (width 47)
      1 RAND               T U{1..100}, width U(odd 7..511)
      2 RANDCONSTHEIGHT    T = 9, width U(odd 7..511)
      3 RANDCONSTWIDTH     T U{1..100}, a = 0.1
      4 SKEWED             skew%: T U{70..100}, width U(odd 411..511); rest T U{1..30}, width U(odd 7..107)
      5 SKEWEDCONSTHEIGHT  skew%: T = 100, width U(odd 7..107); rest as in 4
      6 SKEWEDCONSTWIDTH   skew%: T U{1..30}, one width from U(odd 509..511); rest as in 4
    (RandomDataGenerator.cpp:114-257; the skewed share is ceil(skew% x n))."""
    if isinstance(kind, str):
        kind = THESIS_DATASETS.index(kind)
    rng = np.random.default_rng(seed)
    n_skew = int(np.ceil(skew_percent / 100.0 * n)) if kind >= 4 else 0
    n_rest = n - n_skew
    a = np.full(n, 0.1)
    if kind == 0:
        T = np.full(n, 9)
    elif kind == 1:
        T = rng.integers(1, 101, n)
        a = reversion_rate_for_width(_odd_widths(rng, 7, 511, n))
    elif kind == 2:
        T = np.full(n, 9)
        a = reversion_rate_for_width(_odd_widths(rng, 7, 511, n))
    elif kind == 3:
        T = rng.integers(1, 101, n)
    else:
        if kind == 4:
            T_s = rng.integers(70, 101, n_skew)
            w_s = _odd_widths(rng, 411, 511, n_skew)
        elif kind == 5:
            T_s = np.full(n_skew, 100)
            w_s = _odd_widths(rng, 7, 107, n_skew)
        elif kind == 6:
            T_s = rng.integers(1, 31, n_skew)
            w_s = np.full(n_skew, _odd_widths(rng, 509, 511, 1)[0])
        else:
            raise ValueError(f"unknown dataset kind {kind}")
        T = np.concatenate([T_s, rng.integers(1, 31, n_rest)])
        a = reversion_rate_for_width(np.concatenate([w_s, _odd_widths(rng, 7, 107, n_rest)]))
    perm = rng.permutation(n)
    T = np.asarray(T, dtype=np.float64)[perm]
    a = np.asarray(a, dtype=np.float64)[perm]
    return _batch(np.full(n, 63.0), T, np.full(n, 3.0), np.full(n, 12), a, np.full(n, 0.01), np.ones(n))


WORKLOADS = {
    "uniform_1k": uniform_book,
    "uneven_30k": uneven_batch,
    "skewed_100k": skewed_batch,
}
WORKLOADS.update({name.lower(): (lambda k: (lambda: thesis_dataset(k)))(k) for k, name in enumerate(THESIS_DATASETS)})


# ---------------------------------------------------------------------------
# Surrogate: training box and query batches
# ---------------------------------------------------------------------------
# The network's box is the uneven batch's own parameter box (the batch it must
# price): t in [1, 10], T - t in [1, 10], strike / forward bond price in
# [0.9, 1.1], a in [0.02, 0.20], sigma in [0.005, 0.02], 6..48 steps per year,
# term unit 365.
SURROGATE_BOX = dict(t_min=1.0, t_max=10.0, span_min=1.0, span_max=10.0, moneyness_min=0.9, moneyness_max=1.1,
                     a_min=0.02, a_max=0.20, sigma_min=0.005, sigma_max=0.02, steps_min=6, steps_max=48,
                     term_unit=365)


def surrogate_training_batch(n=4_000_000, seed=3):
    """Training samples: the uneven batch's distribution (seed 3)."""
    return uneven_batch(n, seed)


def surrogate_query_batch(n=1_000_000, seed=4, outside_fraction=0.10):
    """Queries: 90% drawn like the uneven batch, 10% outside the box (longer
    option or bond maturities, faster mean reversion, finer time steps or
    strikes further from the forward), in random order."""
    rng = np.random.default_rng(seed)
    b = uneven_batch(n, seed)
    out = rng.permutation(n)[: int(round(n * outside_fraction))]
    kind = rng.integers(0, 4, len(out))
    t, T, steps, a, strike = (b["option_maturity"], b["bond_maturity"], b["term_steps"], b["a"], b["strike"])
    for k, idx in ((0, out[kind == 0]), (1, out[kind == 1]), (2, out[kind == 2]), (3, out[kind == 3])):
        if k == 0:    # option maturity 11-15 y
            t[idx] = rng.integers(11, 16, len(idx))
            T[idx] = t[idx] + rng.integers(1, 11, len(idx))
        elif k == 1:  # a above the box
            a[idx] = rng.uniform(0.21, 0.30, len(idx))
        elif k == 2:  # 49-64 steps per year
            steps[idx] = rng.integers(49, 65, len(idx))
        else:         # strike 12-20% away from the forward
            sign = np.where(rng.integers(0, 2, len(idx)) == 0, -1.0, 1.0)
            strike[idx] = forward_bond_price(t[idx], T[idx]) * (1.0 + sign * rng.uniform(0.12, 0.20, len(idx)))
    b["outside"] = np.zeros(n, dtype=bool)
    b["outside"][out] = True
    return b


# ---------------------------------------------------------------------------
# Surrogate on the single-tree box: samples drawn as the 1,000-option book draws
# them (t = 5 y, T = 10 y, 12 steps/year, a = 0.10, sigma = 0.01; strike U[75, 95],
# call/put 50/50), so only strike and type vary.  The tree's price is then a
# piecewise-linear function of strike, with a kink at each maturity-row bond value.
# ---------------------------------------------------------------------------
def _book_forward():
    return float(forward_bond_price(5.0, 10.0))


def single_tree_box():
    """Training box of the single-tree surrogate: the book's fixed tree parameters,
    strike / forward bond price in [75, 95] / F(5 y, 10 y)."""
    f = _book_forward()
    return dict(t_min=5.0, t_max=5.0, span_min=5.0, span_max=5.0, moneyness_min=75.0 / f, moneyness_max=95.0 / f,
                a_min=0.10, a_max=0.10, sigma_min=0.01, sigma_max=0.01, steps_min=12, steps_max=12, term_unit=365)


def single_tree_training_batch(n=4_000_000, seed=3):
    """Training samples drawn as the 1,000-option book (seed 3)."""
    return uniform_book(n, seed)


def single_tree_query_batch(n=1_000_000, seed=4, outside_fraction=0.10):
    """Queries: the book's distribution, with 10% drawn outside the single-tree box
    (strike 60-75 or 95-110, a in [0.05, 0.2], sigma in [0.005, 0.02], 6-48 steps per
    year, or option maturity 1-4 y), in random order."""
    rng = np.random.default_rng(seed)
    b = uniform_book(n, seed)
    out = rng.permutation(n)[: int(round(n * outside_fraction))]
    kind = rng.integers(0, 5, len(out))
    strike, a, sigma, steps, t = b["strike"], b["a"], b["sigma"], b["term_steps"], b["option_maturity"]
    for k in range(5):
        idx = out[kind == k]
        if k == 0:
            lo = rng.integers(0, 2, len(idx)) == 0
            strike[idx] = np.where(lo, rng.uniform(60.0, 74.5, len(idx)), rng.uniform(95.5, 110.0, len(idx)))
        elif k == 1:
            a[idx] = np.where(rng.integers(0, 2, len(idx)) == 0, rng.uniform(0.05, 0.095, len(idx)),
                              rng.uniform(0.105, 0.20, len(idx)))
        elif k == 2:
            sigma[idx] = np.where(rng.integers(0, 2, len(idx)) == 0, rng.uniform(0.005, 0.0095, len(idx)),
                                  rng.uniform(0.0105, 0.02, len(idx)))
        elif k == 3:
            steps[idx] = np.where(rng.integers(0, 2, len(idx)) == 0, rng.integers(6, 12, len(idx)),
                                  rng.integers(13, 49, len(idx)))
        else:
            t[idx] = rng.integers(1, 5, len(idx)).astype(np.float64)
    b["outside"] = np.zeros(n, dtype=bool)
    b["outside"][out] = True
    return b
