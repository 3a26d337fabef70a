"""GPU tests of the C ABI beyond the golden sets: full-size parity, size-independent
properties, the device-memory entry point, graphs, error behaviour, the autotuner
and the command-line tools."""
import os
import subprocess

import numpy as np
import pytest

from conftest import FP64_ABS, FP64_REL, GOLDEN, LOWP_ABS, ROOT, assert_fp64, assert_lowp, load_set

pytestmark = pytest.mark.gpu

TOOLS = os.path.join(ROOT, "diku.optionspricing_gb300", "_build")


def _curve(pkg):
    rates, days = pkg.workloads.yield_curve()
    return pkg.Yield(rates, days)


@pytest.fixture(scope="module")
def uneven(pkg, orc):
    opts = pkg.Options.from_batch(pkg.workloads.uneven_batch())
    y = _curve(pkg)
    return opts, y, orc.price(opts, y, "f64")


def test_full_uneven_batch_fp64_and_mixed(pkg, pricer, uneven):
    """The whole 30,000-option uneven batch against the oracle."""
    opts, y, ref = uneven
    assert_fp64(pricer.price(opts, y, pkg.BATCHED_FP64), ref, "uneven_30k fp64")
    assert_fp64(pricer.price(opts, y, pkg.BATCHED_DF64), ref, "uneven_30k df64")
    assert_lowp(pricer.price(opts, y, pkg.BATCHED_MIXED), ref, "uneven_30k mixed")
    assert_lowp(pricer.price(opts, y, pkg.BATCHED_FP32), ref, "uneven_30k fp32")


def test_full_skewed_batch_fp64(pkg, pricer, orc):
    """The whole 100,000-option skewed batch (1% trees up to 3,521 nodes wide)."""
    opts = pkg.Options.from_batch(pkg.workloads.skewed_batch())
    y = _curve(pkg)
    ref = orc.price(opts, y, "f64")
    assert_fp64(pricer.price(opts, y, pkg.BATCHED_FP64), ref, "skewed_100k fp64")
    assert_fp64(pricer.price(opts, y, pkg.BATCHED_DF64), ref, "skewed_100k df64")
    assert_lowp(pricer.price(opts, y, pkg.BATCHED_MIXED), ref, "skewed_100k mixed")


def test_put_call_parity(pkg, pricer):
    """The calibrated tree reprices discount bonds exactly, so for every option
    call - put = 100 P(0, n dt) - X P(0, m dt) with the tree's own discount factors
    (size-independent property, checked on the full skewed batch)."""
    b = pkg.workloads.skewed_batch()
    opts = pkg.Options.from_batch(b)
    y = _curve(pkg)
    calls = opts.subset(np.arange(opts.N))
    calls.Types[:] = 0
    puts = opts.subset(np.arange(opts.N))
    puts.Types[:] = 1
    c = pricer.price(calls, y, pkg.BATCHED_FP64)
    p = pricer.price(puts, y, pkg.BATCHED_FP64)
    s = pkg.shape(opts)
    dt = 1.0 / opts.TermStepCounts
    rates, days = y.Prices, y.TimeSteps

    def disc(k):
        t = k * dt
        r = pkg.workloads._curve_rate(t, rates, days)
        return np.exp(-r * t)

    n, m = s["height"], s["maturity_step"]
    live = (m >= 0) & (m < n)
    lhs = (c - p)[live]
    rhs = (100.0 * disc(n) - opts.StrikePrices * disc(m))[live]
    assert np.max(np.abs(lhs - rhs)) <= 1e-9 * 100


def test_permutation_invariance_and_determinism(pkg, pricer, uneven):
    opts, y, _ = uneven
    a = pricer.price(opts, y, pkg.BATCHED_FP64)
    b = pricer.price(opts, y, pkg.BATCHED_FP64)
    assert np.array_equal(a, b)  # same inputs, same bits
    perm = np.random.default_rng(3).permutation(opts.N)
    c = pricer.price(opts.subset(perm), y, pkg.BATCHED_FP64)
    assert np.array_equal(c, a[perm])  # a tree's arithmetic does not depend on its neighbours


def test_device_entry_point_and_graph_equal_host(pkg, pricer, uneven):
    import torch
    opts, y, _ = uneven
    host = pricer.price(opts, y, pkg.BATCHED_MIXED)
    direct = pricer.price(opts, y, pkg.BATCHED_MIXED, use_graph=False)
    assert np.array_equal(host, direct)
    assert pricer.last_stats.graph_replayed == 0
    pricer.price(opts, y, pkg.BATCHED_MIXED)
    assert pricer.last_stats.graph_replayed == 1
    fields = {"strike": opts.StrikePrices, "bond_maturity": opts.Maturities, "option_maturity": opts.Lengths,
              "term_unit": opts.TermUnits.view(np.int16), "term_steps": opts.TermStepCounts.view(np.int16),
              "a": opts.ReversionRates, "sigma": opts.Volatilities, "type": opts.Types}
    dev = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in fields.items()}
    out = torch.empty(opts.N, dtype=torch.float64, device="cuda")
    st = pricer.price_device({k: t.data_ptr() for k, t in dev.items()}, opts.N, y, out.data_ptr(), pkg.BATCHED_MIXED)
    assert st.h2d_bytes == 0 and st.d2h_bytes == 0
    assert np.array_equal(out.cpu().numpy(), host)


@pytest.mark.parametrize("mode", ["BATCHED_MIXED", "BATCHED_FP64", "PLAIN_FP64"])
def test_pinned_host_arrays_equal_pageable(pkg, pricer, uneven, mode):
    """Pinned (page-locked) host arrays: on a host the GPU reaches coherently the
    sizing kernel reads them in place, elsewhere they are copied; the prices are
    bitwise those of pageable arrays, and an invalid record in pinned memory is
    still rejected with a NaN price."""
    import torch
    opts, y, _ = uneven
    n = 4000 if mode == "PLAIN_FP64" else opts.N
    sub = pkg.Options.from_batch({k: v[:n] for k, v in pkg.workloads.uneven_batch().items()})
    m = getattr(pkg, mode)
    ref = pricer.price(sub, y, m)
    fields = {"strike": sub.StrikePrices, "bond_maturity": sub.Maturities, "option_maturity": sub.Lengths,
              "term_unit": sub.TermUnits.view(np.int16), "term_steps": sub.TermStepCounts.view(np.int16),
              "a": sub.ReversionRates, "sigma": sub.Volatilities, "type": sub.Types}
    pin = {k: torch.from_numpy(np.ascontiguousarray(v)).pin_memory() for k, v in fields.items()}
    out = torch.full((n,), -1.0, dtype=torch.float64).pin_memory()
    st = pricer.price_host_ptrs({k: t.data_ptr() for k, t in pin.items()}, n, y, out.data_ptr(), m)
    assert np.array_equal(out.numpy(), ref)
    assert st.h2d_bytes == 45 * n and st.d2h_bytes == 8 * n
    pin["a"][7] = -1.0  # mean reversion must be > 0
    with pytest.raises(pkg.InvalidInput):
        pricer.price_host_ptrs({k: t.data_ptr() for k, t in pin.items()}, n, y, out.data_ptr(), m)
    got = out.numpy()
    assert np.isnan(got[7]) and np.array_equal(np.delete(got, 7), np.delete(ref, 7))


def test_block_sizes_agree(pkg, pricer, uneven):
    """Group size changes which trees share a warp or a block, not the answer."""
    opts, y, ref = uneven
    for bs in (64, 128, 256, 512):
        for big in (128, 256):
            got = pricer.price(opts, y, pkg.BATCHED_FP64, block_size=bs, big_threshold=big)
            assert_fp64(got, ref, f"bs {bs} big {big}")


def test_invalid_records_are_rejected(pkg, pricer):
    opts, y, g64, _ = load_set(pkg, "book")
    bad = opts.subset(np.arange(opts.N))
    bad.ReversionRates[1] = 0.0
    bad.Types[3] = 5
    out = np.zeros(bad.N)
    with pytest.raises(pkg.InvalidInput) as e:
        pricer.price(bad, y, pkg.BATCHED_FP64, out=out)
    assert "index 1" in str(e.value)
    assert np.isnan(out[1]) and np.isnan(out[3])
    ok = [0, 2, 4]
    assert np.max(np.abs(out[ok] - g64[ok])) <= 1e-10 * np.max(g64) + 1e-12
    # the context stays usable after the error
    assert_fp64(pricer.price(opts, y, pkg.BATCHED_FP64), g64, "after error")


def test_empty_batch_and_too_wide_tree(pkg, pricer):
    opts, y, _, _ = load_set(pkg, "book")
    empty = opts.subset(np.arange(0))
    assert pricer.price(empty, y, pkg.BATCHED_FP64).shape == (0,)
    wide = opts.subset(np.arange(1))
    wide.ReversionRates[0] = 0.0005  # jmax ~ 1e5 at 365 steps per year
    wide.TermStepCounts[0] = 365
    wide.Maturities[0] = 30.0
    with pytest.raises(pkg.InvalidInput):
        pricer.price(wide, y, pkg.BATCHED_FP64)


def test_plain_mode_matches_batched(pkg, pricer):
    opts, y, g64, _ = load_set(pkg, "edge")
    assert_fp64(pricer.price(opts, y, pkg.PLAIN_FP64), g64, "edge plain")


def test_autotune_and_cache(pkg, tmp_path):
    cache = str(tmp_path / "tune.txt")
    opts, y, g64, _ = load_set(pkg, "uneven_2k")
    with pkg.Pricer(0, cache) as p:
        best = p.autotune(opts, y, pkg.BATCHED_MIXED, repeats=1)
        assert best.block_size in (64, 128, 256, 512)
        assert_lowp(p.price(opts, y, pkg.BATCHED_MIXED), g64, "tuned")
    with open(cache) as f:
        assert "|3 " in f.read()
    with pkg.Pricer(0, cache) as p2:
        assert p2.get_config(pkg.BATCHED_MIXED).block_size == best.block_size


def test_measured_peaks_positive(pricer):
    fp64, fp32 = pricer.measure_peaks()
    assert 0.1 < fp64 < fp32


def test_cli_price_and_compare(pkg):
    """The reference's compare.sh loop: { price -o X.in -y yield.in; cat X.out; } | Compare."""
    d = os.path.join(GOLDEN, "reference")
    for mode, extra in (("1", []), ("3", ["--abs", "1e-4"])):
        out = subprocess.run([os.path.join(TOOLS, "hwt-price"), "-o", os.path.join(d, "1_RAND_1000.in"), "-y",
                              os.path.join(d, "yield.in"), "-v", mode], capture_output=True, text=True, check=True)
        with open(os.path.join(d, "1_RAND_1000.out64")) as f:
            gold = f.read()
        r = subprocess.run([os.path.join(TOOLS, "hwt-compare")] + extra, input=out.stdout + gold,
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stdout
    runs = subprocess.run([os.path.join(TOOLS, "hwt-price"), "-o", os.path.join(d, "book.in"), "-y",
                           os.path.join(d, "yield.in"), "-v", "1", "3", "-b", "64", "128", "-r", "2"],
                          capture_output=True, text=True, check=True)
    lines = [l for l in runs.stdout.splitlines() if l.strip()]
    assert len(lines) == 4 and all(len(l.split(",")) == 6 for l in lines)


def test_cpp_adapter_kernel_run(pkg, tmp_path):
    """include/hwtree.hpp: the reference's records and KernelRun::run shape."""
    src = tmp_path / "k.cpp"
    d = os.path.join(GOLDEN, "reference")
    src.write_text(f'''#include "hwtree.hpp"
int main() {{
  hwtree::Options o("{os.path.join(d, 'book.in')}");
  hwtree::Yield y("{os.path.join(d, 'yield.in')}");
  std::vector<double> r;
  hwtree::KernelRun run(HWT_BATCHED_FP64);
  run.run(o, y, r, 128, hwtree::SortType::HEIGHT_DESC, false);
  hwtree::computeOptions(o, y, r, HWT_PLAIN_FP64);
  hwtree::Arrays::write_array(std::cout, r);
  return 0;
}}
''')
    exe = tmp_path / "k"
    subprocess.run(["g++", "-std=c++17", "-O1", "-I" + os.path.join(ROOT, "include"), str(src), "-o", str(exe),
                    "-L" + TOOLS, "-lhwtree", "-Wl,-rpath," + TOOLS], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    got = np.array(pkg.read_arrays(out)[0], dtype=np.float64)
    with open(os.path.join(d, "book.out64")) as f:
        gold = np.array(pkg.read_arrays(f.read())[0], dtype=np.float64)
    assert np.max(np.abs(got - gold)) <= 1e-10 * np.max(gold) + 1e-12


def test_sort_orders_give_the_same_bits(pkg, pricer, uneven):
    """-s changes the schedule (which trees share a warp task, in which order),
    never a tree's arithmetic."""
    opts, y, _ = uneven
    for mode in (pkg.BATCHED_FP64, pkg.BATCHED_MIXED):
        base = pricer.price(opts, y, mode)
        for s in "WwHhi-":
            assert np.array_equal(pricer.price(opts, y, mode, sort=s), base), (mode, s)
    with pytest.raises(pkg.InvalidInput):
        pricer.price(opts, y, pkg.BATCHED_FP64, sort="x")


def test_warp_k_sets(pkg, pricer, uneven):
    """Restricting or widening the nodes-per-lane set moves trees between warp
    classes and tiers (K = 1 alone sends every tree wider than 32 nodes to the
    warp-group tier); prices stay within the mode's bound."""
    opts, y, ref = uneven
    for mask in (0xFF, 0xAF, 0x01, 0x10 | 0x40):
        assert_fp64(pricer.price(opts, y, pkg.BATCHED_FP64, warp_k_mask=mask), ref, f"fp64 mask {mask:#x}")
    for mask in (0xFF, 0x01):
        assert_fp64(pricer.price(opts, y, pkg.BATCHED_DF64, warp_k_mask=mask), ref, f"df64 mask {mask:#x}")
    for mask in (0x3AF, 0x3FF, 0x01, 0x200, 0x400, 0x7FF):
        assert_lowp(pricer.price(opts, y, pkg.BATCHED_MIXED, warp_k_mask=mask), ref, f"mixed mask {mask:#x}")
    # K = 32 alone at a 512-node threshold: every warp task takes 32 nodes per lane,
    # and the launch must carry their shared-memory coefficients
    for mode in (pkg.BATCHED_FP32, pkg.BATCHED_MIXED):
        assert_lowp(pricer.price(opts, y, mode, warp_k_mask=0x400, big_threshold=512), ref, f"{mode} K=32 only")


@pytest.mark.parametrize("mode", ["BATCHED_MIXED", "BATCHED_FP32"])
def test_wide_warp_tasks(pkg, pricer, uneven, mode):
    """Float rows: trees of 513..1,024 nodes as single-warp tasks of 32 nodes per lane
    (their coefficients in shared memory) instead of warp groups: no group-tier trees
    are left in the uneven batch, and the prices stay within 1e-4 of the oracle and
    within float rounding of the warp-group path."""
    opts, y, ref = uneven
    m = getattr(pkg, mode)
    wide = pricer.price(opts, y, m, big_threshold=1024)
    assert pricer.last_stats.n_block_trees == 0
    assert_lowp(wide, ref, f"{mode} K=32")
    groups = pricer.price(opts, y, m, big_threshold=512)
    assert pricer.last_stats.n_block_trees > 0
    assert np.max(np.abs(wide - groups)) < 5e-5
    # 32 nodes per lane only: every tree up to 1,024 nodes, however narrow, on 32-node lanes
    only = pricer.price(opts, y, m, big_threshold=1024, warp_k_mask=0x400)
    assert_lowp(only, ref, f"{mode} K=32 only")
