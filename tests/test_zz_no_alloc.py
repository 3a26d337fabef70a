"""hwt_price_device_noalloc: the allocation-free entry point, for callers that
cannot call cudaMalloc (their device memory belongs to another allocator, or the
pricing path may not run cudaMalloc/cudaFree, which can synchronise the device).
Its scratch is a static device array of the library, so its prices must equal
those of hwt_price_device - the entry point that allocates its scratch - on the
same device inputs, call after call.  Collected last so that a failure here
leaves the rest of the suite already run; passes alone and after the others."""
import ctypes

import numpy as np
import pytest

from conftest import FP64_ABS, FP64_REL, LOWP_ABS, load_set

pytestmark = pytest.mark.gpu

FIELDS = ("strike", "bond_maturity", "option_maturity", "term_unit", "term_steps", "a", "sigma", "type")


def _device_inputs(pkg, opts):
    import torch
    host = {"strike": opts.StrikePrices, "bond_maturity": opts.Maturities, "option_maturity": opts.Lengths,
            "term_unit": opts.TermUnits.view(np.int16), "term_steps": opts.TermStepCounts.view(np.int16),
            "a": opts.ReversionRates, "sigma": opts.Volatilities, "type": opts.Types}
    return {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in host.items()}


def _c_options(pkg, dev, n):
    return pkg._Options(n, *(dev[k].data_ptr() for k in FIELDS))


@pytest.mark.parametrize("mode_name", ["BATCHED_FP64", "BATCHED_FP32", "BATCHED_MIXED"])
def test_noalloc_matches_allocating_entry_point(pkg, mode_name):
    import torch
    mode = getattr(pkg, mode_name)
    opts_a, y, _, _ = load_set(pkg, "uneven_2k")
    opts_b, _, _, _ = load_set(pkg, "skewed_512")
    opts = pkg.Options(*(np.concatenate([getattr(opts_a, f), getattr(opts_b, f)]) for f in (
        "StrikePrices", "Maturities", "Lengths", "TermUnits", "TermStepCounts", "ReversionRates", "Volatilities",
        "Types")))
    n = opts.N
    dev = _device_inputs(pkg, opts)
    rate = torch.from_numpy(y.Prices).cuda()
    day = torch.from_numpy(y.TimeSteps).cuda()
    with pkg.Pricer(0) as p:
        ref = torch.empty(n, dtype=torch.float64, device="cuda")
        p.price_device({k: dev[k].data_ptr() for k in FIELDS}, n, y, ref.data_ptr(), mode, block_size=128,
                       big_threshold=256)
        ref = ref.cpu().numpy()
    c_opts = _c_options(pkg, dev, n)
    c_yield = pkg._Yield(y.N, rate.data_ptr(), day.data_ptr())
    for call in range(2):
        out = torch.full((n,), float("nan"), dtype=torch.float64, device="cuda")
        rc = pkg.lib().hwt_price_device_noalloc(ctypes.byref(c_opts), ctypes.byref(c_yield), mode, out.data_ptr(),
                                                None)
        assert rc == pkg.HWT_OK, (call, rc)
        got = out.cpu().numpy()
        err = np.abs(got - ref)
        if mode == pkg.BATCHED_FP64:
            assert np.all(err <= FP64_REL * np.abs(ref) + FP64_ABS), (call, np.max(err))
        else:
            assert np.all(err <= LOWP_ABS), (call, np.max(err))


def test_noalloc_rejects_oversized_batch(pkg):
    import torch
    opts, y, _, _ = load_set(pkg, "book")
    n = 32769
    big = pkg.Options(*(np.resize(getattr(opts, f), n) for f in (
        "StrikePrices", "Maturities", "Lengths", "TermUnits", "TermStepCounts", "ReversionRates", "Volatilities",
        "Types")))
    dev = _device_inputs(pkg, big)
    rate = torch.from_numpy(y.Prices).cuda()
    day = torch.from_numpy(y.TimeSteps).cuda()
    out = torch.empty(n, dtype=torch.float64, device="cuda")
    c_yield = pkg._Yield(y.N, rate.data_ptr(), day.data_ptr())
    rc = pkg.lib().hwt_price_device_noalloc(ctypes.byref(_c_options(pkg, dev, n)), ctypes.byref(c_yield),
                                            pkg.BATCHED_FP64, out.data_ptr(), None)
    assert rc == pkg.HWT_EINVAL
    # the largest accepted batch still prices
    rc = pkg.lib().hwt_price_device_noalloc(ctypes.byref(_c_options(pkg, dev, 32768)), ctypes.byref(c_yield),
                                            pkg.BATCHED_FP64, out.data_ptr(), None)
    assert rc == pkg.HWT_OK
    assert np.all(np.isfinite(out[:32768].cpu().numpy()))


def test_noalloc_rejects_non_finite_curve(pkg):
    """A curve rate that is not finite makes every price suspect: HWT_EINVAL."""
    import torch
    opts, y, _, _ = load_set(pkg, "book")
    dev = _device_inputs(pkg, opts)
    rates = y.Prices.copy()
    rates[len(rates) // 2] = np.nan
    rate = torch.from_numpy(rates).cuda()
    day = torch.from_numpy(y.TimeSteps).cuda()
    out = torch.empty(opts.N, dtype=torch.float64, device="cuda")
    c_yield = pkg._Yield(y.N, rate.data_ptr(), day.data_ptr())
    rc = pkg.lib().hwt_price_device_noalloc(ctypes.byref(_c_options(pkg, dev, opts.N)), ctypes.byref(c_yield),
                                            pkg.BATCHED_MIXED, out.data_ptr(), None)
    assert rc == pkg.HWT_EINVAL
