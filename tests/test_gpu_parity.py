"""GPU parity: every pricing mode against the reference's golden vectors and
against the oracle (C restatement of the reference's seq/), through the C ABI."""
import numpy as np
import pytest

from conftest import REF_SETS, SYN_SETS, assert_fp64, assert_lowp, load_set

pytestmark = pytest.mark.gpu

ALL_SETS = REF_SETS + SYN_SETS


@pytest.mark.parametrize("name", ALL_SETS)
@pytest.mark.parametrize("mode", ["BATCHED_FP64", "BATCHED_DF64", "PLAIN_FP64"])
def test_fp64_matches_reference_goldens(pkg, pricer, name, mode):
    opts, y, g64, _ = load_set(pkg, name)
    got = pricer.price(opts, y, getattr(pkg, mode))
    assert_fp64(got, g64, f"{name} {mode}")


@pytest.mark.parametrize("name", ALL_SETS)
@pytest.mark.parametrize("mode", ["BATCHED_FP64", "BATCHED_DF64"])
def test_fp64_matches_oracle(pkg, orc, pricer, name, mode):
    """Double rows, and double-float rows on the FP32 pipes, within 1e-10 relative."""
    opts, y, _, _ = load_set(pkg, name)
    ref = orc.price(opts, y, "f64")
    got = pricer.price(opts, y, getattr(pkg, mode))
    assert_fp64(got, ref, f"{name} {mode}")


@pytest.mark.parametrize("name", ALL_SETS)
def test_fp64_passes_reference_compare_margin(pkg, pricer, name):
    """The reference's Compare criterion (test/Compare.hpp:8-24 with Catch's
    Approx): |t-g| <= 1000*DBL_EPSILON or |t-g| <= 100*FLT_EPSILON*|g|."""
    opts, y, g64, _ = load_set(pkg, name)
    got = pricer.price(opts, y, pkg.BATCHED_FP64)
    d = np.abs(got - g64)
    ok = (d <= 1000 * np.finfo(np.float64).eps) | (d <= 100 * np.finfo(np.float32).eps * np.abs(g64))
    assert ok.all()


@pytest.mark.parametrize("name", ALL_SETS)
@pytest.mark.parametrize("mode", ["BATCHED_MIXED", "BATCHED_FP32"])
def test_low_precision_within_1e4(pkg, pricer, name, mode):
    opts, y, g64, _ = load_set(pkg, name)
    got = pricer.price(opts, y, getattr(pkg, mode))
    assert_lowp(got, g64, f"{name} {mode}")
