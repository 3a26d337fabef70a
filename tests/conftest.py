import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")
REF_SETS = ["book", "options-1000", "0_UNIFORM_1000", "1_RAND_1000", "2_RANDCONSTHEIGHT_1000",
            "3_RANDCONSTWIDTH_1000"] + [f"{n}_every64" for n in (
                "0_UNIFORM", "1_RAND", "2_RANDCONSTHEIGHT", "3_RANDCONSTWIDTH", "4_SKEWED",
                "5_SKEWEDCONSTHEIGHT", "6_SKEWEDCONSTWIDTH")]
SYN_SETS = ["uniform_1k", "uneven_2k", "skewed_512", "book_100", "edge"]

# Parity bars (the required tolerances, written here once):
#   FP64 paths: |p - p_ref| <= 1e-10 * |p_ref| + 1e-12   (relative 1e-10; the
#               absolute floor covers prices that are zero up to rounding)
#   FP32 / mixed paths: |p - p_ref| <= 1e-4 (absolute, per 100 face)
FP64_REL, FP64_ABS = 1e-10, 1e-12
LOWP_ABS = 1e-4


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu on a GB300)")


@pytest.fixture(scope="session")
def pkg():
    import __graft_entry__ as g
    return g.package()


@pytest.fixture(scope="session")
def orc():
    import __graft_entry__ as g
    o = g.oracle()
    o.build()
    return o


@pytest.fixture(scope="session")
def pricer(pkg):
    p = pkg.Pricer(0)
    yield p
    p.close()


def load_set(pkg, name):
    """(Options, Yield, gold64, gold32-as-text-tokens) of a golden fixture."""
    if name in SYN_SETS:
        d = os.path.join(GOLDEN, "synthetic")
        opts = pkg.Options.from_file(os.path.join(d, f"{name}.in"))
        y = pkg.Yield.from_file(os.path.join(d, "curve11.in"))
    else:
        d = os.path.join(GOLDEN, "reference")
        opts = pkg.Options.from_file(os.path.join(d, f"{name}.in"))
        y = pkg.Yield.from_file(os.path.join(d, "yield.in"))
    with open(os.path.join(d, f"{name}.out64")) as f:
        g64 = np.array(pkg.read_arrays(f.read())[0], dtype=np.float64)
    with open(os.path.join(d, f"{name}.out32")) as f:
        g32 = pkg.read_arrays(f.read())[0]
    return opts, y, g64, g32


def assert_fp64(got, ref, what=""):
    err = np.abs(got - ref)
    bound = FP64_REL * np.abs(ref) + FP64_ABS
    bad = np.where(~(err <= bound))[0]
    assert bad.size == 0, (f"{what}: {bad.size} prices off; first index {bad[0]}: {got[bad[0]]!r} vs {ref[bad[0]]!r} "
                           f"(max abs err {np.nanmax(err):.3e})")


def assert_lowp(got, ref, what=""):
    err = np.abs(got - ref)
    bad = np.where(~(err <= LOWP_ABS))[0]
    assert bad.size == 0, (f"{what}: {bad.size} prices off by more than 1e-4; first index {bad[0]}: "
                           f"{got[bad[0]]!r} vs {ref[bad[0]]!r} (max abs err {np.nanmax(err):.3e})")
