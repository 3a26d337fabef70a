"""The oracle (oracle/hwt_seq.c) pinned against the reference's own golden
vectors and against the reference's seq/ built from its sources."""
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, REF_SETS, SYN_SETS, load_set

DBL_MARGIN = 1000 * np.finfo(np.float64).eps
FLT_MARGIN = 1000 * np.finfo(np.float32).eps


@pytest.mark.parametrize("name", REF_SETS + SYN_SETS)
def test_oracle_f64_matches_fp64_goldens(pkg, orc, name):
    opts, y, g64, _ = load_set(pkg, name)
    got = orc.price(opts, y, "f64")
    # data/out/*.out came from the reference's double build on another machine:
    # libm differences in exp/log leave ~1e-14; the reference's own margin is 1000 eps.
    assert np.max(np.abs(got - g64)) <= DBL_MARGIN


@pytest.mark.parametrize("name", SYN_SETS)
def test_oracle_f64_text_identical_to_reference_build(pkg, orc, name):
    """Synthetic goldens were written by the reference's seq/ compiled here: the
    restatement reproduces its printed digits."""
    opts, y, _, _ = load_set(pkg, name)
    with open(os.path.join(GOLDEN, "synthetic", f"{name}.out64")) as f:
        gold = pkg.read_arrays(f.read())[0]
    mine = pkg.format_array(orc.price(opts, y, "f64"), 17)[1:-2].split(", ")
    same = np.mean([a == b for a, b in zip(mine, gold)])
    assert same >= 0.97, same


@pytest.mark.parametrize("name", REF_SETS + SYN_SETS)
def test_oracle_f32_matches_fp32_goldens(pkg, orc, name):
    """The float build's goldens (data/out32) are reproduced digit for digit."""
    opts, y, _, g32 = load_set(pkg, name)
    mine = pkg.format_array(orc.price(opts, y, "f32"), 9)[1:-2].split(", ")
    exact = np.mean([a == b for a, b in zip(mine, g32)])
    assert exact >= 0.99, exact
    err = np.abs(np.array(mine, dtype=np.float64) - np.array(g32, dtype=np.float64))
    assert np.max(err) <= FLT_MARGIN


def test_oracle_equals_live_reference_build(pkg, orc, tmp_path):
    """A fresh seeded batch priced by the reference's seq/ built from its sources
    (oracle/_ref, present only where the reference is mounted)."""
    exe = orc.reference_binary("f64")
    if exe is None:
        pytest.skip("reference seq/ not built here")
    wl = pkg.workloads
    b = {k: v[::97] for k, v in wl.uneven_batch(30000, seed=11).items()}
    opts = pkg.Options.from_batch(b)
    opts.write_to_file(str(tmp_path / "o.in"))
    rates, days = wl.yield_curve()
    with open(tmp_path / "y.in", "w") as f:
        pkg.write_array(f, rates, 17)
        pkg.write_array(f, days, 0)
    out = subprocess.run([exe, "-o", str(tmp_path / "o.in"), "-y", str(tmp_path / "y.in")], capture_output=True,
                         text=True, check=True).stdout
    ref = np.array(pkg.read_arrays(out)[0], dtype=np.float64)
    mine = orc.price(pkg.Options.from_file(str(tmp_path / "o.in")), pkg.Yield.from_file(str(tmp_path / "y.in")), "f64")
    assert np.max(np.abs(mine - ref)) <= 1e-15 * max(1.0, np.max(np.abs(ref)))


def test_oracle_shape_matches_product_host_shape(pkg, orc):
    """Tree sizing: the product's host-side hwt_shape and the oracle agree
    (jmax, height, width, maturity step), including the maturity truncation traps."""
    for name in REF_SETS + SYN_SETS:
        opts, _, _, _ = load_set(pkg, name)
        a = pkg.shape(opts)
        b = orc.shape(opts, "f64")
        ok = b["height"] >= 0
        for k in ("jmax", "height", "width", "maturity_step"):
            assert np.array_equal(a[k][ok], b[k][ok]), (name, k)


def test_maturity_truncation_trap_present(pkg):
    """Steps 75 per year put t/dt just below the integer: (int)(3/(1/75)) = 224."""
    opts, _, _, _ = load_set(pkg, "edge")
    s = pkg.shape(opts)
    idx = np.where((opts.TermStepCounts == 75) & (opts.Lengths == 3.0))[0]
    assert idx.size and np.all(s["maturity_step"][idx] == 224)


def test_planted_mistake_is_caught(pkg, orc):
    """A wrong oracle answer (one option perturbed by 1e-9 relative) fails the
    FP64 parity bar the GPU tests use."""
    from conftest import FP64_ABS, FP64_REL
    opts, y, g64, _ = load_set(pkg, "uniform_1k")
    got = orc.price(opts, y, "f64")
    got[17] *= 1 + 1e-9
    err = np.abs(got - g64)
    assert np.sum(err > FP64_REL * np.abs(g64) + FP64_ABS) == 1
