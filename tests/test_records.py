"""Records and the .in / [..] text format (common/Options.hpp, Yield.hpp, Arrays.hpp),
the hwt-compare harness and the C++ adapter header."""
import io
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT, REF_SETS, SYN_SETS, load_set

TOOLS = os.path.join(ROOT, "diku.optionspricing_gb300", "_build")


@pytest.mark.parametrize("name", REF_SETS + SYN_SETS)
def test_price_arrays_reformat_byte_identical(pkg, name):
    """Golden outputs were written by the reference's write_array (std::fixed,
    max_digits10): parsing and re-writing reproduces them byte for byte."""
    d = "synthetic" if name in SYN_SETS else "reference"
    for ext, digits in (("out64", 17), ("out32", 9)):
        with open(os.path.join(GOLDEN, d, f"{name}.{ext}")) as f:
            text = f.read()
        vals = np.array(pkg.read_arrays(text)[0], dtype=np.float64 if digits == 17 else np.float32)
        assert pkg.format_array(vals, digits) == text


def test_options_roundtrip(pkg, tmp_path):
    opts, _, _, _ = load_set(pkg, "edge")
    opts.write_to_file(str(tmp_path / "e.in"))
    back = pkg.Options.from_file(str(tmp_path / "e.in"))
    for f in ("StrikePrices", "Maturities", "Lengths", "TermUnits", "TermStepCounts", "ReversionRates",
              "Volatilities", "Types"):
        assert np.array_equal(getattr(opts, f), getattr(back, f)), f


def test_read_array_stream(pkg):
    s = io.StringIO("[1, 2.5, 3]\n[4]\n")
    assert pkg.read_array(s) == ["1", "2.5", "3"]
    assert pkg.read_array(s) == ["4"]


def test_bad_records(pkg, tmp_path):
    with pytest.raises(ValueError):
        pkg.Options.from_file(str(tmp_path / "missing.in"))
    with pytest.raises(ValueError):
        pkg.Options.from_file("")
    p = tmp_path / "badtype.in"
    p.write_text("[1]\n[2]\n[1]\n[365]\n[12]\n[0.1]\n[0.01]\n[7]\n")
    with pytest.raises(IndexError):  # the reference throws out_of_range
        pkg.Options.from_file(str(p))


def _compare(args, stdin):
    return subprocess.run([os.path.join(TOOLS, "hwt-compare")] + args, input=stdin, capture_output=True, text=True)


def test_compare_harness_semantics(pkg):
    """hwt-compare accepts |t-g| <= 1000 eps or <= 100 FLT_EPSILON |g| (Catch Approx in
    test/Compare.hpp) and rejects anything else; --fp32 uses the float margin."""
    ok = _compare([], "[1.0, 100.0, 0.0]\n[1.0, 100.0001, 1e-13]\n")
    assert ok.returncode == 0, ok.stdout
    bad = _compare([], "[1.0]\n[1.001]\n")
    assert bad.returncode == 1 and "FAILED" in bad.stdout
    f32 = _compare(["--fp32"], "[0.00001]\n[0.0001]\n")
    assert f32.returncode == 0
    size = _compare([], "[1.0, 2.0]\n[1.0]\n")
    assert size.returncode == 1


def test_compare_harness_on_golden_pair():
    with open(os.path.join(GOLDEN, "reference", "1_RAND_1000.out64")) as f:
        gold = f.read()
    r = _compare([], gold + gold)
    assert r.returncode == 0 and "All tests passed" in r.stdout


def test_cpp_adapter_compiles(tmp_path):
    src = tmp_path / "t.cpp"
    src.write_text('#include "hwtree.hpp"\nint main(){ hwtree::Options o(0); hwtree::Yield y; (void)o; (void)y; return 0; }\n')
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-I" + os.path.join(ROOT, "include"), str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
