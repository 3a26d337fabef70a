"""The library's file readers (hwt_read_options / hwt_read_yield / binary cache)
against the Python restatement of the reference's reader (common/Arrays.hpp:15-32)."""
import glob
import os
import subprocess
import time

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

FIELDS = ("StrikePrices", "Maturities", "Lengths", "TermUnits", "TermStepCounts", "ReversionRates", "Volatilities",
          "Types")


def _same(a, b):
    for f in FIELDS:
        x, y = getattr(a, f), getattr(b, f)
        assert x.dtype == y.dtype and np.array_equal(x.view(np.uint8), y.view(np.uint8)), f


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "*", "*.in"))))
def test_reader_matches_python_parser(pkg, path):
    with open(path) as f:
        text = f.read()
    if text.count("[") >= 8:
        _same(pkg.Options.from_file(path), pkg.Options.from_text(text))
    else:  # a yield curve
        y = pkg.Yield.from_file(path)
        arrs = pkg.read_arrays(text)
        assert np.array_equal(y.Prices, np.array(arrs[0], dtype=np.float64))
        assert np.array_equal(y.TimeSteps, np.array([int(t) for t in arrs[1]], dtype=np.int32))


def test_large_file_threaded_and_binary_round_trip(pkg, tmp_path):
    """300,000 options (bodies of several MB, parsed by many threads) read as the
    Python parser reads them; the binary cache gives back the exact doubles (the
    reference's fixed 17-fractional-digit text does not, for values below 1)."""
    b = pkg.workloads.uneven_batch(300_000, seed=9)
    o = pkg.Options.from_batch(b)
    t = tmp_path / "big.in"
    text = o.to_text()
    t.write_text(text)
    got = pkg.Options.from_file(str(t))
    _same(got, pkg.Options.from_text(text))
    assert np.array_equal(got.StrikePrices, o.StrikePrices)  # values above 1 keep 17+ digits
    bpath = tmp_path / "big.bin"
    o.to_bin(str(bpath))
    _same(pkg.Options.from_file(str(bpath)), o)
    assert os.path.getsize(bpath) == 32 + 300_000 * (5 * 8) + 2 * 300_000 * 2 + 300_000


def test_reader_errors(pkg, tmp_path):
    ok = "[1.0, 2.0]\n[9, 9]\n[3, 3]\n[365, 365]\n[12, 12]\n[0.1, 0.1]\n[0.01, 0.01]\n[0, 1]\n"

    def write(text):
        p = tmp_path / "x.in"
        p.write_text(text)
        return str(p)

    assert pkg.Options.from_file(write(ok)).N == 2
    with pytest.raises(ValueError, match="arrays, expected 8"):
        pkg.Options.from_file(write("[1.0]\n[2.0]\n"))
    with pytest.raises(ValueError, match="different length"):
        pkg.Options.from_file(write(ok.replace("[9, 9]", "[9]")))
    with pytest.raises(ValueError, match="bad value in StrikePrices"):
        pkg.Options.from_file(write(ok.replace("[1.0, 2.0]", "[1.0, abc]")))
    with pytest.raises(ValueError, match="bad value in TermUnits"):
        pkg.Options.from_file(write(ok.replace("[365, 365]", "[365, 70000]")))
    with pytest.raises(ValueError, match="bad value in TermStepCounts"):
        pkg.Options.from_file(write(ok.replace("[12, 12]", "[12, 12.5]")))
    with pytest.raises(IndexError):  # the reference throws out_of_range for a bad type
        pkg.Options.from_file(write(ok.replace("[0, 1]", "[0, 2]")))
    with pytest.raises(ValueError, match="does not exist"):
        pkg.Options.from_file(str(tmp_path / "missing.in"))
    bad = tmp_path / "t.bin"
    pkg.Options.from_file(write(ok)).to_bin(str(bad))
    data = bad.read_bytes()
    bad.write_bytes(data[:-8])
    with pytest.raises(ValueError, match="size does not match"):
        pkg.Options.from_file(str(bad))
    y = tmp_path / "y.in"
    y.write_text("[0.01, 0.02]\n[91, 183.5]\n")
    with pytest.raises(ValueError, match="whole days"):
        pkg.Yield.from_file(str(y))


def test_cli_reads_binary_cache(pkg, tmp_path):
    """hwt-price -w writes the binary cache; the cache and the text give the same
    records to the reader."""
    src = os.path.join(GOLDEN, "reference", "book.in")
    exe = os.path.join(ROOT, "diku.optionspricing_gb300", "_build", "hwt-price")
    out = tmp_path / "book.bin"
    subprocess.run([exe, "-o", src, "-w", str(out)], check=True, capture_output=True)
    _same(pkg.Options.from_file(str(out)), pkg.Options.from_file(src))


def test_reader_is_faster_than_python(pkg, tmp_path):
    b = pkg.workloads.uneven_batch(100_000, seed=4)
    o = pkg.Options.from_batch(b)
    p = tmp_path / "m.in"
    text = o.to_text()
    p.write_text(text)
    t0 = time.perf_counter()
    pkg.Options.from_file(str(p))
    t_c = time.perf_counter() - t0
    t0 = time.perf_counter()
    pkg.Options.from_text(text)
    t_py = time.perf_counter() - t0
    assert t_c < t_py
