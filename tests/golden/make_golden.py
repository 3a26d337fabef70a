"""Generates the committed golden fixtures of tests/golden/.

Run where the reference sources are mounted and its seq/ pricer has been built
from them (``make -C oracle ref``):  ``python tests/golden/make_golden.py``

reference/  copies of the reference's own test vectors (data/*.in, the FP64
            goldens data/out/*.out written by its seq/ double build and the FP32
            goldens data/out32/*.out); the 65,536-option sets are thinned to
            every 64th option, with the matching golden entries.
synthetic/  seeded batches (workloads.py) and edge cases - parity traps of the
            maturity step, jmax 1 and 2 trees, maturity at/after bond maturity,
            zero height, short term units, trees that never reach +-jmax, block
            trees of every width class - priced by the reference's seq/ compiled
            from its sources (oracle/_ref/Seq64 and Seq32), outputs kept verbatim.
"""
from __future__ import annotations

import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("HWT_REFERENCE", "/root/reference")
sys.path.insert(0, ROOT)

import __graft_entry__ as g  # noqa: E402

pkg = g.package()
wl = pkg.workloads

SMALL_SETS = ["book", "options-1000", "0_UNIFORM_1000", "1_RAND_1000", "2_RANDCONSTHEIGHT_1000",
              "3_RANDCONSTWIDTH_1000"]
BIG_SETS = ["0_UNIFORM", "1_RAND", "2_RANDCONSTHEIGHT", "3_RANDCONSTWIDTH", "4_SKEWED", "5_SKEWEDCONSTHEIGHT",
            "6_SKEWEDCONSTWIDTH"]
THIN = 64


def _read(path):
    with open(path) as f:
        return pkg.read_arrays(f.read())


def _write_tokens(path, arrays):
    with open(path, "w") as f:
        for toks in arrays:
            f.write("[" + ", ".join(toks) + "]\n")


def reference_sets():
    out = os.path.join(HERE, "reference")
    os.makedirs(out, exist_ok=True)
    with open(os.path.join(REF, "data", "yield.in")) as f, open(os.path.join(out, "yield.in"), "w") as o:
        o.write(f.read())
    for name in SMALL_SETS:
        for src, dst in ((f"data/{name}.in", f"{name}.in"), (f"data/out/{name}.out", f"{name}.out64"),
                         (f"data/out32/{name}.out", f"{name}.out32")):
            with open(os.path.join(REF, src)) as f, open(os.path.join(out, dst), "w") as o:
                o.write(f.read())
    for name in BIG_SETS:
        arrs = _read(os.path.join(REF, "data", f"{name}.in"))
        _write_tokens(os.path.join(out, f"{name}_every{THIN}.in"), [a[::THIN] for a in arrs])
        for sub, ext in (("out", "out64"), ("out32", "out32")):
            gold = _read(os.path.join(REF, "data", sub, f"{name}.out"))[0]
            _write_tokens(os.path.join(out, f"{name}_every{THIN}.{ext}"), [gold[::THIN]])


def edge_cases() -> dict:
    rows = []  # (strike, T, t, unit, steps, a, sigma, type)
    # maturity-step truncation traps: (int)(t/dt) lands one below t*steps in double
    for steps in (75, 77, 7, 49):
        for t in (1.0, 2.0, 3.0, 4.0, 5.0):
            rows.append((90.0, t + 4.0, t, 365, steps, 0.1, 0.01, 1))
            rows.append((90.0, t + 4.0, t, 365, steps, 0.1, 0.01, 0))
    # jmax 1 and 2 (edge jumps onto the same node), one and few steps per year
    for a in (0.1, 0.2, 0.25, 0.5, 1.0):
        for steps in (1, 2, 3):
            rows.append((95.0, 6.0, 2.0, 365, steps, a, 0.02, 1))
            rows.append((80.0, 6.0, 2.0, 365, steps, a, 0.02, 0))
    # option maturity at, after and just before bond maturity; m == 0; n == 1; n == 0
    for t, T in ((5.0, 5.0), (7.0, 5.0), (4.99, 5.0), (0.01, 5.0), (0.0, 3.0), (1.0, 1.0), (0.5, 1.0 / 12.0),
                 (1.0, 0.0)):
        rows.append((90.0, T, t, 365, 12, 0.1, 0.01, 1))
        rows.append((70.0, T, t, 365, 12, 0.1, 0.01, 0))
    # term units shorter than a year: units per year = ceil(365/unit)
    for unit in (30, 91, 182, 360):
        rows.append((88.0, 4.0, 1.0, unit, 2, 0.1, 0.01, 1))
        rows.append((88.0, 4.0, 1.0, unit, 3, 0.15, 0.015, 0))
    # trees that never reach +-jmax (tiny a) and zero volatility
    for a in (0.0005, 0.002, 0.01):
        rows.append((85.0, 5.0, 2.0, 365, 12, a, 0.01, 1))
        rows.append((85.0, 5.0, 2.0, 365, 24, a, 0.01, 0))
    rows.append((90.0, 5.0, 2.0, 365, 12, 0.1, 0.0, 1))
    rows.append((90.0, 5.0, 2.0, 365, 12, 0.1, 0.0, 0))
    # deep in / out of the money
    for X in (0.0, 1.0, 50.0, 99.0, 150.0):
        rows.append((X, 10.0, 5.0, 365, 12, 0.1, 0.01, 1))
        rows.append((X, 10.0, 5.0, 365, 12, 0.1, 0.01, 0))
    # block trees: widths around the warp/block switch and every block K class
    for a, steps, T in ((0.06, 48, 6.0), (0.05, 48, 8.0), (0.03, 48, 10.0), (0.02, 64, 12.0), (0.015, 96, 12.0),
                        (0.012, 96, 14.0), (0.045, 60, 8.0), (0.035, 48, 12.0)):
        rows.append((80.0, T, T / 2, 365, steps, a, 0.01, 1))
        rows.append((80.0, T, T / 2, 365, steps, a, 0.012, 0))
    cols = list(zip(*rows))
    return dict(strike=np.array(cols[0]), bond_maturity=np.array(cols[1]), option_maturity=np.array(cols[2]),
                term_unit=np.array(cols[3], dtype=np.uint16), term_steps=np.array(cols[4], dtype=np.uint16),
                a=np.array(cols[5]), sigma=np.array(cols[6]), type=np.array(cols[7], dtype=np.int8))


def synthetic_sets():
    out = os.path.join(HERE, "synthetic")
    os.makedirs(out, exist_ok=True)
    rates, days = wl.yield_curve()
    pkg.Yield(rates, days)
    with open(os.path.join(out, "curve11.in"), "w") as f:
        pkg.write_array(f, rates, 17)
        pkg.write_array(f, days, 0)
    uneven = wl.uneven_batch()
    skew = wl.skewed_batch()
    heavy = np.where(skew["a"] < 0.05)[0]
    light = np.where(skew["a"] >= 0.05)[0]
    skew_idx = np.concatenate([heavy[:48], light[:464]])
    sets = {
        "uniform_1k": wl.uniform_book(),
        "uneven_2k": {k: v[:2000] for k, v in uneven.items()},
        "skewed_512": {k: v[skew_idx] for k, v in skew.items()},
        "book_100": wl.book_batch(100),
        "edge": edge_cases(),
    }
    seq64 = os.path.join(ROOT, "oracle", "_ref", "Seq64")
    seq32 = os.path.join(ROOT, "oracle", "_ref", "Seq32")
    for name, b in sets.items():
        opts = pkg.Options.from_batch(b)
        path = os.path.join(out, f"{name}.in")
        opts.write_to_file(path)
        for exe, ext in ((seq64, "out64"), (seq32, "out32")):
            res = subprocess.run([exe, "-o", path, "-y", os.path.join(out, "curve11.in")], capture_output=True,
                                 text=True, check=True)
            with open(os.path.join(out, f"{name}.{ext}"), "w") as f:
                f.write(res.stdout)


if __name__ == "__main__":
    if not os.path.isdir(REF):
        sys.exit("reference sources not mounted")
    reference_sets()
    synthetic_sets()
    print("golden fixtures written")
