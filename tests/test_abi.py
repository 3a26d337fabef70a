"""The C-ABI library loads, exports every entry point include/hwtree.h declares,
and its host-only functions behave (no GPU compute here)."""
import os
import re

import numpy as np
import pytest

from conftest import ROOT, REF_SETS, SYN_SETS, load_set

HEADER = os.path.join(ROOT, "include", "hwtree.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(hwt_[a-z_0-9]+)\s*\(", text)))


def test_every_declared_symbol_is_exported(pkg):
    lib = pkg.lib()
    names = declared_functions()
    assert len(names) >= 10
    for n in names:
        assert hasattr(lib, n), n


def test_python_binding_covers_header(pkg):
    assert set(declared_functions()) == set(pkg._SIGNATURES)


def test_abi_version(pkg):
    assert pkg.lib().hwt_abi_version() == 2


def test_record_layouts_match_the_library(pkg):
    """Every record the binding passes has the size the library was built with
    (hwt_struct_size); an unknown name answers 0."""
    import ctypes
    lib = pkg.lib()
    for cname, cls in pkg._RECORDS.items():
        assert lib.hwt_struct_size(cname.encode()) == ctypes.sizeof(cls), cname
    assert lib.hwt_struct_size(b"hwt_nothing") == 0 and lib.hwt_struct_size(None) == 0


def test_active_nodes_formula(pkg):
    for n, j in ((0, 5), (1, 5), (5, 5), (6, 5), (7, 5), (120, 23), (2880, 1767), (10, 100)):
        brute = sum(2 * min(i, j) + 1 for i in range(n))
        assert pkg.lib().hwt_active_nodes(n, j) == brute
        assert pkg.active_nodes(n, j) == brute


def test_shape_of_uniform_book(pkg):
    opts, _, _, _ = load_set(pkg, "uniform_1k")
    s = pkg.shape(opts)
    assert s["status"] == 0
    assert np.all(s["jmax"] == 23) and np.all(s["width"] == 47) and np.all(s["height"] == 120)
    assert np.all(s["maturity_step"] == 60)


def test_shape_rejects_bad_records(pkg):
    opts, _, _, _ = load_set(pkg, "book")
    opts.ReversionRates[2] = 0.0
    opts.TermStepCounts[3] = 0
    s = pkg.shape(opts)
    assert s["status"] == pkg.HWT_EINVAL
    assert s["jmax"][2] == -1 and s["jmax"][3] == -1 and s["jmax"][0] > 0


def test_null_context_is_einval(pkg):
    assert pkg.lib().hwt_price(None, None, None, 1, None, None) == pkg.HWT_EINVAL


def test_warp_layout_policy(pkg):
    """How trees are laid out (the sizing kernel's choice, queried on the host):
    the smallest K x L covering the width with ties to the larger K, K = 32 (shared
    memory coefficients) only where no smaller K fits, the widest warp task set by
    the threshold and the K set."""
    lay = pkg.warp_layout
    for mode in (pkg.BATCHED_MIXED, pkg.BATCHED_FP32):
        assert lay(mode, 5) == (8, 1)
        assert lay(mode, 100) == (16, 8)
        assert lay(mode, 140) == (16, 16)
        assert lay(mode, 512) == (16, 32)
        assert lay(mode, 513) == (32, 32)      # default threshold 1,024: one warp
        assert lay(mode, 1025) == (0, 0)       # warp groups
        assert lay(mode, 600, big_threshold=512) == (0, 0)
        assert lay(mode, 13, warp_k_mask=0x400, big_threshold=512) == (32, 1)  # K = 32 alone
        assert lay(mode, 600, warp_k_mask=0x400, big_threshold=512) == (0, 0)
    assert lay(pkg.BATCHED_FP64, 200) == (7, 32)   # double rows: every K in 1..8, 224 slots
    assert lay(pkg.BATCHED_FP64, 13) == (7, 2)
    assert lay(pkg.BATCHED_FP64, 257) == (0, 0)    # threshold 256
    assert lay(pkg.BATCHED_FP64, 200, warp_k_mask=0x7FF) == (7, 32)  # no K above 8 for double rows
    assert lay(pkg.BATCHED_DF64, 200) == (8, 32)   # {1, 2, 3, 4, 6, 8}
    for bad in ((pkg.PLAIN_FP64, 10), (pkg.BATCHED_MIXED, 0), (pkg.BATCHED_MIXED, 5000)):
        with pytest.raises(pkg.InvalidInput):
            lay(*bad)
