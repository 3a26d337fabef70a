"""ORACLE - test infrastructure, not the product.

ctypes wrapper over liboracle.so, the plain-C restatement of the reference's CPU
pricer (oracle/hwt_seq.c: seq/Seq.hpp:24-190, common/OptionConstants.hpp:29-53,
common/Domain.hpp:11-169).  Used only by tests/, __graft_entry__.smoke() and
bench.py's CPU baseline, always to check results against or as the timed CPU
reference.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")

_FIELDS = ("StrikePrices", "Maturities", "Lengths", "TermUnits", "TermStepCounts", "ReversionRates",
           "Volatilities", "Types")
_lib = None


def build() -> str:
    """Compiles the restatement with gcc -O2 -fopenmp (no -ffast-math)."""
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    src = [os.path.join(HERE, "hwt_seq.c"), os.path.join(HERE, "hwt_seq_body.h")]
    if not os.path.exists(LIB) or any(os.path.getmtime(s) > os.path.getmtime(LIB) for s in src):
        subprocess.run(["gcc", "-O2", "-fopenmp", "-fPIC", "-shared", "-o", LIB, src[0], "-lm"], check=True)
    return LIB


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        _lib = ctypes.CDLL(LIB)
        for fn in ("oracle_price_f64", "oracle_price_f32"):
            getattr(_lib, fn).restype = ctypes.c_int
        _lib.oracle_max_threads.restype = ctypes.c_int
    return _lib


def _arrays(options, real):
    conv = (real, real, real, np.uint16, np.uint16, real, real, np.int8)
    return [np.ascontiguousarray(getattr(options, f), dtype=t) for f, t in zip(_FIELDS, conv)]


def price(options, yield_, precision: str = "f64", threads: int = 0) -> np.ndarray:
    """Reference seq pricer restated in C: 'f64' (the -DUSE_DOUBLE build) or 'f32'
    (the default float build).  threads <= 0: OpenMP default."""
    real = np.float64 if precision == "f64" else np.float32
    arrs = _arrays(options, real)
    rates = np.ascontiguousarray(yield_.Prices, dtype=real)
    days = np.ascontiguousarray(yield_.TimeSteps, dtype=np.int32)
    out = np.zeros(len(arrs[0]), dtype=real)
    fn = lib().oracle_price_f64 if precision == "f64" else lib().oracle_price_f32
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    rc = fn(ctypes.c_int(len(out)), *[P(a) for a in arrs], ctypes.c_int(len(rates)), P(rates), P(days), P(out),
            ctypes.c_int(threads))
    if rc != 0:
        raise MemoryError("oracle scratch allocation failed")
    return out


def shape(options, precision: str = "f64") -> dict:
    real = np.float64 if precision == "f64" else np.float32
    arrs = _arrays(options, real)
    n = len(arrs[0])
    out = {k: np.zeros(n, dtype=np.int32) for k in ("jmax", "height", "width", "maturity_step")}
    fn = lib().oracle_shape_f64 if precision == "f64" else lib().oracle_shape_f32
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    fn(ctypes.c_int(n), P(arrs[1]), P(arrs[2]), P(arrs[3]), P(arrs[4]), P(arrs[5]), P(arrs[6]),
       P(out["jmax"]), P(out["height"]), P(out["width"]), P(out["maturity_step"]))
    return out


def max_threads() -> int:
    return int(lib().oracle_max_threads())


def reference_binary(precision: str = "f64") -> str | None:
    """Path of the reference seq/ built from its sources (oracle/Makefile), if built."""
    p = os.path.join(REF_DIR, "Seq64" if precision == "f64" else "Seq32")
    return p if os.path.exists(p) else None
