"""GB300 Hull-White trinomial-tree batch pricer - Python side of the C ABI.

Mirrors the reference project's batch pricing interface (MartinMetaksov/
diku.OptionsPricing) for Python callers and tests:

  Options / Yield        common/Options.hpp:48-125, common/Yield.hpp:14-40 (SoA records,
                         same .in text files)
  read_array/write_array common/Arrays.hpp:15-46 ("[a, b, c]", std::fixed, max_digits10)
  compute_options        seq::computeOptions (seq/Seq.hpp:181-190)
  KernelRun.run          KernelRunBase::run (cuda-option/Kernel.cuh:303-314)

Every pricing call goes through libhwtree.so (include/hwtree.h) to the sm_103a
kernels; there is no CPU pricing path in this package.  Loading fails loudly when
the library has not been built (``python diku.optionspricing_gb300/build.py`` or
``__graft_entry__.build()``).
"""
from __future__ import annotations

import ctypes
import enum
import io
import os
import re
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libhwtree.so")
ABI_VERSION = 2  # include/hwtree.h HWT_ABI_VERSION

# Status codes (hwtree.h)
HWT_OK, HWT_EINVAL, HWT_ECUDA, HWT_ENOMEM, HWT_EUNSUPPORTED, HWT_ENODEV, HWT_ETIMEOUT = 0, -1, -2, -3, -4, -5, -6

# Pricing modes (hwtree.h)
PLAIN_FP64, BATCHED_FP64, BATCHED_FP32, BATCHED_MIXED, BATCHED_DF64 = 0, 1, 2, 3, 4
MODE_NAMES = {PLAIN_FP64: "plain_fp64", BATCHED_FP64: "batched_fp64", BATCHED_FP32: "batched_fp32",
              BATCHED_MIXED: "batched_mixed", BATCHED_DF64: "batched_df64"}


class OptionType(enum.IntEnum):
    """common/Options.hpp:24-28"""
    CALL = 0
    PUT = 1


class SortType(str, enum.Enum):
    """common/Options.hpp:15-22: the order the engine schedules trees in (results
    never depend on it).  NONE is the engine's own order (heaviest first); INPUT,
    an addition, keeps arrival order without binning by size."""
    WIDTH_DESC = "W"
    WIDTH_ASC = "w"
    HEIGHT_DESC = "H"
    HEIGHT_ASC = "h"
    NONE = "-"
    INPUT = "i"


class HwtError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"[{code}] {message}")
        self.code = code


class InvalidInput(HwtError, ValueError):
    pass


# ---------------------------------------------------------------------------
# C ABI
# ---------------------------------------------------------------------------
class _Options(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int32), ("strike", ctypes.c_void_p), ("bond_maturity", ctypes.c_void_p),
                ("option_maturity", ctypes.c_void_p), ("term_unit", ctypes.c_void_p),
                ("term_steps", ctypes.c_void_p), ("a", ctypes.c_void_p), ("sigma", ctypes.c_void_p),
                ("type", ctypes.c_void_p)]


class _Yield(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int32), ("rate", ctypes.c_void_p), ("day", ctypes.c_void_p)]


class Config(ctypes.Structure):
    """hwt_config: mode, block_size, sort, big_threshold, use_graph, record_busy, warp_k_mask."""
    _fields_ = [("mode", ctypes.c_int32), ("block_size", ctypes.c_int32), ("sort", ctypes.c_int32),
                ("big_threshold", ctypes.c_int32), ("use_graph", ctypes.c_int32), ("record_busy", ctypes.c_int32),
                ("warp_k_mask", ctypes.c_int32)]


class Stats(ctypes.Structure):
    """hwt_stats (see include/hwtree.h for field meanings)."""
    _fields_ = [("total_ms", ctypes.c_double), ("pricing_ms", ctypes.c_double), ("sizing_ms", ctypes.c_double),
                ("nodes", ctypes.c_int64), ("h2d_bytes", ctypes.c_int64), ("d2h_bytes", ctypes.c_int64),
                ("device_bytes", ctypes.c_int64), ("kernel_launches", ctypes.c_int32),
                ("n_block_trees", ctypes.c_int32), ("n_warp_tasks", ctypes.c_int32), ("grid", ctypes.c_int32),
                ("block_size", ctypes.c_int32), ("max_width", ctypes.c_int32), ("max_height", ctypes.c_int32),
                ("graph_replayed", ctypes.c_int32), ("busy_max_ms", ctypes.c_double),
                ("busy_mean_ms", ctypes.c_double)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


_lib = None

# Every function the header declares, with its ctypes signature.
_SIGNATURES = {
    "hwt_abi_version": (ctypes.c_int, []),
    "hwt_struct_size": (ctypes.c_size_t, [ctypes.c_char_p]),
    "hwt_create": (ctypes.c_void_p, [ctypes.c_int, ctypes.c_char_p]),
    "hwt_create_status": (ctypes.c_int, []),
    "hwt_destroy": (None, [ctypes.c_void_p]),
    "hwt_last_error": (ctypes.c_char_p, [ctypes.c_void_p]),
    "hwt_price": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(_Options), ctypes.POINTER(_Yield), ctypes.c_int,
                                 ctypes.c_void_p, ctypes.POINTER(Stats)]),
    "hwt_price_ex": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(_Options), ctypes.POINTER(_Yield),
                                    ctypes.POINTER(Config), ctypes.c_void_p, ctypes.POINTER(Stats)]),
    "hwt_price_device": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(_Options), ctypes.POINTER(_Yield),
                                        ctypes.POINTER(Config), ctypes.c_void_p, ctypes.POINTER(Stats)]),
    "hwt_shape": (ctypes.c_int, [ctypes.POINTER(_Options), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                 ctypes.c_void_p]),
    "hwt_active_nodes": (ctypes.c_int64, [ctypes.c_int32, ctypes.c_int32]),
    "hwt_warp_layout": (ctypes.c_int, [ctypes.c_int, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                       ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32)]),
    "hwt_autotune": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(_Options), ctypes.POINTER(_Yield), ctypes.c_int,
                                    ctypes.c_int, ctypes.POINTER(Config)]),
    "hwt_get_config": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(Config)]),
    "hwt_measure_peaks": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double),
                                         ctypes.POINTER(ctypes.c_double)]),
    "hwt_price_device_noalloc": (ctypes.c_int, [ctypes.POINTER(_Options), ctypes.POINTER(_Yield), ctypes.c_int,
                                                ctypes.c_void_p, ctypes.c_void_p]),
    "hwt_read_options": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(_Options), ctypes.c_char_p, ctypes.c_int]),
    "hwt_free_options": (None, [ctypes.POINTER(_Options)]),
    "hwt_write_options_bin": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(_Options)]),
    "hwt_read_yield": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(_Yield), ctypes.c_char_p, ctypes.c_int]),
    "hwt_free_yield": (None, [ctypes.POINTER(_Yield)]),
}


def lib() -> ctypes.CDLL:
    """The loaded C-ABI library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build the native library first "
                              "(python diku.optionspricing_gb300/build.py)")
        handle = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(handle, name)
            fn.restype = res
            fn.argtypes = args
        if handle.hwt_abi_version() != ABI_VERSION:
            raise ImportError(f"{LIB_PATH} has ABI version {handle.hwt_abi_version()}, this binding {ABI_VERSION}: "
                              "rebuild the native library")
        for cname, cls in _RECORDS.items():
            if handle.hwt_struct_size(cname.encode()) != ctypes.sizeof(cls):
                raise ImportError(f"{cname}: {handle.hwt_struct_size(cname.encode())} bytes in {LIB_PATH}, "
                                  f"{ctypes.sizeof(cls)} in this binding: rebuild the native library")
        _lib = handle
    return _lib


# ---------------------------------------------------------------------------
# Records and text format
# ---------------------------------------------------------------------------
_ARRAY_RE = re.compile(r"\[([^\]]*)\]")


def read_arrays(text: str) -> list[list[str]]:
    """All "[..]" arrays of a text, as token lists (common/Arrays.hpp:15-32)."""
    out = []
    for body in _ARRAY_RE.findall(text):
        toks = [t.strip() for t in body.split(",")]
        out.append([t for t in toks if t])
    return out


def read_array(stream) -> list[str]:
    """Reads the next "[..]" array from a text stream."""
    buf = []
    started = False
    while True:
        ch = stream.read(1)
        if not ch:
            break
        if ch == "[":
            started = True
            continue
        if started:
            if ch == "]":
                break
            buf.append(ch)
    return [t.strip() for t in "".join(buf).split(",") if t.strip()]


def format_array(values, digits: int = 17) -> str:
    """common/Arrays.hpp:34-46: '[' std::fixed values at max_digits10 ']'.
    digits=17 for double, 9 for float, 0 for integer arrays."""
    arr = np.asarray(values)
    if arr.dtype.kind in "iub" or digits == 0:
        body = ", ".join(str(int(v)) for v in arr)
    else:
        body = ", ".join("%.*f" % (digits, float(v)) for v in arr)
    return "[" + body + "]\n"


def write_array(stream, values, digits: int = 17) -> None:
    stream.write(format_array(values, digits))


@dataclass
class Options:
    """SoA option records (common/Options.hpp:48-58) with real = double."""
    StrikePrices: np.ndarray
    Maturities: np.ndarray
    Lengths: np.ndarray
    TermUnits: np.ndarray
    TermStepCounts: np.ndarray
    ReversionRates: np.ndarray
    Volatilities: np.ndarray
    Types: np.ndarray

    def __post_init__(self):
        self.StrikePrices = np.ascontiguousarray(self.StrikePrices, dtype=np.float64)
        self.Maturities = np.ascontiguousarray(self.Maturities, dtype=np.float64)
        self.Lengths = np.ascontiguousarray(self.Lengths, dtype=np.float64)
        self.TermUnits = np.ascontiguousarray(self.TermUnits, dtype=np.uint16)
        self.TermStepCounts = np.ascontiguousarray(self.TermStepCounts, dtype=np.uint16)
        self.ReversionRates = np.ascontiguousarray(self.ReversionRates, dtype=np.float64)
        self.Volatilities = np.ascontiguousarray(self.Volatilities, dtype=np.float64)
        self.Types = np.ascontiguousarray(self.Types, dtype=np.int8)
        n = len(self.StrikePrices)
        for name in ("Maturities", "Lengths", "TermUnits", "TermStepCounts", "ReversionRates", "Volatilities",
                     "Types"):
            if len(getattr(self, name)) != n:
                raise ValueError(f"option array {name} has {len(getattr(self, name))} entries, expected {n}")

    @property
    def N(self) -> int:
        return len(self.StrikePrices)

    @classmethod
    def from_file(cls, filename: str) -> "Options":
        """Options(const std::string&) (common/Options.hpp:73-98): eight arrays in
        field order (or a binary cache file from to_bin); a type other than 0/1 is
        rejected.  Parsed by the library's threaded reader (hwt_read_options)."""
        if not filename:
            raise ValueError("File not specified.")
        if not os.path.exists(filename):
            raise ValueError(f"File '{filename}' does not exist.")
        o = _Options()
        err = ctypes.create_string_buffer(512)
        rc = lib().hwt_read_options(filename.encode(), ctypes.byref(o), err, len(err))
        if rc != 0:
            msg = err.value.decode()
            # the reference throws out_of_range for a bad type, invalid_argument otherwise
            raise (IndexError if msg.startswith("Invalid OptionType") else ValueError)(msg)
        try:
            n = o.n

            def arr(ptr, dt):
                return np.ctypeslib.as_array((ctypes.c_char * (n * np.dtype(dt).itemsize)).from_address(ptr)) \
                    .view(dt).copy() if n else np.zeros(0, dtype=dt)
            return cls(arr(o.strike, np.float64), arr(o.bond_maturity, np.float64), arr(o.option_maturity, np.float64),
                       arr(o.term_unit, np.uint16), arr(o.term_steps, np.uint16), arr(o.a, np.float64),
                       arr(o.sigma, np.float64), arr(o.type, np.int8))
        finally:
            lib().hwt_free_options(ctypes.byref(o))

    def to_bin(self, filename: str) -> None:
        """Writes the binary cache file hwt_read_options / from_file read back."""
        o = self._c()
        if lib().hwt_write_options_bin(filename.encode(), ctypes.byref(o)) != 0:
            raise OSError(f"cannot write '{filename}'")

    @classmethod
    def from_text(cls, text: str) -> "Options":
        """Parses the eight "[..]" arrays of a text in Python (common/Arrays.hpp:15-32)."""
        arrs = read_arrays(text)
        if len(arrs) < 8:
            raise ValueError(f"The text holds {len(arrs)} arrays, expected 8.")
        types = np.array([int(float(t)) for t in arrs[7]], dtype=np.int64)
        if np.any((types != 0) & (types != 1)):
            raise IndexError("Invalid OptionType read from stream.")
        return cls(np.array(arrs[0], dtype=np.float64), np.array(arrs[1], dtype=np.float64),
                   np.array(arrs[2], dtype=np.float64), np.array([int(float(t)) for t in arrs[3]]),
                   np.array([int(float(t)) for t in arrs[4]]), np.array(arrs[5], dtype=np.float64),
                   np.array(arrs[6], dtype=np.float64), types)

    @classmethod
    def from_batch(cls, b: dict) -> "Options":
        """From a workloads.py batch dict."""
        return cls(b["strike"], b["bond_maturity"], b["option_maturity"], b["term_unit"], b["term_steps"], b["a"],
                   b["sigma"], b["type"])

    def to_text(self) -> str:
        buf = io.StringIO()
        for arr, digits in ((self.StrikePrices, 17), (self.Maturities, 17), (self.Lengths, 17),
                            (self.TermUnits, 0), (self.TermStepCounts, 0), (self.ReversionRates, 17),
                            (self.Volatilities, 17), (self.Types, 0)):
            write_array(buf, arr, digits)
        return buf.getvalue()

    def write_to_file(self, filename: str) -> None:
        """Options::writeToFile (common/Options.hpp:100-124)."""
        with open(filename, "w") as f:
            f.write(self.to_text())

    def subset(self, idx) -> "Options":
        return Options(*(getattr(self, f)[idx] for f in _OPTION_FIELDS))

    def _c(self) -> _Options:
        return _Options(self.N, self.StrikePrices.ctypes.data, self.Maturities.ctypes.data, self.Lengths.ctypes.data,
                        self.TermUnits.ctypes.data, self.TermStepCounts.ctypes.data,
                        self.ReversionRates.ctypes.data, self.Volatilities.ctypes.data, self.Types.ctypes.data)


_OPTION_FIELDS = ("StrikePrices", "Maturities", "Lengths", "TermUnits", "TermStepCounts", "ReversionRates",
                  "Volatilities", "Types")


@dataclass
class Yield:
    """Yield curve (common/Yield.hpp:14-40): zero rates at whole-day maturities."""
    Prices: np.ndarray
    TimeSteps: np.ndarray

    def __post_init__(self):
        self.Prices = np.ascontiguousarray(self.Prices, dtype=np.float64)
        self.TimeSteps = np.ascontiguousarray(self.TimeSteps, dtype=np.int32)
        if len(self.Prices) != len(self.TimeSteps):
            raise ValueError("yield arrays differ in length")

    @property
    def N(self) -> int:
        return len(self.Prices)

    @classmethod
    def from_file(cls, filename: str) -> "Yield":
        if not filename:
            raise ValueError("File not specified.")
        if not os.path.exists(filename):
            raise ValueError("File does not exist.")
        y = _Yield()
        err = ctypes.create_string_buffer(512)
        if lib().hwt_read_yield(filename.encode(), ctypes.byref(y), err, len(err)) != 0:
            raise ValueError(err.value.decode())
        try:
            n = y.n
            rates = np.ctypeslib.as_array((ctypes.c_double * n).from_address(y.rate)).copy()
            days = np.ctypeslib.as_array((ctypes.c_int32 * n).from_address(y.day)).copy()
        finally:
            lib().hwt_free_yield(ctypes.byref(y))
        return cls(rates, days)

    def _c(self) -> _Yield:
        return _Yield(self.N, self.Prices.ctypes.data, self.TimeSteps.ctypes.data)


def shape(options: Options) -> dict:
    """Tree shape per option as the reference computes it, on the host (no GPU):
    jmax, height n, width 2*jmax+1, maturity step (common/OptionConstants.hpp:29-53)."""
    n = options.N
    out = {k: np.empty(n, dtype=np.int32) for k in ("jmax", "height", "width", "maturity_step")}
    o = options._c()
    rc = lib().hwt_shape(ctypes.byref(o), out["jmax"].ctypes.data, out["height"].ctypes.data,
                         out["width"].ctypes.data, out["maturity_step"].ctypes.data)
    out["status"] = rc
    return out


def warp_layout(mode: int, width: int, warp_k_mask: int = 0, big_threshold: int = 0) -> tuple[int, int]:
    """(nodes per lane, lanes) of the warp task the batched engine gives a tree of
    `width` nodes, or (0, 0) when the tree goes to a warp group (host only)."""
    k, l = ctypes.c_int32(), ctypes.c_int32()
    rc = lib().hwt_warp_layout(mode, width, warp_k_mask, big_threshold, ctypes.byref(k), ctypes.byref(l))
    if rc != HWT_OK:
        raise InvalidInput(rc, f"no warp layout for mode {mode}, width {width}")
    return k.value, l.value


def active_nodes(height, jmax) -> np.ndarray:
    """Active nodes of one pass: sum_{i<n} (2 min(i, jmax) + 1), the work unit."""
    h = np.asarray(height, dtype=np.int64)
    j = np.asarray(jmax, dtype=np.int64)
    h = np.maximum(h, 0)
    full = (j + 1) ** 2 + (h - j - 1) * (2 * j + 1)
    return np.where(h <= j + 1, h * h, full)


# ---------------------------------------------------------------------------
# Pricer
# ---------------------------------------------------------------------------
class Pricer:
    """One pricing context on one GPU (hwt_create / hwt_destroy)."""

    def __init__(self, device: int = 0, tune_cache: str | None = None):
        L = lib()
        self._ctx = L.hwt_create(device, tune_cache.encode() if tune_cache else None)
        if not self._ctx:
            code = L.hwt_create_status()
            raise HwtError(code, "no CUDA device" if code == HWT_ENODEV else "hwt_create failed")
        self.last_stats = Stats()

    def close(self):
        if getattr(self, "_ctx", None):
            lib().hwt_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc: int):
        if rc != HWT_OK:
            msg = lib().hwt_last_error(self._ctx)
            msg = msg.decode() if msg else ""
            if rc == HWT_EINVAL:
                raise InvalidInput(rc, msg)
            raise HwtError(rc, msg)

    def config(self, mode: int, block_size: int = 0, big_threshold: int = 0, use_graph: bool = True,
               record_busy: bool = False, sort: str = "-", warp_k_mask: int = 0) -> Config:
        return Config(mode, block_size, ord(sort), big_threshold, 1 if use_graph else 0, 1 if record_busy else 0,
                      warp_k_mask)

    def price(self, options: Options, yield_: Yield, mode: int = BATCHED_FP64, out: np.ndarray | None = None,
              **cfg) -> np.ndarray:
        """Prices host-memory options; returns float64 prices in input order."""
        if out is None:
            out = np.empty(options.N, dtype=np.float64)
        o, y, c = options._c(), yield_._c(), self.config(mode, **cfg)
        rc = lib().hwt_price_ex(self._ctx, ctypes.byref(o), ctypes.byref(y), ctypes.byref(c), out.ctypes.data,
                                ctypes.byref(self.last_stats))
        self._check(rc)
        return out

    def price_host_ptrs(self, ptrs: dict, n: int, yield_: Yield, out_ptr: int, mode: int, **cfg) -> Stats:
        """Prices options whose arrays are given as raw host pointers (e.g. pinned
        torch tensors), writing prices to out_ptr."""
        o = _Options(n, *(ptrs[k] for k in ("strike", "bond_maturity", "option_maturity", "term_unit", "term_steps",
                                            "a", "sigma", "type")))
        y, c = yield_._c(), self.config(mode, **cfg)
        rc = lib().hwt_price_ex(self._ctx, ctypes.byref(o), ctypes.byref(y), ctypes.byref(c), out_ptr,
                                ctypes.byref(self.last_stats))
        self._check(rc)
        return self.last_stats

    def price_device(self, ptrs: dict, n: int, yield_: Yield, out_ptr: int, mode: int, **cfg) -> Stats:
        """Prices options already in device memory (raw device pointers)."""
        o = _Options(n, *(ptrs[k] for k in ("strike", "bond_maturity", "option_maturity", "term_unit", "term_steps",
                                            "a", "sigma", "type")))
        y, c = yield_._c(), self.config(mode, **cfg)
        rc = lib().hwt_price_device(self._ctx, ctypes.byref(o), ctypes.byref(y), ctypes.byref(c), out_ptr,
                                    ctypes.byref(self.last_stats))
        self._check(rc)
        return self.last_stats

    def autotune(self, options: Options, yield_: Yield, mode: int, repeats: int = 3) -> Config:
        best = Config()
        o, y = options._c(), yield_._c()
        self._check(lib().hwt_autotune(self._ctx, ctypes.byref(o), ctypes.byref(y), mode, repeats,
                                       ctypes.byref(best)))
        return best

    def get_config(self, mode: int) -> Config:
        c = Config()
        self._check(lib().hwt_get_config(self._ctx, mode, ctypes.byref(c)))
        return c

    def measure_peaks(self) -> tuple[float, float]:
        """(FP64, FP32) FMA peaks of this GPU in TFLOP/s."""
        a, b = ctypes.c_double(), ctypes.c_double()
        self._check(lib().hwt_measure_peaks(self._ctx, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value


_default_pricer = None


def default_pricer() -> Pricer:
    global _default_pricer
    if _default_pricer is None:
        _default_pricer = Pricer(0)
    return _default_pricer


def compute_options(options: Options, yield_: Yield, results=None, mode: int = BATCHED_FP64) -> np.ndarray:
    """seq::computeOptions(options, yield, results) (seq/Seq.hpp:181-190) on the GPU."""
    out = default_pricer().price(options, yield_, mode)
    if results is not None:
        results[:] = out
    return out


class KernelRun:
    """KernelRunBase (cuda-option/Kernel.cuh:218-327): run() prices, runtime keeps stats."""

    def __init__(self, mode: int = BATCHED_FP64):
        self.mode = mode
        self.runtime: dict = {}

    def run(self, options: Options, yield_: Yield, results=None, block_size: int = -1,
            sort_type: SortType = SortType.NONE, is_test: bool = False) -> np.ndarray:
        p = default_pricer()
        out = p.price(options, yield_, self.mode, block_size=max(block_size, 0), sort=SortType(sort_type).value)
        self.runtime = p.last_stats.as_dict()
        if results is not None:
            results[:] = out
        if is_test:
            print(f"Kernel executed in {self.runtime['pricing_ms'] * 1000:.0f} microsec")
            print(f"Total execution time {self.runtime['total_ms'] * 1000:.0f} microsec")
        return out


# ---------------------------------------------------------------------------
# Learned surrogate (hwt_surrogate_*)
# ---------------------------------------------------------------------------
class Box(ctypes.Structure):
    """hwt_box: the surrogate's training box."""
    _fields_ = [("t_min", ctypes.c_double), ("t_max", ctypes.c_double), ("span_min", ctypes.c_double),
                ("span_max", ctypes.c_double), ("moneyness_min", ctypes.c_double),
                ("moneyness_max", ctypes.c_double), ("a_min", ctypes.c_double), ("a_max", ctypes.c_double),
                ("sigma_min", ctypes.c_double), ("sigma_max", ctypes.c_double), ("steps_min", ctypes.c_int32),
                ("steps_max", ctypes.c_int32), ("term_unit", ctypes.c_int32), ("residual", ctypes.c_int32)]


class TrainConfig(ctypes.Structure):
    _fields_ = [("epochs", ctypes.c_int32), ("batch", ctypes.c_int32), ("lr", ctypes.c_double),
                ("lr_min", ctypes.c_double), ("seed", ctypes.c_uint64), ("err_weight", ctypes.c_double),
                ("route_tolerance", ctypes.c_double), ("holdout", ctypes.c_double),
                ("kink_oversample", ctypes.c_int32), ("hard_every", ctypes.c_int32),
                ("hard_fraction", ctypes.c_double)]


class TrainStats(ctypes.Structure):
    _fields_ = [("final_loss", ctypes.c_double), ("train_ms", ctypes.c_double), ("label_ms", ctypes.c_double),
                ("steps", ctypes.c_int64), ("samples", ctypes.c_int64), ("samples_per_s", ctypes.c_double),
                ("y_mean", ctypes.c_double), ("y_std", ctypes.c_double), ("route_threshold", ctypes.c_double),
                ("holdout_answered", ctypes.c_double), ("holdout_max_abs", ctypes.c_double),
                ("holdout_p99_abs", ctypes.c_double), ("holdout_all_max_abs", ctypes.c_double),
                ("holdout", ctypes.c_int64), ("n_kinks", ctypes.c_int64), ("kink_delta", ctypes.c_double),
                ("ladder_tolerance", ctypes.c_double * 12), ("ladder_answered", ctypes.c_double * 12),
                ("holdout_over", ctypes.c_int64), ("hard_minings", ctypes.c_int64),
                ("hard_threshold_abs", ctypes.c_double)]

    def as_dict(self) -> dict:
        d = {name: getattr(self, name) for name, _ in self._fields_}
        d["ladder_tolerance"] = list(d["ladder_tolerance"])
        d["ladder_answered"] = list(d["ladder_answered"])
        return d


class SurrogateStats(ctypes.Structure):
    _fields_ = [("n_in_box", ctypes.c_int64), ("n_routed", ctypes.c_int64), ("n_judged", ctypes.c_int64),
                ("fell_back", ctypes.c_int32), ("pad", ctypes.c_int32), ("judge_max_abs", ctypes.c_double), ("judge_p99_abs", ctypes.c_double),
                ("judge_mean_abs", ctypes.c_double), ("network_ms", ctypes.c_double), ("tree_ms", ctypes.c_double),
                ("route_ms", ctypes.c_double), ("total_ms", ctypes.c_double), ("n_flagged", ctypes.c_int64),
                ("n_network", ctypes.c_int64), ("route_tolerance", ctypes.c_double), ("copy_ms", ctypes.c_double)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


# Records whose layout must match the library's (checked when it is loaded).
_RECORDS = {"hwt_options": _Options, "hwt_yield": _Yield, "hwt_config": Config, "hwt_stats": Stats, "hwt_box": Box,
            "hwt_train_config": TrainConfig, "hwt_train_stats": TrainStats, "hwt_surrogate_stats": SurrogateStats}


_SIGNATURES.update({
    "hwt_surrogate_create": (ctypes.c_void_p, [ctypes.c_void_p, ctypes.POINTER(Box), ctypes.c_uint64]),
    "hwt_surrogate_destroy": (None, [ctypes.c_void_p]),
    "hwt_surrogate_last_error": (ctypes.c_char_p, [ctypes.c_void_p]),
    "hwt_surrogate_train": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(_Options), ctypes.POINTER(_Yield),
                                           ctypes.POINTER(TrainConfig), ctypes.POINTER(TrainStats)]),
    "hwt_surrogate_price": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(_Options), ctypes.POINTER(_Yield),
                                           ctypes.c_double, ctypes.c_uint64, ctypes.c_int, ctypes.c_double,
                                           ctypes.c_void_p, ctypes.POINTER(SurrogateStats)]),
    "hwt_surrogate_save": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p]),
    "hwt_surrogate_load": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p]),
    "hwt_surrogate_param_count": (ctypes.c_int64, [ctypes.c_void_p]),
    "hwt_surrogate_params": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int]),
    "hwt_surrogate_forward": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]),
    "hwt_surrogate_forward_ex": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                                ctypes.c_int]),
    "hwt_surrogate_forward_device": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                                    ctypes.POINTER(ctypes.c_double)]),
    "hwt_surrogate_inject_stall": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "hwt_find_kinks": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                      ctypes.c_void_p, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32)]),
    "hwt_route_distances": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.c_int64, ctypes.c_double, ctypes.c_void_p,
                                           ctypes.POINTER(ctypes.c_double)]),
    "hwt_surrogate_loss_grads": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                                ctypes.c_double, ctypes.POINTER(ctypes.c_double), ctypes.c_void_p]),
})

# first fan-in: 7 features + 1 zero pad row; outputs: price residual, log-error estimate
SURROGATE_DIMS = (8, 256, 256, 256, 256, 2)


class Surrogate:
    """MLP surrogate with the tree as fallback (outside the box) and judge."""

    def __init__(self, pricer: Pricer, box: dict | None = None, seed: int = 1, residual: bool = True):
        from .workloads import SURROGATE_BOX
        b = dict(SURROGATE_BOX if box is None else box)
        b.setdefault("residual", 1 if residual else 0)
        self.box = Box(**b)
        self.pricer = pricer
        self._s = lib().hwt_surrogate_create(pricer._ctx, ctypes.byref(self.box), seed)
        if not self._s:
            raise HwtError(HWT_ECUDA, "hwt_surrogate_create failed")
        self.train_stats = TrainStats()
        self.stats = SurrogateStats()

    def close(self):
        if getattr(self, "_s", None):
            lib().hwt_surrogate_destroy(self._s)
            self._s = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != HWT_OK:
            msg = lib().hwt_surrogate_last_error(self._s)
            raise (InvalidInput if rc == HWT_EINVAL else HwtError)(rc, msg.decode() if msg else "")

    def train(self, samples: Options, yield_: Yield, epochs: int = 1, batch: int = 8192, lr: float = 1e-3,
              lr_min: float = 0.0, seed: int = 7, err_weight: float = 0.0, route_tolerance: float = 1e-4,
              holdout: float = 0.05, kink_oversample: int = 1, hard_every: int = 0,
              hard_fraction: float = 0.0) -> dict:
        """Labels the samples with the FP64 tree and trains; with err_weight > 0 the
        error head is trained too and routes (held-out calibration at route_tolerance);
        on a single-tree box samples near a payoff kink can be repeated per epoch;
        with hard_every > 0 the hard_fraction of training samples with the largest
        errors is repeated per epoch (mined again every hard_every epochs)."""
        cfg = TrainConfig(epochs, batch, lr, lr_min, seed, err_weight, route_tolerance, holdout, kink_oversample,
                          hard_every, hard_fraction)
        o, y = samples._c(), yield_._c()
        self._check(lib().hwt_surrogate_train(self._s, ctypes.byref(o), ctypes.byref(y), ctypes.byref(cfg),
                                              ctypes.byref(self.train_stats)))
        return self.train_stats.as_dict()

    def price(self, options: Options, yield_: Yield, judge_fraction: float = 0.01, seed: int = 11,
              tree_mode: int = BATCHED_MIXED, judge_tolerance: float = 0.0) -> np.ndarray:
        """Network inside the box, tree outside it and on the judged sample; with
        judge_tolerance > 0 a batch whose judged error exceeds it is priced by the tree."""
        out = np.empty(options.N, dtype=np.float64)
        o, y = options._c(), yield_._c()
        self._check(lib().hwt_surrogate_price(self._s, ctypes.byref(o), ctypes.byref(y), judge_fraction, seed,
                                              tree_mode, judge_tolerance, out.ctypes.data, ctypes.byref(self.stats)))
        return out

    def save(self, path: str):
        self._check(lib().hwt_surrogate_save(self._s, path.encode()))

    def load(self, path: str):
        self._check(lib().hwt_surrogate_load(self._s, path.encode()))

    def params(self) -> list[tuple[np.ndarray, np.ndarray]]:
        n = lib().hwt_surrogate_param_count(self._s)
        flat = np.empty(n, dtype=np.float32)
        self._check(lib().hwt_surrogate_params(self._s, flat.ctypes.data, n, 0))
        out, off = [], 0
        for fi, fo in zip(SURROGATE_DIMS[:-1], SURROGATE_DIMS[1:]):
            W = flat[off:off + fi * fo].reshape(fi, fo).copy(); off += fi * fo
            b = flat[off:off + fo].copy(); off += fo
            out.append((W, b))
        return out

    def set_params(self, params):
        flat = np.concatenate([np.concatenate([np.asarray(W, np.float32).ravel(), np.asarray(b, np.float32)])
                               for W, b in params]).astype(np.float32)
        self._check(lib().hwt_surrogate_params(self._s, flat.ctypes.data, len(flat), 1))

    def inject_stall(self, mode) -> None:
        """Test hook: tensor-core kernels wait on an mbarrier phase nothing completes
        (bounded) - mode 1 before their first MMA, 2 after their first K block's MMAs
        (True means 1) - so calls return HWT_ETIMEOUT; the context stays usable."""
        self._check(lib().hwt_surrogate_inject_stall(self._s, int(mode)))

    def forward(self, x: np.ndarray, fused: bool = True) -> np.ndarray:
        """Network outputs [n, 2] for standardised features x [n, 7]: the fused
        inference kernel, or the layer-by-layer training kernels."""
        x = np.ascontiguousarray(x, dtype=np.float32)
        out = np.empty((len(x), 2), dtype=np.float32)
        self._check(lib().hwt_surrogate_forward_ex(self._s, x.ctypes.data, len(x), out.ctypes.data, 0 if fused else 1))
        return out

    def forward_device(self, x_ptr: int, n: int, out_ptr: int) -> float:
        """Fused kernel on device buffers (x [n][8] float32 with a zero last column,
        out [n][2] float32); returns the kernel's CUDA-event time in ms."""
        ms = ctypes.c_double()
        self._check(lib().hwt_surrogate_forward_device(self._s, x_ptr, n, out_ptr, ctypes.byref(ms)))
        return ms.value

    def loss_grads(self, x: np.ndarray, y: np.ndarray, err_weight: float = 0.0):
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.ascontiguousarray(y, dtype=np.float32)
        n = lib().hwt_surrogate_param_count(self._s)
        g = np.empty(n, dtype=np.float32)
        loss = ctypes.c_double()
        self._check(lib().hwt_surrogate_loss_grads(self._s, x.ctypes.data, y.ctypes.data, len(x), err_weight,
                                                   ctypes.byref(loss), g.ctypes.data))
        grads, off = [], 0
        for fi, fo in zip(SURROGATE_DIMS[:-1], SURROGATE_DIMS[1:]):
            gW = g[off:off + fi * fo].reshape(fi, fo).copy(); off += fi * fo
            gb = g[off:off + fo].copy(); off += fo
            grads.append((gW, gb))
        return loss.value, grads


from . import workloads  # noqa: E402  (seeded synthetic batches)


def find_kinks(x, price, type_, cap: int = 256) -> np.ndarray:
    """Payoff kinks (moneyness, ascending) of one tree from labelled samples
    (hwt_find_kinks; host only, the surrogate training's own code)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    price = np.ascontiguousarray(price, dtype=np.float64)
    t = np.ascontiguousarray(type_, dtype=np.int8)
    out = np.empty(cap, dtype=np.float64)
    count = ctypes.c_int32(0)
    rc = lib().hwt_find_kinks(x.ctypes.data, price.ctypes.data, t.ctypes.data, len(x), out.ctypes.data, cap,
                              ctypes.byref(count))
    if rc != 0:
        raise ValueError(f"hwt_find_kinks: {count.value} kinks (cap {cap}), status {rc}")
    return out[:count.value].copy()


def route_distances(points, x, err, tol: float) -> tuple[np.ndarray, float]:
    """Routing distance per point and the answered fraction (hwt_route_distances;
    host only, the surrogate training's calibration)."""
    p = np.ascontiguousarray(points, dtype=np.float64)
    x = np.ascontiguousarray(x, dtype=np.float64)
    e = np.ascontiguousarray(err, dtype=np.float64)
    d = np.empty(len(p), dtype=np.float64)
    ans = ctypes.c_double(0.0)
    rc = lib().hwt_route_distances(p.ctypes.data, len(p), x.ctypes.data, e.ctypes.data, len(x), tol, d.ctypes.data,
                                   ctypes.byref(ans))
    if rc != 0:
        raise ValueError(f"hwt_route_distances: status {rc}")
    return d, ans.value
