"""Benchmark: options/sec of the Hull-White trinomial-tree batch pricer on one GB300
(or N replicas under torchrun), with the FP64 oracle's CPU time beside it.

Workload (default): the 30,000-option uneven batch (seed 1): option maturity
U{1..10} y, bond maturity = option maturity + U{1..10} y, steps/year U{6..48},
a U[0.02,0.20], sigma U[0.005,0.02], strike = forward bond price x U[0.9,1.1],
11-node curve.  The headline is the batched mixed-precision tree (the fastest
mode whose prices stay within 1e-4 absolute per 100 face of the FP64 oracle; the
error is measured in this run and reported).  One step = one hwt_price call on
the whole batch.

  value  options/s with inputs resident in device memory (hwt_price_device),
         device time from CUDA events on the pricer's stream, L2 flushed between
         steps (256 MB memset)
  e2e    options/s through hwt_price with pinned host inputs/outputs: host clock
         around the call, which includes the H2D copy of the options, validation,
         binning, pricing and the D2H copy of the prices

`--impl reference` times the reference's CPU algorithm instead (the oracle: the
C restatement of seq/, OpenMP over options, all host threads) on a bounded sample.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "options/sec at <=1e-4 abs err: FP64 tree vs mixed/batched tree vs surrogate"
# Best CUDA options/s the reference's thesis reports per benchmark set (FP64, FP32):
# max over cuda-option and cuda-multi of 65,536 / best kernel time, GTX 780 Ti
# (results/main/option.csv:107,66,266,2796,416,2844,566,2894,876,814,1019,3044;
# results/main/multi.csv:361,346 for 4_SKEWED).
THESIS_BEST = {
    "0_UNIFORM": (2.66e5, 1.24e6), "1_RAND": (7.85e3, 3.29e4), "2_RANDCONSTHEIGHT": (1.22e5, 6.28e5),
    "3_RANDCONSTWIDTH": (4.40e4, 2.26e5), "4_SKEWED": (5.75e4, 1.47e5), "5_SKEWEDCONSTHEIGHT": (1.01e5, 2.74e5),
    "6_SKEWEDCONSTWIDTH": (1.05e5, 2.94e5),
}
# FLOP per active node of the two sweeps (forward: Q*E*G 2 + 3-term gather 5 +
# alpha accumulate 2; backward: gather 5 + discount 2), the fixed work unit.
FLOP_PER_NODE = 16


WORKLOAD_NAMES = ["uniform_1k", "uneven_30k", "skewed_100k", "0_uniform", "1_rand", "2_randconstheight",
                  "3_randconstwidth", "4_skewed", "5_skewedconstheight", "6_skewedconstwidth"]


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def init_dist(world: int, backend: str):
    if world <= 1:
        return None
    import torch.distributed as dist
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group(backend=backend)
    return dist


def max_over_ranks(value: float, dist, device=None) -> float:
    """Max of a float over ranks (barrier included)."""
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def shard_lpt(work: np.ndarray, world: int) -> list[np.ndarray]:
    """Longest-processing-time partition of options by work (16 x active nodes):
    how a batch splits across GPUs when it is sharded instead of replicated."""
    order = np.argsort(-work, kind="stable")
    loads = np.zeros(world)
    parts = [[] for _ in range(world)]
    for i in order:
        r = int(np.argmin(loads))
        parts[r].append(i)
        loads[r] += work[i]
    return [np.array(sorted(p), dtype=np.int64) for p in parts]


def shard_parts(pkg, opts, world: int) -> list[np.ndarray]:
    """The LPT split of a batch by its tree work (host shapes, no GPU)."""
    shp = pkg.shape(opts)
    work = FLOP_PER_NODE * pkg.active_nodes(shp["height"], shp["jmax"]).astype(np.float64)
    return shard_lpt(work, world)


def gather_prices(local, parts, dist, device=None):
    """Every rank's shard prices (`local`: this rank's, in the order of its part)
    into one float64 tensor in input order, on every rank: an all-gather of the
    shards padded to the widest one, then a scatter by the parts' indices.  The
    only exchange of the sharded path (options are independent)."""
    import torch
    world = len(parts)
    n = int(sum(len(p) for p in parts))
    width = max(len(p) for p in parts)
    buf = torch.zeros(width, dtype=torch.float64, device=device)
    buf[:local.numel()] = local
    outs = [torch.empty_like(buf) for _ in range(world)]
    dist.all_gather(outs, buf)
    full = torch.empty(n, dtype=torch.float64, device=device)
    for r, p in enumerate(parts):
        full[torch.from_numpy(p).to(device)] = outs[r][:len(p)]
    return full


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi while running."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def load_json(path):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return None


def single_thread_rate(orc, opts, y, count=400):
    """The oracle on one host thread over the first `count` options (best of 2)."""
    import __graft_entry__ as g
    pkg = g.package()
    sub = opts.subset(np.arange(min(count, opts.N)))
    best = 1e300
    for _ in range(2):
        t0 = time.perf_counter()
        orc.price(sub, y, "f64", threads=1)
        best = min(best, time.perf_counter() - t0)
    return {"value": sub.N / best, "unit": "options/s", "cores": 1, "sample": f"first {sub.N} options, best of 2"}


def cpu_reference(args, rank, world):
    """--impl reference: the reference's CPU algorithm (oracle port) on the host."""
    import __graft_entry__ as g
    if rank != 0:
        return 0
    pkg, orc = g.package(), g.oracle()
    orc.build()
    wl = pkg.workloads
    batch = wl.WORKLOADS[args.workload]()
    rates, days = wl.yield_curve()
    y = pkg.Yield(rates, days)
    n_total = len(batch["strike"])
    sample = min(n_total, args.ref_sample)
    opts = pkg.Options.from_batch({k: v[:sample] for k, v in batch.items()})
    threads = orc.max_threads()
    for _ in range(args.warmup):
        orc.price(opts, y, "f64")
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        orc.price(opts, y, "f64")
        times.append(time.perf_counter() - t0)
    per = sum(times) / len(times)
    value = sample / per
    one = single_thread_rate(orc, opts, y)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "options/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": per * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded numpy)",
        "config": {"workload": args.workload, "options": n_total},
        "implementation": "oracle/hwt_seq.c: C restatement of the reference seq/ pricer (pinned to the reference's "
                          "own seq/ build and goldens), OpenMP over options",
        "cpu_baseline": {"value": value, "unit": "options/s", "cores": threads, "kind": "port",
                         "sample": f"first {sample} of the {n_total} options of {args.workload} per step, "
                                   f"{args.steps} timed steps",
                         "single_thread": one},
        "e2e": {"value": value, "unit": "options/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def errors(got, ref) -> dict:
    """Max / p99 absolute error and max relative error, the latter against
    max(|ref|, 1e-6) so that prices that are zero up to rounding do not divide by 0."""
    err = np.abs(got - ref)
    return {"max_abs_err": float(np.max(err)), "p99_abs_err": float(np.percentile(err, 99)),
            "max_rel_err": float(np.max(err / np.maximum(np.abs(ref), 1e-6)))}


def config_runs(pkg, orc, pricer, y, reps: int) -> dict:
    """The other benchmark configurations, outside the timed region: device time per
    batch (CUDA events on the pricer's stream, best of `reps`), options/s and errors
    against the FP64 oracle priced here.
      uniform_1k   the 1,000-option book (latency-bound: one tiny tree per option)
      skewed_100k  1% heavy trees (up to 3,5xx nodes wide, 2,880 steps): per-block busy
                   time (tail imbalance) under the engine's binned persistent schedule,
                   under arrival order without binning ('i'), and with the one-block-per-
                   option plain kernel, the scheduler of the plain method"""
    wl = pkg.workloads
    out = {}

    def run(opts, mode, **cfg):
        best, st = 1e300, None
        for _ in range(reps):
            got = pricer.price(opts, y, mode, **cfg)
            s = pricer.last_stats
            if s.sizing_ms + s.pricing_ms < best:
                best, st = s.sizing_ms + s.pricing_ms, pkg.Stats.from_buffer_copy(s)
        return got, best, st

    # config 1
    book = pkg.Options.from_batch(wl.uniform_book())
    ref = orc.price(book, y, "f64")
    entry = {"options": book.N}
    for m in (pkg.BATCHED_MIXED, pkg.BATCHED_FP32, pkg.BATCHED_FP64, pkg.BATCHED_DF64, pkg.PLAIN_FP64):
        got, ms, st = run(book, m)
        entry[pkg.MODE_NAMES[m]] = {"device_ms": ms, "options_per_s": book.N / (ms * 1e-3),
                                    "call_ms_with_copies": st.total_ms, **errors(got, ref)}
    out["uniform_1k"] = entry
    # config 3
    sk = pkg.Options.from_batch(wl.skewed_batch())
    ref = orc.price(sk, y, "f64")
    entry = {"options": sk.N, "max_width": None, "max_height": None}
    for m in (pkg.BATCHED_FP64, pkg.BATCHED_MIXED, pkg.BATCHED_FP32, pkg.BATCHED_DF64):
        for sort in ("-", "i"):
            if sort == "i" and m not in (pkg.BATCHED_FP64, pkg.BATCHED_MIXED):
                continue
            got, ms, st = run(sk, m, sort=sort, record_busy=True)
            name = pkg.MODE_NAMES[m] + ("" if sort == "-" else "_arrival_order")
            entry[name] = {"device_ms": ms, "options_per_s": sk.N / (ms * 1e-3), "busy_max_ms": st.busy_max_ms,
                           "busy_mean_ms": st.busy_mean_ms, "tail": st.busy_max_ms / max(st.busy_mean_ms, 1e-12) - 1,
                           **errors(got, ref)}
            entry["max_width"], entry["max_height"] = st.max_width, st.max_height
    got, ms, st = run(sk, pkg.PLAIN_FP64)
    entry["plain_fp64_one_block_per_option"] = {"device_ms": ms, "options_per_s": sk.N / (ms * 1e-3),
                                                **errors(got, ref)}
    entry["note"] = ("tail = busiest pricing block / mean block busy time - 1; the reference's cuda-multi rejects "
                     "trees wider than 1,024 nodes (cuda-multi/Kernel.cuh:395-400), so it cannot price this batch")
    out["skewed_100k"] = entry
    return out


# FLOP per row of the surrogate network: 2 x (8 x 256 + 3 x 256 x 256 + 256 x 2); the
# tensor cores execute layer 1 twice (its input as a bf16 hi / lo pair): 4 x 256 x 256 MACs
NETWORK_FLOP_PER_ROW = 2 * (8 * 256 + 3 * 256 * 256 + 256 * 2)
NETWORK_TENSOR_FLOP_PER_ROW = 2 * 4 * 256 * 256


def network_kernel_time(pkg, pricer, rows: int, steps: int, warmup: int, dev) -> dict:
    """The fused network kernel alone on device-resident standardised features
    (random weights: its cost does not depend on them), CUDA-event time per launch,
    L2 flushed between launches."""
    import torch
    sur = pkg.Surrogate(pricer, seed=1)
    g = torch.Generator(device="cpu").manual_seed(0)
    x = torch.randn(rows, 8, generator=g, dtype=torch.float32)
    x[:, 7] = 0
    x = x.to(dev)
    out = torch.empty(rows, 2, dtype=torch.float32, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    for _ in range(warmup):
        sur.forward_device(x.data_ptr(), rows, out.data_ptr())
    ms = []
    for _ in range(steps):
        flush.zero_()
        torch.cuda.synchronize(dev)
        ms.append(sur.forward_device(x.data_ptr(), rows, out.data_ptr()))
    sur.close()
    t = sum(ms) / len(ms)
    measured = load_json(os.path.join(ROOT, "MEASURED_PEAKS.json")) or {}
    peak = measured.get("bf16_tflops")
    tensor_tflops = rows * NETWORK_TENSOR_FLOP_PER_ROW / (t * 1e-3) / 1e12
    return {"rows": rows, "kernel_ms": t, "rows_per_s": rows / (t * 1e-3),
            "tflops": rows * NETWORK_FLOP_PER_ROW / (t * 1e-3) / 1e12, "tensor_tflops_executed": tensor_tflops,
            "tensor_frac_of_bf16_peak": tensor_tflops / peak if peak else None,
            "flop_note": "tflops: the network's FLOP per row; tensor_tflops_executed: the MMAs the tensor cores "
                         "run (layer 1 twice)",
            "peak": f"bf16 burst {peak} TFLOP/s of measured (MEASURED_PEAKS.json)" if peak else None,
            "flop_per_row": NETWORK_FLOP_PER_ROW}


def surrogate_run(pkg, pricer, y, box, train, queries, epochs: int, reps: int, batch=None,
                  kink_oversample: int = 1) -> dict:
    """Trains the surrogate on `train` (labels from the FP64 tree), then prices the
    1M `queries` through hwt_surrogate_price (host arrays in and out; network inside
    the box unless routed, tree outside it, for routed options and for the judge's 1%
    sample), against the batched trees on the same queries.  Errors against the
    batched FP64 tree (itself within 1e-10 relative of the oracle)."""
    sur = pkg.Surrogate(pricer, box=box, seed=1)
    t0 = time.perf_counter()
    tstats = sur.train(pkg.Options.from_batch(train), y, epochs=epochs, batch=8192, lr=2e-3, lr_min=2e-6,
                       route_tolerance=1e-4, holdout=0.1, kink_oversample=kink_oversample)
    train_s = time.perf_counter() - t0
    qo = pkg.Options.from_batch(queries)
    trees = {}
    ref = None
    for m in (pkg.BATCHED_FP64, pkg.BATCHED_MIXED, pkg.BATCHED_FP32, pkg.PLAIN_FP64):
        best_dev, best_host = 1e300, 1e300
        for _ in range(reps if m != pkg.PLAIN_FP64 else 1):
            t0 = time.perf_counter()
            got = pricer.price(qo, y, m)
            best_host = min(best_host, time.perf_counter() - t0)
            best_dev = min(best_dev, pricer.last_stats.total_ms)
        if m == pkg.BATCHED_FP64:
            ref = got
        trees[pkg.MODE_NAMES[m]] = {"options_per_s": qo.N / best_host, "host_ms": 1e3 * best_host,
                                    "device_ms_with_copies": best_dev, **errors(got, ref)}
    inb = ~queries["outside"]
    mixed_rate = trees["batched_mixed"]["options_per_s"]
    # options/s at each judge tolerance: the routing calibrated on the held-out samples
    # for it, the judge enforcing it (answers above it send the network's answers to the tree)
    # Every call draws its own judge sample (seed), so a call can fall back where another
    # does not: options/s is the mean over the calls after the first (total options over
    # total wall time, fallbacks included), with the best call and the fallback count beside.
    at = {}
    calls = max(reps, 16)
    for tol in (1e-4, 2e-4, 5e-4, 1e-3):
        wall, sts, worst, worst_inb_p99 = [], [], 0.0, 0.0
        for k in range(calls + 1):
            t0 = time.perf_counter()
            got = sur.price(qo, y, judge_fraction=0.01, seed=7 + k, tree_mode=pkg.BATCHED_MIXED, judge_tolerance=tol)
            wall.append(time.perf_counter() - t0)
            sts.append(sur.stats.as_dict())
            err = np.abs(got - ref)
            worst = max(worst, float(np.max(err)))
            worst_inb_p99 = max(worst_inb_p99, float(np.percentile(err[inb], 99)))
        mean = sum(wall[1:]) / calls
        best = min(wall[1:])
        timed = sts[1:]
        st = timed[-1]
        at[f"{tol:g}"] = {
            "options_per_s": qo.N / mean, "host_ms": 1e3 * mean, "x_batched_mixed": (qo.N / mean) / mixed_rate,
            "x_plain_fp64": (qo.N / mean) / trees["plain_fp64"]["options_per_s"],
            "best_call_options_per_s": qo.N / best, "calls": calls,
            "calls_fell_back": sum(int(t["fell_back"]) for t in timed),
            "network_answered_min": min(t["n_network"] for t in timed),
            "network_answered_max": max(t["n_network"] for t in timed),
            "routed_in_box": st["n_flagged"], "outside_box": st["n_routed"],
            "route_tolerance": st["route_tolerance"],
            "judge_max_abs_over_calls": max(t["judge_max_abs"] for t in timed),
            "n_judged": st["n_judged"],
            "max_abs_err_over_calls": worst, "in_box_p99_abs_err_over_calls": worst_inb_p99,
            "device_ms_mean": {k: sum(t[k] for t in timed) / calls
                               for k in ("copy_ms", "network_ms", "tree_ms", "total_ms")}}
    on_batch = None
    if batch is not None:
        # the same network on a batch of its own box (the 30,000-option uneven batch)
        bopts, bref = batch
        on_batch = {}
        for name, tol in (("unjudged", 0.0), ("judged_1e-4", 1e-4)):
            wall = []
            for k in range(4):
                t0 = time.perf_counter()
                got = sur.price(bopts, y, judge_fraction=0.01, seed=100 + k, tree_mode=pkg.BATCHED_MIXED,
                                judge_tolerance=tol)
                wall.append(time.perf_counter() - t0)
            st = sur.stats.as_dict()
            e = {"options_per_s": bopts.N / min(wall[1:]), "fell_back_to_tree": bool(st["fell_back"]),
                 "network_answered": st["n_network"], "judge_max_abs": st["judge_max_abs"],
                 "n_judged": st["n_judged"]}
            if bref is not None:
                e.update(errors(got, bref))
            on_batch[name] = e
    sur.close()
    return {
        "on_uneven_30k": on_batch,
        "train": {**tstats, "wall_s": train_s, "epochs": epochs, "samples_offered": len(train["strike"]),
                  "kink_oversample": kink_oversample},
        "queries": {"n": int(qo.N), "outside_box": int(queries["outside"].sum()), "at_judge_tolerance": at,
                    "timing": "host clock around hwt_surrogate_price (host arrays in and out), mean of the calls "
                              "after the first, each with its own judge sample; trees: host clock around "
                              "hwt_price_ex on the same queries, best call; errors against the batched FP64 tree"},
        "trees": trees,
    }


def run_ours(args, rank, world, local):
    import torch
    import __graft_entry__ as g

    pkg = g.package()
    wl = pkg.workloads
    dist = init_dist(world, "nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    batch = wl.WORKLOADS[args.workload]()
    opts = pkg.Options.from_batch(batch)
    rates, days = wl.yield_curve()
    y = pkg.Yield(rates, days)
    n = opts.N
    shp = pkg.shape(opts)
    nodes = int(np.sum(pkg.active_nodes(shp["height"], shp["jmax"])))
    flop_per_batch = FLOP_PER_NODE * nodes

    pricer = pkg.Pricer(local)
    if args.network_rows:
        # the surrogate's fused network kernel alone (profiling runs)
        res = network_kernel_time(pkg, pricer, args.network_rows, args.steps, args.warmup, dev)
        if rank == 0:
            print(json.dumps({"network_kernel": res}))
        pricer.close()
        return 0
    mode = {"mixed": pkg.BATCHED_MIXED, "fp64": pkg.BATCHED_FP64, "fp32": pkg.BATCHED_FP32, "df64": pkg.BATCHED_DF64,
            "plain": pkg.PLAIN_FP64}[args.mode]
    # the library's autotuner (hwt_autotune) picks group size, warp-task width
    # threshold and K set for this batch, untimed, for every batched mode used below
    tuned = {}
    if not args.no_tune:
        for m in (pkg.BATCHED_MIXED, pkg.BATCHED_FP32, pkg.BATCHED_FP64, pkg.BATCHED_DF64):
            if m == mode or not args.skip_survey:
                c = pricer.autotune(opts, y, m, repeats=2)
                tuned[pkg.MODE_NAMES[m]] = {"block_size": c.block_size, "big_threshold": c.big_threshold,
                                            "warp_k_mask": c.warp_k_mask}

    # device-resident inputs
    fields = {"strike": opts.StrikePrices, "bond_maturity": opts.Maturities, "option_maturity": opts.Lengths,
              "term_unit": opts.TermUnits.view(np.int16), "term_steps": opts.TermStepCounts.view(np.int16),
              "a": opts.ReversionRates, "sigma": opts.Volatilities, "type": opts.Types}
    dev_t = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in fields.items()}
    dev_ptr = {k: t.data_ptr() for k, t in dev_t.items()}
    dev_out = torch.empty(n, dtype=torch.float64, device=dev)
    # pinned host inputs / outputs for the end-to-end path
    host_t = {k: torch.from_numpy(np.ascontiguousarray(v)).pin_memory() for k, v in fields.items()}
    host_ptr = {k: t.data_ptr() for k, t in host_t.items()}
    host_out = torch.empty(n, dtype=torch.float64).pin_memory()
    h2d_bytes = int(sum(t.numel() * t.element_size() for t in host_t.values()))
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def flush_l2():
        flush.zero_()
        torch.cuda.synchronize(dev)

    def device_steps(m, steps, warm):
        for _ in range(warm):
            pricer.price_device(dev_ptr, n, y, dev_out.data_ptr(), m)
        times, launches, stats, kernel = [], 0, None, []
        for _ in range(steps):
            flush_l2()
            st = pricer.price_device(dev_ptr, n, y, dev_out.data_ptr(), m)
            times.append(st.total_ms)
            kernel.append(st.pricing_ms)  # CUDA events around the pricing kernel, on its stream
            launches += st.kernel_launches
            stats = pkg.Stats.from_buffer_copy(st)
        stats.pricing_ms = sum(kernel) / len(kernel)
        return times, launches, stats

    # CPU baseline first (rank 0, N=1): also gives the FP64 reference prices
    cpu = None
    ref_prices = None
    if rank == 0 and world == 1 and not args.no_cpu:
        orc = g.oracle()
        orc.build()
        t0 = time.perf_counter()
        ref_prices = orc.price(opts, y, "f64")
        dt = time.perf_counter() - t0
        cpu = {"value": n / dt, "unit": "options/s", "cores": orc.max_threads(), "kind": "port",
               "sample": f"all {n} options of {args.workload}, one pass, OpenMP over options",
               "single_thread": single_thread_rate(orc, opts, y)}

    # per-mode survey (prices + errors + device time), untimed by the contract
    modes = {}
    for m in (() if args.skip_survey else (pkg.BATCHED_MIXED, pkg.BATCHED_FP32, pkg.BATCHED_FP64, pkg.BATCHED_DF64,
                                           pkg.PLAIN_FP64)):
        name = pkg.MODE_NAMES[m]
        k = args.steps if m != pkg.PLAIN_FP64 else max(1, min(args.steps, 3))
        t, _, st = device_steps(m, k, 1)
        entry = {"options_per_s": n / (sum(t) / len(t) / 1e3), "ms_per_step": sum(t) / len(t),
                 "pricing_ms": st.pricing_ms}
        if ref_prices is not None:
            got = dev_out.cpu().numpy()
            err = np.abs(got - ref_prices)
            entry.update({"max_abs_err": float(np.max(err)), "p99_abs_err": float(np.percentile(err, 99)),
                          "max_rel_err": float(np.max(err / np.maximum(np.abs(ref_prices), 1e-300)))})
        modes[name] = entry
    # the other configurations (the 1,000-option book, the skewed batch), untimed
    configs = None
    if modes and not args.no_configs and rank == 0:
        orc_c = g.oracle()
        orc_c.build()
        configs = config_runs(pkg, orc_c, pricer, y, reps=3)
    # learned surrogate: trained on tree prices, tree fallback outside its box and
    # tree judge on 1% of every batch: the single-tree box (samples drawn as the
    # 1,000-option book draws them) and the uneven batch's box
    surrogate = None
    if modes and not args.no_surrogate and rank == 0:
        surrogate = {"network_kernel": network_kernel_time(pkg, pricer, 1 << 20, 10, 3, dev)}
        surrogate["single_tree"] = surrogate_run(
            pkg, pricer, y, box=wl.single_tree_box(), train=wl.single_tree_training_batch(args.sur_samples, 3),
            queries=wl.single_tree_query_batch(1_000_000, 4), epochs=args.sur_epochs, reps=3, kink_oversample=3)
        surrogate["uneven_box"] = surrogate_run(
            pkg, pricer, y, box=None, train=wl.surrogate_training_batch(args.sur_samples, 3),
            queries=wl.surrogate_query_batch(1_000_000, 4), epochs=args.sur_epochs_uneven, reps=3,
            batch=(opts, ref_prices))
        # the judged surrogate at 1e-4 beside the trees (its own workload: 1M queries on
        # the single-tree box, 10% outside it)
        a = surrogate["single_tree"]["queries"]["at_judge_tolerance"]["0.0001"]
        modes["surrogate"] = {
            "workload": "single_tree_1m (4M training samples, 1M queries, 10% outside the box)",
            "judge_tolerance": 1e-4, "options_per_s": a["options_per_s"],
            "x_batched_mixed_same_queries": a["x_batched_mixed"], "calls": a["calls"],
            "calls_fell_back": a["calls_fell_back"], "max_abs_err_over_calls": a["max_abs_err_over_calls"],
            "judge_max_abs_over_calls": a["judge_max_abs_over_calls"]}
    # the reference's seven benchmark distributions (65,536 options each, data/yield.in
    # curve), device time per batch, beside the thesis's best CUDA numbers
    datasets = None
    if modes and not args.no_datasets:
        datasets = {}
        y15 = pkg.Yield.from_file(os.path.join(ROOT, "tests", "golden", "reference", "yield.in"))
        for k, name in enumerate(wl.THESIS_DATASETS):
            dopts = pkg.Options.from_batch(wl.thesis_dataset(k, 65536, seed=k))
            dsh = pkg.shape(dopts)
            entry = {"options": dopts.N,
                     "active_nodes_per_pass": int(np.sum(pkg.active_nodes(dsh["height"], dsh["jmax"])))}
            for m in (pkg.BATCHED_FP64, pkg.BATCHED_DF64, pkg.BATCHED_FP32, pkg.BATCHED_MIXED):
                best = 1e300
                for _ in range(3):
                    pricer.price(dopts, y15, m)
                    best = min(best, pricer.last_stats.total_ms)
                entry[pkg.MODE_NAMES[m] + "_options_per_s"] = dopts.N / (best * 1e-3)
            th = THESIS_BEST[name]
            entry["thesis_best_cuda_fp64_options_per_s"] = th[0]
            entry["thesis_best_cuda_fp32_options_per_s"] = th[1]
            datasets[name] = entry
    if modes:
        fp64_rate = modes["batched_fp64"]["options_per_s"]
        plain_rate = modes["plain_fp64"]["options_per_s"]
        for e in modes.values():
            if "workload" in e:
                continue  # measured on its own workload, against the trees on the same queries
            e["x_batched_fp64"] = e["options_per_s"] / fp64_rate
            e["x_plain_fp64"] = e["options_per_s"] / plain_rate

    # ---- sharded N > 1: each rank prices its LPT part of the batch, then the prices
    # are all-gathered (the step's only exchange); the whole job is one batch
    parts = shard_parts(pkg, opts, world) if (args.shard and world > 1) else None
    if parts is not None:
        mine = parts[rank]
        sub = opts.subset(mine)
        sub_dev = {k: torch.from_numpy(np.ascontiguousarray(v[mine])).to(dev) for k, v in fields.items()}
        sub_ptr = {k: t.data_ptr() for k, t in sub_dev.items()}
        sub_out = torch.empty(len(mine), dtype=torch.float64, device=dev)
        sub_host = {k: torch.from_numpy(np.ascontiguousarray(v[mine])).pin_memory() for k, v in fields.items()}
        sub_host_ptr = {k: t.data_ptr() for k, t in sub_host.items()}
        sub_host_out = torch.empty(len(mine), dtype=torch.float64).pin_memory()
        full_host = torch.empty(n, dtype=torch.float64).pin_memory()

        def shard_step():
            st_ = pricer.price_device(sub_ptr, len(mine), y, sub_out.data_ptr(), mode)
            gather_prices(sub_out, parts, dist, dev)
            torch.cuda.synchronize(dev)
            return st_

        def shard_step_host():
            pricer.price_host_ptrs(sub_host_ptr, len(mine), y, sub_host_out.data_ptr(), mode)
            full = gather_prices(sub_host_out.to(dev, non_blocking=True), parts, dist, dev)
            full_host.copy_(full)
            torch.cuda.synchronize(dev)

    # ---- timed region: K device-resident steps of the headline mode
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize(dev)
    # NVTX range "timed" marks the measured steps (ncu --nvtx --nvtx-include "timed/"
    # limits a launch list to them)
    nvtx = getattr(torch.cuda, "nvtx", None)
    if nvtx is not None:
        nvtx.range_push("timed")
    with ClockSampler(local) as clk:
        if parts is None:
            times, launches, st = device_steps(mode, args.steps, args.warmup)
        else:
            # host clock around price + all-gather (the pricer's call waits for its
            # stream, the gather is synchronised), L2 flushed between steps
            for _ in range(args.warmup):
                shard_step()
            times, launches, kernel = [], 0, []
            for _ in range(args.steps):
                flush_l2()
                t0 = time.perf_counter()
                st_ = shard_step()
                times.append(1e3 * (time.perf_counter() - t0))
                kernel.append(st_.pricing_ms)
                launches += st_.kernel_launches
            st = pkg.Stats.from_buffer_copy(st_)
            st.pricing_ms = sum(kernel) / len(kernel)
        torch.cuda.synchronize(dev)
        if dist is not None:
            dist.barrier()
        # e2e through the public host-memory API (pinned buffers), host clock
        for _ in range(args.warmup):
            if parts is None:
                pricer.price_host_ptrs(host_ptr, n, y, host_out.data_ptr(), mode)
            else:
                shard_step_host()
        e2e_t = []
        for _ in range(args.steps):
            flush_l2()
            t0 = time.perf_counter()
            if parts is None:
                pricer.price_host_ptrs(host_ptr, n, y, host_out.data_ptr(), mode)
            else:
                shard_step_host()
            e2e_t.append(time.perf_counter() - t0)
    if nvtx is not None:
        nvtx.range_pop()
    ms = sum(times) / len(times)
    ms = max_over_ranks(ms, dist, dev)
    e2e_ms = max_over_ranks(1e3 * sum(e2e_t) / len(e2e_t), dist, dev)
    pricing_ms = st.pricing_ms
    # options the whole job prices per step: replicas price the batch once per rank
    job_options = n if parts is not None else world * n

    peaks = pricer.measure_peaks()
    measured = load_json(os.path.join(ROOT, "MEASURED_PEAKS.json")) or {}
    fp32_peak = peaks[1]
    achieved = flop_per_batch / (pricing_ms * 1e-3) / 1e12
    prof = load_json(os.path.join(ROOT, "profiles", f"pricing_{args.workload}_{args.mode}.json")) or {}
    traffic = prof.get("dram_bytes_per_launch")
    bound = {"mixed": "fp32", "fp32": "fp32", "fp64": "fp64", "df64": "fp32", "plain": "fp64"}[args.mode]
    peak = fp32_peak if bound == "fp32" else peaks[0]

    if rank == 0:
        line = {
            "metric": METRIC,
            "value": job_options / (ms * 1e-3),
            "unit": "options/s",
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": ms,
            "higher_is_better": True,
            "scaling": "strong" if parts is not None else "weak",
            "vs_baseline": None,
            "dtype": {"mixed": "f32+f64", "fp32": "f32", "fp64": "f64", "df64": "f32x2+f64", "plain": "f64"}[args.mode],
            "data": "synthetic (seeded numpy; no public data set exists for this workload)",
            "config": {"workload": args.workload, "options": n},
            "engine": {"mode": pkg.MODE_NAMES[mode], "active_nodes_per_pass": nodes,
                       "parallelism": ("lpt shards + all-gather" if parts is not None else "replicas")
                       if world > 1 else "single",
                       "l2": "flushed between steps (256 MB memset), inputs 1.35 MB",
                       "block_size": st.block_size, "grid": st.grid,
                       "tuned": tuned.get(pkg.MODE_NAMES[mode], "library defaults")},
            "clocks": clk.summary(),
            "gpu_launches": launches,
            "e2e": {"value": job_options / (e2e_ms * 1e-3), "unit": "options/s",
                    "h2d_bytes_per_step": h2d_bytes if parts is None else
                    int(sum(t.numel() * t.element_size() for t in sub_host.values())) + 8 * len(mine),
                    "d2h_bytes_per_step": 8 * n if parts is None else 8 * len(mine) + 8 * n},
            "roofline": {"bound": bound, "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "work": f"{FLOP_PER_NODE} FLOP x {nodes} active nodes per launch; peak = FMA microbenchmark "
                                 f"on this GPU (MEASURED_PEAKS.json has no FP32/FP64 entries; its HBM figure is "
                                 f"{measured.get('hbm_gbs')} GB/s)",
                         "kernel_ms": pricing_ms},
            "peaks_measured": {"fp64_tflops": peaks[0], "fp32_tflops": peaks[1]},
            "modes": modes,
        }
        if modes and cpu is not None:
            # like-for-like multiples beside the headline (which sets mixed precision
            # on the GPU against the FP64 CPU pricer)
            line["like_for_like"] = {
                "batched_fp64_over_cpu_fp64": modes["batched_fp64"]["options_per_s"] / cpu["value"],
                "batched_df64_over_cpu_fp64": modes["batched_df64"]["options_per_s"] / cpu["value"],
                "mixed_over_batched_fp64": modes["batched_mixed"]["options_per_s"] / modes["batched_fp64"]["options_per_s"],
                "mixed_over_plain_fp64": modes["batched_mixed"]["options_per_s"] / modes["plain_fp64"]["options_per_s"],
                "note": "all on the same batch; cpu = the FP64 oracle on every host core, the whole batch"}
        if configs is not None:
            line["configs"] = configs
        if surrogate is not None:
            line["surrogate"] = surrogate
        if datasets is not None:
            line["thesis_datasets"] = {
                "note": "distributions of data-generator/RandomDataGenerator.cpp (seeded numpy draws, not the "
                        "reference's files); device time per batch (sizing + pricing, no transfers), best of 3; "
                        "thesis numbers: best CUDA kernel time on a GTX 780 Ti over versions, block sizes and sorts "
                        "(results/main/option.csv, multi.csv)",
                "sets": datasets}
        if cpu is not None:
            line["cpu_baseline"] = cpu
        print(json.dumps(line))
    pricer.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="uneven_30k", choices=sorted(WORKLOAD_NAMES))
    ap.add_argument("--mode", default="mixed", choices=["mixed", "fp64", "fp32", "df64", "plain"])
    ap.add_argument("--ref-sample", type=int, default=6000)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="library defaults instead of the autotuned configuration")
    ap.add_argument("--skip-survey", action="store_true", help="time only the headline mode (profiling runs)")
    ap.add_argument("--no-surrogate", action="store_true")
    ap.add_argument("--no-datasets", action="store_true", help="skip the seven thesis benchmark distributions")
    ap.add_argument("--no-configs", action="store_true", help="skip the 1,000-option book and the skewed batch")
    ap.add_argument("--network-rows", type=int, default=0,
                    help="time only the surrogate's fused network kernel on this many rows (profiling runs)")
    ap.add_argument("--sur-samples", type=int, default=4_000_000)
    ap.add_argument("--sur-epochs", type=int, default=800, help="surrogate epochs on the single-tree box")
    ap.add_argument("--sur-epochs-uneven", type=int, default=48, help="surrogate epochs on the uneven batch's box")
    ap.add_argument("--shard", action="store_true",
                    help="N>1: split the batch across ranks by tree work (LPT) and gather the prices, instead of "
                         "one replica of the whole batch per GPU")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    rank, world, local = dist_env()
    if args.gpus != world:
        # one process per GPU: N > 1 runs under torchrun, which sets WORLD_SIZE
        print(json.dumps({"error": f"--gpus {args.gpus} but WORLD_SIZE={world}: run N > 1 as "
                                   f"python -m torch.distributed.run --nproc-per-node {args.gpus} "
                                   f"--master-addr 127.0.0.1 bench.py --gpus {args.gpus} ..."}))
        return 2
    if args.impl == "reference":
        return cpu_reference(args, rank, world)
    return run_ours(args, rank, world, local)


if __name__ == "__main__":
    sys.exit(main())
