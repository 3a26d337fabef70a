"""N>1 host logic of bench.py on CPU: two gloo ranks (127.0.0.1).  The pricer
runs as independent replicas per GPU (options are independent; no collective on
the data path); the only cross-rank steps are the barrier, the max-over-ranks of
the step time and, when a batch is sharded instead of replicated (bench.py
--shard), the LPT split of options by work and the all-gather of the shards'
prices."""
import os
import socket
import sys

import numpy as np
import pytest
import torch.multiprocessing as mp

from conftest import ROOT


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench
    dist = bench.init_dist(world, "gloo")
    t = bench.max_over_ranks(1.0 + rank, dist)
    work = np.random.default_rng(5).integers(1, 10_000, 1000).astype(np.float64)
    parts = bench.shard_lpt(work, world)
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, t, [p.tolist() for p in parts]))


def test_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    assert res[0][1] == res[1][1] == 2.0           # max over ranks
    assert res[0][2] == res[1][2]                  # every rank computes the same split
    parts = [np.array(p) for p in res[0][2]]
    allidx = np.sort(np.concatenate(parts))
    assert np.array_equal(allidx, np.arange(1000))
    work = np.random.default_rng(5).integers(1, 10_000, 1000).astype(np.float64)
    loads = [work[p].sum() for p in parts]
    assert max(loads) / min(loads) < 1.01


def test_lpt_single_rank():
    sys.path.insert(0, ROOT)
    import bench
    parts = bench.shard_lpt(np.array([5.0, 1.0, 3.0]), 1)
    assert [p.tolist() for p in parts] == [[0, 1, 2]]


def _shard_worker(rank, world, port, q):
    """One rank of the sharded path with the oracle (CPU) standing in for the GPU
    pricer: price this rank's LPT part, all-gather, return the full price array."""
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch
    import bench
    import __graft_entry__ as g
    pkg, orc = g.package(), g.oracle()
    wl = pkg.workloads
    opts = pkg.Options.from_batch({k: v[:1500] for k, v in wl.uneven_batch().items()})
    rates, days = wl.yield_curve()
    y = pkg.Yield(rates, days)
    dist = bench.init_dist(world, "gloo")
    parts = bench.shard_parts(pkg, opts, world)
    local = torch.from_numpy(orc.price(opts.subset(parts[rank]), y, "f64", threads=1))
    full = bench.gather_prices(local, parts, dist)
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, full.numpy().tobytes(), [len(p) for p in parts]))


def test_sharded_prices_equal_one_rank_bitwise():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_shard_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    import __graft_entry__ as g
    pkg, orc = g.package(), g.oracle()
    wl = pkg.workloads
    opts = pkg.Options.from_batch({k: v[:1500] for k, v in wl.uneven_batch().items()})
    rates, days = wl.yield_curve()
    one = orc.price(opts, pkg.Yield(rates, days), "f64", threads=1)
    assert all(min(sizes) > 0 for _, _, sizes in res)
    for _, blob, _ in res:  # every rank holds the whole batch's prices, in input order
        assert np.frombuffer(blob, dtype=np.float64).tobytes() == one.tobytes()


def test_bench_refuses_gpus_without_ranks():
    """--gpus N > 1 without torchrun's WORLD_SIZE would silently time one GPU."""
    import subprocess
    env = {k: v for k, v in os.environ.items() if k not in ("WORLD_SIZE", "RANK", "LOCAL_RANK")}
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--gpus", "2"], capture_output=True,
                       text=True, env=env, timeout=120)
    assert r.returncode == 2 and "WORLD_SIZE" in r.stdout
