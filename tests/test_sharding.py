"""The multi-GPU path of bench.py on CPU: two gloo ranks shard the seed space
(weak scaling, no data-path collective), and the timing barrier and max/sum
reductions give the whole-job figures. The per-rank work is the oracle's
Stage0 on a few worlds, standing in for the GPU pipeline."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import sys
    import time
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank), BSF_DIST_BACKEND="gloo")
    import bench
    from oracle import pyoracle as po
    d = bench.Dist()
    start = bench.seed_start(20261203, d.rank, 0)
    seeds = np.arange(start, start + 4, dtype=np.int64)
    d.barrier()
    t0 = time.perf_counter()
    rec = po.stage0_batch(seeds, centers=8, profile=1, research=False)
    dt = time.perf_counter() - t0
    d.barrier()
    out.put((rank, start, dt, d.max(dt), d.sum(len(seeds)), bytes(rec[:32])))
    d.close()


def test_two_gloo_ranks_shard_seed_ranges_and_reduce_timings():
    from oracle import pyoracle as po
    po.build()
    ctx = torch.multiprocessing.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, s0, t0, m0, n0, b0), (r1, s1, t1, m1, n1, b1) = res
    assert (r0, r1) == (0, 1)
    assert abs(s0 - s1) >= 4                      # disjoint consecutive ranges
    assert m0 == m1 == max(t0, t1)                # whole-job time = slowest rank
    assert n0 == n1 == 8                          # units of all ranks
    assert b0 != b1                               # different worlds, different records
