"""Multi-GPU is replicas only: each rank advances its own replica (own seeds)
with no data-path collective; the job time is the max over ranks.  This runs
the host logic of that path as two gloo ranks on CPU, each advancing a small
oracle replica."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import time

    import torch.distributed as dist

    import bench
    from oracle.oracle import Oracle
    from phafd_gb300 import workloads as W

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    cfg = bench.replica_cfg(dict(W.CONFIGS["32cube_64beads"], n=16, L=16.0, origin=-8.0, nchains=1,
                                 chain_len=10), rank)
    o = Oracle()
    W.apply(o, cfg)
    o.setup()
    t0 = time.perf_counter()
    o.run(3)
    ms = 1000 * (time.perf_counter() - t0) + 10.0 * rank  # rank 1 is the slow one
    ms_max = bench.max_over_ranks(ms, dist, "cpu")
    phi_sum = float(o.grid_get("phi").sum())
    out.put((rank, ms, ms_max, bench.job_throughput(world, 3, ms_max), phi_sum))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_run_independent_replicas():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, ms0, max0, v0, s0), (r1, ms1, max1, v1, s1) = res
    assert max0 == max1 == max(ms0, ms1)
    assert v0 == v1 == pytest.approx(2 * 3 / (max0 / 1000.0))
    assert s0 != s1  # different seeds: different replicas
