"""The multi-process (replica) path of bench.py on CPU: two gloo ranks set up the
process group, meet at barriers, take the maximum step time over ranks and
aggregate the whole-job value; the reference arm runs on rank 0 only."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

from tests.conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, port, q):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": "2", "LOCAL_RANK": str(rank), "GH1_DIST_BACKEND": "gloo"})
    sys.path.insert(0, ROOT)
    import bench
    ws, r, local = bench.dist_setup(2)
    bench.barrier(ws)
    tmax = bench.max_over_ranks(0.5 + rank, ws)        # rank 1 is the slower one
    value = bench.replica_value(1e9, 0.5 + rank, ws)    # 2 ranks x 1e9 units / 1.5 s
    # the reference arm: only rank 0 does work (rank 1 returns before any)
    ran = None
    if r != 0:
        class A:
            gpus, steps, warmup, nx, order = 2, 1, 0, 4, 1
        ran = bench.run_reference(A, ws, r)
    bench.barrier(ws)
    import torch.distributed as dist
    dist.destroy_process_group()
    q.put((r, ws, local, tmax, value, ran))


def test_two_gloo_replicas():
    pytest.importorskip("torch.distributed")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r, (rank, ws, local, tmax, value, ran) in enumerate(res):
        assert rank == r and ws == 2 and local == r
        assert tmax == 1.5
        assert abs(value - 2.0 / 1.5) < 1e-12
        assert ran is None
