"""bench.py's multi-GPU form, checked with two gloo ranks on the CPU.

The product needs no exchange between GPUs, so `bench.py --gpus N` runs N
independent replicas of the workload, one per GPU. The job's figures come
from the slowest rank (the maximum over ranks of the time per product) and
count every rank's products. This test runs that rank arithmetic with two
processes on the gloo backend; no GPU is involved."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import torch
    import torch.distributed as dist

    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        w, r, loc = bench.replica_layout()
        ms = 3.0 + 2.0 * rank  # rank 1 is the slow one
        slowest = bench.max_over_ranks(ms, dist, torch.device("cpu"))
        out.put((r, w, loc, slowest, bench.job_rate(w, slowest * 1e-3)))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")  # never fork a process that may hold a CUDA context
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[0] for r in results] == [0, 1] and all(r[1] == 2 for r in results)
    assert [r[2] for r in results] == [0, 1]
    for r in results:
        assert r[3] == 5.0  # the maximum over ranks, on every rank
        assert r[4] == pytest.approx(2 / 5e-3)  # two replicas' products per second


def test_single_process_defaults(monkeypatch):
    import bench
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    assert bench.replica_layout() == (1, 0, 0)
    assert bench.max_over_ranks(2.5, None, None) == 2.5
    assert bench.job_rate(1, 2e-3) == pytest.approx(500.0)
