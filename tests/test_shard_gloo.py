"""The exchange of a row-sharded product, with two gloo ranks on the CPU.

A sharded product (hmgpu.sharded) all-gathers x in the permuted source order
before every product, each rank contributing the slice it owns, and each rank
computes its own range of permuted rows of y (row ownership as in
src/mult.jl:144, so no reduction). This test runs the exchange code itself
(gather_slices, allgather_ranges) on two processes over gloo with uneven
slices; the rows each rank computes come from the oracle's CPU product (a
stand-in for the GPU shard here; tests/test_shard_gpu.py runs the shards).
The rows gathered from both ranks must equal the single-process product
bitwise."""
import os
import socket
import sys

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    for p in (REPO, os.path.join(REPO, "hmatrixgpu.jl_gb300")):
        if p not in sys.path:
            sys.path.insert(0, p)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch
    import torch.distributed as dist

    from hmgpu import sharded
    from oracle import oracle as O
    from tests import geometry
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        P = geometry.cube(1500, seed=4)
        T = O.Tree(P.T, 32)
        H = O.HMatrix(O.Kernel("laplace", P.T, P.T), T, T, eta=2.0, eps=1e-6)
        perm = H.source_index_map - 1          # permuted position -> original index
        tperm = H.target_index_map - 1
        n = H.n
        splits = [(0, 611), (611, n)]          # uneven, as tile boundaries make them
        ranges = sharded.allgather_ranges(splits[rank])
        assert ranges == splits
        x = np.random.default_rng(9).standard_normal(n)
        xp = x[perm]                            # the whole x in permuted order
        b, e = splits[rank]
        x_full = sharded.gather_slices(torch.tensor(xp[b:e]), splits).numpy()
        assert np.array_equal(x_full, xp)
        # this rank's rows of y, permuted order (the oracle stands in for the shard)
        y = np.empty(n)
        y[perm] = x_full                        # back to the original order
        yo = H.mul(y)[tperm]
        y_rows = torch.tensor(yo[b:e])
        y_all = sharded.gather_slices(y_rows, splits).numpy()
        out.put((rank, bool(np.array_equal(y_all, H.mul(x)[tperm]))))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_sharded_exchange_two_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")  # never fork a process that may hold a CUDA context
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=300) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == [(0, True), (1, True)]


def test_even_splits_cover_once():
    sys.path.insert(0, os.path.join(REPO, "hmatrixgpu.jl_gb300"))
    from hmgpu import sharded
    for n, w in ((10, 3), (7, 7), (1000, 8), (5, 1)):
        s = sharded.even_splits(n, w)
        assert s[0][0] == 0 and s[-1][1] == n
        assert all(a[1] == b[0] for a, b in zip(s, s[1:]))
