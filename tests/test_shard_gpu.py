"""Row shards (hmgpu_hmatrix_shard, hmgpu_matvec_shard) on the GPU.

Rows are owned as in the reference's product (src/mult.jl:144): each row of
the permuted output is written once, so shards split the rows with no
reduction. Every shard's rows must be bitwise the rows of the whole
H-matrix's product, the shards of one H-matrix must cover its rows once, and
two processes exchanging x over gloo (both on the one GPU here; their kernels
never wait on each other) must together give the single-process product."""
import os
import socket
import sys

import numpy as np
import pytest

import hmgpu
from oracle import oracle as O
from tests import geometry

pytestmark = pytest.mark.gpu
REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _full_perm(H, x):
    """The whole product H x in the permuted target order."""
    import torch
    tmap, _ = H.index_maps()
    return (H * x)[torch.tensor(tmap - 1, device=x.device)]


@pytest.mark.parametrize("precision", ["f64", "f32", "mixed"])
def test_shards_equal_whole_product(gpu, precision):
    import torch
    P = geometry.cube(6000, seed=3)
    T = hmgpu.ClusterTree(P, max_points_per_leaf=32)
    H = hmgpu.HMatrix(hmgpu.Kernel("laplace", P), T, T, eta=2.0, eps=1e-6, precision=precision)
    dt = torch.float64 if precision == "f64" else torch.float32
    x = torch.randn(H.shape[1], dtype=dt, device=gpu, generator=torch.Generator(gpu).manual_seed(2))
    _, smap = H.index_maps()
    xp = x[torch.tensor(smap - 1, device=gpu)].contiguous()
    ref = _full_perm(H, x)
    for world in (1, 2, 3, 5):
        shards = [H.shard(r, world) for r in range(world)]
        assert shards[0].rows[0] == 0 and shards[-1].rows[1] == H.shape[0]
        assert all(a.rows[1] == b.rows[0] for a, b in zip(shards, shards[1:]))
        for S in shards:
            b, e = S.rows
            y = torch.full((e - b,), float("nan"), dtype=dt, device=gpu)
            S.mul_permuted(y, xp)
            assert torch.equal(y, ref[b:e]), (world, b, e)
    with pytest.raises(hmgpu.HMGPUError, match="shard"):
        hmgpu.mul_(torch.empty(H.shape[0], dtype=dt, device=gpu), shards[0], x)


def test_shard_of_imported_matrix_matches_oracle(gpu):
    """Shards of the oracle's own H-matrix (imported through the reference's
    flattened layout) against the oracle's CPU mul! at 1e-12 in FP64; the
    parent is freed before the shards multiply."""
    import torch
    P = geometry.sphere(3000, seed=8)
    Ho = O.HMatrix(O.Kernel("laplace", P.T, P.T), O.Tree(P.T, 32), O.Tree(P.T, 32), eta=1.5, eps=1e-6,
                   nthreads=8)
    H = hmgpu.HMatrix.from_flat(Ho.m, Ho.n, Ho.target_index_map, Ho.source_index_map, Ho.dense_block_indices,
                                Ho.dense_blocks, Ho.U_block_indices, Ho.U_matrices, Ho.V_block_indices,
                                Ho.V_matrices, precision="f64")
    shards = [H.shard(r, 4) for r in range(4)]
    del H
    x = np.random.default_rng(5).standard_normal(Ho.n)
    yo = Ho.mul(x)[Ho.target_index_map - 1]
    xp = torch.tensor(x[Ho.source_index_map - 1], device=gpu)
    for S in shards:
        b, e = S.rows
        y = torch.empty(e - b, dtype=torch.float64, device=gpu)
        S.mul_permuted(y, xp)
        err = np.linalg.norm(y.cpu().numpy() - yo[b:e]) / max(np.linalg.norm(yo[b:e]), 1e-300)
        assert err <= 1e-12, (b, e, err)


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

    import hmgpu
    from hmgpu import sharded
    from tests import geometry
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        torch.cuda.set_device(0)
        dev = torch.device("cuda", 0)
        P = geometry.film(96, 80, seed=6)
        T = hmgpu.ClusterTree(P, max_points_per_leaf=64)
        H = hmgpu.HMatrix(hmgpu.Kernel("laplace", P), T, T, eta=2.0, eps=1e-5, precision="f64")
        prod = sharded.ShardedProduct(H)
        _, smap = H.index_maps()
        x = torch.tensor(np.random.default_rng(11).standard_normal(H.shape[1]), device=dev)
        xp = x[torch.tensor(smap - 1, device=dev)]
        b, e = prod.x_splits[rank]
        y_rows = prod.mul(xp[b:e].contiguous())
        torch.cuda.synchronize()
        y_all = sharded.gather_slices(y_rows.cpu(), prod.row_splits)
        ref = _full_perm(H, x).cpu()
        out.put((rank, bool(torch.equal(y_all, ref)), prod.row_splits))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_ranks_exchange_x_over_gloo(gpu):
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted((q.get(timeout=600) for _ in ps), key=lambda t: t[0])
    for p in ps:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [True, True]
    splits = res[0][2]
    assert splits[0][0] == 0 and splits[0][1] == splits[1][0] and 0 < splits[0][1] < splits[1][1]
