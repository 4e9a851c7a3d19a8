"""hmgpu_matvec_noalloc: the product for callers that cannot allocate device
memory while it runs (graph capture without allocation, fixed-footprint loops,
hosts whose allocator belongs to another framework). Its scratch is a static
device array of HMGPU_NOALLOC_SCRATCH_BYTES shared by every call, so this file
is collected last and checks two calls in a row against hmgpu_matvec and
against the oracle's CPU product."""
import ctypes as C

import numpy as np
import pytest

import hmgpu
from hmgpu import _lib
from oracle import oracle as O
from tests import geometry

pytestmark = pytest.mark.gpu


def _noalloc(H, x, y, stream):
    return _lib.lib().hmgpu_matvec_noalloc(H._h, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()),
                                           C.c_void_p(stream))


@pytest.mark.parametrize("precision,tol", [("f32", 1e-5), ("f64", 1e-12)])
def test_noalloc_matches_matvec_twice(gpu, precision, tol):
    import torch
    P = geometry.cube(4096, seed=0)
    T = hmgpu.ClusterTree(P, max_points_per_leaf=32)
    H = hmgpu.HMatrix(hmgpu.Kernel("laplace", P), T, T, eta=2.0, eps=1e-6, precision=precision)
    dt = torch.float32 if precision == "f32" else torch.float64
    stream = torch.cuda.current_stream(gpu).cuda_stream
    g = torch.Generator(gpu).manual_seed(3)
    for _ in range(2):  # the second call starts from the first call's leftovers
        x = torch.randn(4096, dtype=dt, device=gpu, generator=g)
        y_ref = torch.empty(4096, dtype=dt, device=gpu)
        hmgpu.mul_(y_ref, H, x)
        y = torch.full((4096,), float("nan"), dtype=dt, device=gpu)
        assert _noalloc(H, x, y, stream) == 0, _lib.lib().hmgpu_last_error()
        torch.cuda.synchronize()
        err = float(torch.linalg.norm((y - y_ref).double()) / torch.linalg.norm(y_ref.double()))
        assert err <= tol


def test_noalloc_matches_oracle_mul(gpu):
    """The oracle's own H-matrix (imported through the reference's flattened
    layout) multiplied by hmgpu_matvec_noalloc, twice, against the oracle's CPU
    mul! (src/mult.jl:6-32) on the same matrix: 1e-12 in FP64."""
    import torch
    P = geometry.cube(4096, seed=0)
    Ho = O.HMatrix(O.Kernel("laplace", P.T, P.T), O.Tree(P.T, 32), O.Tree(P.T, 32), eta=2.0, eps=1e-6,
                   nthreads=8)
    H = hmgpu.HMatrix.from_flat(Ho.m, Ho.n, Ho.target_index_map, Ho.source_index_map,
                                Ho.dense_block_indices, Ho.dense_blocks, Ho.U_block_indices, Ho.U_matrices,
                                Ho.V_block_indices, Ho.V_matrices, precision="f64")
    stream = torch.cuda.current_stream(gpu).cuda_stream
    rng = np.random.default_rng(17)
    for _ in range(2):
        x = rng.standard_normal(Ho.n)
        xd = torch.tensor(x, device=gpu)
        y = torch.full((Ho.m,), float("nan"), dtype=torch.float64, device=gpu)
        assert _noalloc(H, xd, y, stream) == 0, _lib.lib().hmgpu_last_error()
        torch.cuda.synchronize()
        yo = Ho.mul(x)
        assert np.linalg.norm(y.cpu().numpy() - yo) / np.linalg.norm(yo) <= 1e-12


def test_noalloc_rejects_oversized_matrix(gpu):
    import torch
    n = (32 << 20) // 4 + 1000  # the permuted x alone overflows the 32 MiB scratch in FP32
    Hf = hmgpu.HMatrix.from_flat(1, n, np.array([1]), np.arange(1, n + 1),
                                 np.array([[1, 1, 1, n, 0]]), np.full(n, 0.5),
                                 np.zeros((0, 5), np.int64), np.zeros(0), np.zeros((0, 3), np.int64),
                                 np.zeros(0), precision="f32")
    x = torch.ones(n, device=gpu)
    y = torch.empty(1, device=gpu)
    rc = _noalloc(Hf, x, y, torch.cuda.current_stream(gpu).cuda_stream)
    assert rc == -1  # HMGPU_ERR_INVALID
    assert b"scratch" in _lib.lib().hmgpu_last_error()
    hmgpu.mul_(y, Hf, x)  # the allocating entry point still serves it
    assert abs(float(y.item()) - 0.5 * n) <= 1e-5 * 0.5 * n
