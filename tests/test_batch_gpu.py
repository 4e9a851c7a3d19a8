"""Batches of H-matrices (hmgpu_hmatrix_batch), CUDA-graph products and the
autotuner, on the GPU.

A batch is the block-diagonal operator diag(H_1, ..., H_k); its products must
equal the members' own products bit for bit, in every precision mode and for
one and many right-hand sides. Graph replays and autotuned products must
equal the plain products bit for bit too."""
import numpy as np
import pytest

import hmgpu
from tests import geometry

pytestmark = pytest.mark.gpu

MEMBERS = [  # points, kernel, leaf, eta, eps: sizes and kernels of a mixed batch
    (lambda: geometry.sphere(3000, seed=1), "yukawa", 32, 1.5, 1e-5),
    (lambda: geometry.cube(5000, seed=2), "laplace", 32, 2.0, 1e-5),
    (lambda: geometry.film(90, 70, seed=3), "laplace", 64, 2.0, 1e-4),
    (lambda: geometry.sphere(700, seed=4), "laplace", 16, 1.0, 1e-6),
]


def _members(precision):
    hs = []
    for pts_fn, kind, leaf, eta, eps in MEMBERS:
        P = pts_fn()
        T = hmgpu.ClusterTree(P, max_points_per_leaf=leaf)
        hs.append(hmgpu.HMatrix(hmgpu.Kernel(kind, P), T, T, eta=eta, eps=eps, precision=precision))
    return hs


@pytest.mark.parametrize("precision,nrhs", [("f64", 1), ("f32", 1), ("f32", 40), ("mixed", 1),
                                             ("mixed", 32), ("f64", 5)])
def test_batch_equals_members(gpu, precision, nrhs):
    import torch
    hs = _members(precision)
    B = hmgpu.batch(hs)
    m = sum(H.shape[0] for H in hs)
    n = sum(H.shape[1] for H in hs)
    assert B.shape == (m, n)
    assert B.info()["admissible_leaves"] == sum(H.info()["admissible_leaves"] for H in hs)
    dt = torch.float64 if precision == "f64" else torch.float32
    g = torch.Generator(device=gpu).manual_seed(nrhs)
    if nrhs == 1:
        x = torch.randn(n, device=gpu, dtype=dt, generator=g)
    else:
        x = torch.randn(nrhs, n, device=gpu, dtype=dt, generator=g).t()
    y = B * x
    r0 = c0 = 0
    for H in hs:
        mk, nk = H.shape
        xk = x[c0:c0 + nk] if nrhs == 1 else x[c0:c0 + nk].t().contiguous().t()
        yk = H * xk
        assert torch.equal(y[r0:r0 + mk], yk), (precision, nrhs, r0)
        r0 += mk
        c0 += nk
    assert B.status() == 0
    del hs  # the batch owns copies: it outlives its members
    torch.cuda.synchronize()
    assert torch.equal(B * x, y)


@pytest.mark.parametrize("nrhs", [32, 64])
def test_batch_nonfinite_member_stays_contained(gpu, nrhs):
    """An Inf or a NaN in one member's x reaches only that member's rows of y:
    the padding columns of every tensor-core tile read zeros, never a
    neighbouring member's x or t rows (0 * Inf would be NaN). The other
    members' rows stay finite and bitwise equal to their own products."""
    import torch
    hs = _members("mixed")
    B = hmgpu.batch(hs)
    n = sum(H.shape[1] for H in hs)
    g = torch.Generator(device=gpu).manual_seed(7)
    x = torch.randn(nrhs, n, device=gpu, generator=g).t()
    bad = 1  # member whose x gets non-finite entries
    c0 = sum(H.shape[1] for H in hs[:bad])
    x[c0 + 3, :] = float("inf")
    x[c0 + hs[bad].shape[1] - 1, :] = float("nan")
    y = B * x
    r0 = c0 = 0
    for k, H in enumerate(hs):
        mk, nk = H.shape
        if k != bad:
            yk = H * x[c0:c0 + nk].t().contiguous().t()
            assert torch.isfinite(y[r0:r0 + mk]).all(), k
            assert torch.equal(y[r0:r0 + mk], yk), k
        r0 += mk
        c0 += nk
    assert B.status() == 0


def test_batch_rejects_mixed_precisions(gpu):
    P = geometry.sphere(500, seed=5)
    T = hmgpu.ClusterTree(P, max_points_per_leaf=16)
    a = hmgpu.HMatrix(hmgpu.Kernel("laplace", P), T, T, eta=1.0, eps=1e-5, precision="f32")
    b = hmgpu.HMatrix(hmgpu.Kernel("laplace", P), T, T, eta=1.0, eps=1e-5, precision="f64")
    with pytest.raises(hmgpu.HMGPUError):
        hmgpu.batch([a, b])
    with pytest.raises(hmgpu.HMGPUError):
        hmgpu.batch([])


@pytest.mark.parametrize("precision,nrhs", [("f32", 1), ("mixed", 32), ("f64", 3)])
def test_graph_replay(gpu, precision, nrhs):
    import torch
    hs = _members(precision)
    H = hmgpu.batch(hs)
    m, n = H.shape
    dt = torch.float64 if precision == "f64" else torch.float32
    g = torch.Generator(device=gpu).manual_seed(11)
    shape = (n,) if nrhs == 1 else (nrhs, n)
    x = torch.randn(*shape, device=gpu, dtype=dt, generator=g)
    x = x if nrhs == 1 else x.t()
    y = torch.empty((m,) if nrhs == 1 else (nrhs, m), device=gpu, dtype=dt)
    y = y if nrhs == 1 else y.t()
    G = hmgpu.Graph(H, x, y)
    for k in range(3):
        x.copy_(torch.randn(*x.shape, device=gpu, dtype=dt, generator=g))
        G.launch()
        ref = H * x
        torch.cuda.synchronize()
        assert torch.equal(y, ref), k
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        x.mul_(-1.0)
        G.launch()
    s.synchronize()
    assert torch.equal(y, -ref)
    assert H.status() == 0


def test_autotune_keeps_results_and_caches(gpu, tmp_path):
    import torch
    hs = _members("f32")
    H = hmgpu.batch(hs)
    x = torch.randn(H.shape[1], device=gpu)
    y0 = H * x
    cache = tmp_path / "tune.txt"
    r = H.autotune(cache)
    assert r["unit_rows"] in (8, 16, 32, 64) and r["vunit_kib"] in (32, 64, 128)
    assert r["multi_rhs_from"] >= 2 and not r["from_cache"]
    assert torch.equal(H * x, y0)
    r2 = H.autotune(cache)
    assert r2["from_cache"] and {k: r2[k] for k in ("unit_rows", "vunit_kib", "multi_rhs_from")} == \
        {k: r[k] for k in ("unit_rows", "vunit_kib", "multi_rhs_from")}
    assert torch.equal(H * x, y0)
    assert "hmgpu-tune" in cache.read_text()
    X = torch.randn(6, H.shape[1], device=gpu).t()
    Y = H * X  # whichever path the threshold picks, the columns agree with single products
    for k in range(6):
        yk = H * X[:, k].contiguous()
        assert float((Y[:, k] - yk).norm() / yk.norm()) < 1e-5


def test_tuning_parameters_never_change_results(gpu):
    """Every combination of near/U unit rows, V unit size and V schedule (byte-
    balanced warp ranges or tickets) gives the same product bit for bit; bad
    values are rejected."""
    import torch
    P = geometry.cube(20000, seed=21)
    T = hmgpu.ClusterTree(P, max_points_per_leaf=32, gpu=True)
    H = hmgpu.HMatrix(hmgpu.Kernel("laplace", P), T, T, eta=2.0, eps=1e-6, precision="f32")
    x = torch.randn(P.shape[1], device=gpu)
    y0 = H * x
    for ur in (8, 16, 32, 64):
        for kib in (32, 64, 128):
            for vd in (0, 1):
                H.set_tuning(ur, kib, 3, vd)
                assert H.tuning() == {"unit_rows": ur, "vunit_kib": kib, "multi_rhs_from": 3, "v_dynamic": bool(vd)}
                assert torch.equal(H * x, y0), (ur, kib, vd)
    with pytest.raises(hmgpu.HMGPUError):
        H.set_tuning(12, 64, 3, 0)
    with pytest.raises(hmgpu.HMGPUError):
        H.set_tuning(16, 64, 3, 2)
    assert H.status() == 0
