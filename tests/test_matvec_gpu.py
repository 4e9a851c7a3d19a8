"""Product parity on the GPU: H-matrices assembled by the oracle, imported in the
reference's flattened layout through the C ABI, multiplied by the CUDA kernels
and compared with the oracle's CPU mul! (src/mult.jl:6-32) on the same matrix.

Tolerances (relative 2-norm against the FP64 oracle): FP64 mode 1e-12, FP32
mode 1e-5 (the reference's correctness targets for this path)."""
import numpy as np
import pytest

import hmgpu
from oracle import oracle as O
from tests import geometry

pytestmark = pytest.mark.gpu


def _flat(H):
    return dict(m=H.m, n=H.n, target_index_map=H.target_index_map,
                source_index_map=H.source_index_map, dense_block_indices=H.dense_block_indices,
                dense_blocks=H.dense_blocks, U_block_indices=H.U_block_indices,
                U_matrices=H.U_matrices, V_block_indices=H.V_block_indices, V_matrices=H.V_matrices)


def _cases():
    c = geometry.circle(1000)
    yield "circle_log2d", O.Kernel("log2d", c.T, c.T), O.Tree(c.T, 64), O.Tree(c.T, 64), 1.5, 1e-6
    yield "circle_vector", O.Kernel("vector_r", c.T, c.T), O.Tree(c.T, 64), O.Tree(c.T, 64, 3), 1.5, 1e-6
    p = geometry.cube(4096, seed=0)
    yield "cube4096_laplace", O.Kernel("laplace", p.T, p.T), O.Tree(p.T, 32), O.Tree(p.T, 32), 2.0, 1e-6
    s = geometry.sphere(3000, seed=2)
    yield "sphere_yukawa", O.Kernel("yukawa", s.T, s.T), O.Tree(s.T, 16), O.Tree(s.T, 16), 1.0, 1e-5
    f = geometry.film(48, 40)
    yield "film_laplace", O.Kernel("laplace", f.T, f.T), O.Tree(f.T, 64), O.Tree(f.T, 64), 2.0, 1e-4
    # leaves of up to 200 points: row tiles of more than 64 rows
    b = geometry.cube(6000, seed=3)
    yield "cube_bigleaf_laplace", O.Kernel("laplace", b.T, b.T), O.Tree(b.T, 200), O.Tree(b.T, 200), 1.5, 1e-5
    # wide source groups: the multi-RHS V pass cuts them into column pieces
    # whose partial products are summed afterwards
    w = geometry.film(200, 160)
    yield "film_wide_laplace", O.Kernel("laplace", w.T, w.T), O.Tree(w.T, 64), O.Tree(w.T, 64), 2.0, 1e-4
    # rectangular: 3000 targets in a cube, 2000 sources on a sphere beside it
    tx, sy = geometry.cube(3000, seed=4), geometry.sphere(2000, seed=5) * 0.6 + np.array([[2.0], [0.3], [0.1]])
    yield "rect_cube_sphere", O.Kernel("laplace", tx.T, sy.T), O.Tree(tx.T, 32), O.Tree(sy.T, 32), 1.5, 1e-6
    # no admissible block at all (eta 1e9): an empty far field, dense blocks only
    d = geometry.cube(300, seed=6)
    yield "all_dense", O.Kernel("laplace", d.T, d.T), O.Tree(d.T, 16), O.Tree(d.T, 16), 1e9, 1e-6


CASES = {c[0]: c[1:] for c in _cases()}


@pytest.fixture(scope="module", params=sorted(CASES))
def case(request):
    K, X, Y, eta, eps = CASES[request.param]
    H = O.HMatrix(K, X, Y, eta=eta, eps=eps, nthreads=8)
    return request.param, K, H


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))


def test_f64_matches_oracle(case, gpu):
    import torch
    name, K, Ho = case
    H = hmgpu.HMatrix.from_flat(**_flat(Ho), precision="f64")
    assert H.shape == (Ho.m, Ho.n)
    rng = np.random.default_rng(1)
    for _ in range(2):
        x = rng.standard_normal(Ho.n)
        y_ref = Ho.mul(x)
        y = H * torch.tensor(x, device=gpu)
        assert rel(y.cpu().numpy(), y_ref) <= 1e-12, name
        yh = H * x  # host buffers
        assert rel(yh, y_ref) <= 1e-12


def test_f32_matches_oracle(case, gpu):
    import torch
    name, K, Ho = case
    for comp in (False, True):
        H = hmgpu.HMatrix.from_flat(**_flat(Ho), precision="f32", compensated=comp)
        x = np.random.default_rng(2).standard_normal(Ho.n)
        y_ref = Ho.mul(x.astype(np.float32).astype(np.float64))
        y = H * torch.tensor(x, dtype=torch.float32, device=gpu)
        assert rel(y.cpu().numpy(), y_ref) <= 1e-5, (name, comp)


def test_deterministic_and_overwrite(case, gpu):
    import torch
    _, _, Ho = case
    H = hmgpu.HMatrix.from_flat(**_flat(Ho), precision="f32")
    x = torch.randn(Ho.n, device=gpu)
    y1 = torch.full((Ho.m,), float("nan"), device=gpu)
    hmgpu.mul_(y1, H, x)
    y2 = torch.zeros(Ho.m, device=gpu)
    hmgpu.mul_(y2, H, x)
    assert torch.equal(y1, y2)  # bitwise: fixed summation order, y overwritten


def test_multiple_rhs(case, gpu):
    import torch
    _, _, Ho = case
    H = hmgpu.HMatrix.from_flat(**_flat(Ho), precision="f64")
    X = np.random.default_rng(3).standard_normal((Ho.n, 3))
    Y = H * torch.tensor(X, device=gpu).t().contiguous().t()
    ref = np.stack([Ho.mul(X[:, k]) for k in range(3)], 1)
    assert rel(Y.cpu().numpy(), ref) <= 1e-12


def test_import_rejects_bad_tables(gpu):
    c = geometry.circle(300)
    Ho = O.HMatrix(O.Kernel("log2d", c.T, c.T), O.Tree(c.T, 32), O.Tree(c.T, 32), eta=1.5, eps=1e-6)
    f = _flat(Ho)
    bad = dict(f, target_index_map=np.ones(Ho.m, np.int64))
    with pytest.raises(hmgpu.HMGPUError, match="permutation"):
        hmgpu.HMatrix.from_flat(**bad)
    di = f["dense_block_indices"].copy()
    di[0, 1] = Ho.m + 5
    with pytest.raises(hmgpu.HMGPUError, match="invalid range"):
        hmgpu.HMatrix.from_flat(**dict(f, dense_block_indices=di))
    vi = f["V_block_indices"].copy()
    vi[0, 2] += 1
    with pytest.raises(hmgpu.HMGPUError, match="inconsistent|out of range"):
        hmgpu.HMatrix.from_flat(**dict(f, V_block_indices=vi))


@pytest.mark.parametrize("prec,tol", [("f64", 1e-12), ("f32", 1e-5)])
def test_many_rhs_two_passes(case, gpu, prec, tol):
    """40 right-hand sides: one 32-wide pass and one 8-wide pass of the multi-RHS kernels."""
    import torch
    _, _, Ho = case
    H = hmgpu.HMatrix.from_flat(**_flat(Ho), precision=prec)
    X = np.random.default_rng(7).standard_normal((Ho.n, 40))
    dt = torch.float64 if prec == "f64" else torch.float32
    Xd = torch.tensor(X, dtype=dt, device=gpu).t().contiguous().t()
    Y = (H * Xd).double().cpu().numpy()
    Xr = X.astype(np.float32).astype(np.float64) if prec == "f32" else X
    ref = np.stack([Ho.mul(Xr[:, k]) for k in range(40)], 1)
    for k in range(40):
        assert rel(Y[:, k], ref[:, k]) <= tol, k
    # a single column of the batch equals the single-RHS product up to rounding
    y0 = (H * Xd[:, 0].contiguous()).double().cpu().numpy()
    assert rel(Y[:, 0], y0) <= tol


@pytest.mark.parametrize("prec,tol", [("f64", 1e-12), ("f32", 1e-5)])
def test_pass_widths(case, gpu, prec, tol):
    """Passes 8, 16 and 32 wide (chosen by the column count), in alternating
    order on one H-matrix, each column against the oracle's product."""
    import torch
    _, _, Ho = case
    H = hmgpu.HMatrix.from_flat(**_flat(Ho), precision=prec)
    dt = torch.float64 if prec == "f64" else torch.float32
    rng = np.random.default_rng(17)
    for nrhs in (8, 30, 3, 16, 9, 17, 8, 32, 12):
        X = rng.standard_normal((Ho.n, nrhs))
        Xd = torch.tensor(X, dtype=dt, device=gpu).t().contiguous().t()
        Y = (H * Xd).double().cpu().numpy()
        Xr = X.astype(np.float32).astype(np.float64) if prec == "f32" else X
        for k in range(nrhs):
            assert rel(Y[:, k], Ho.mul(Xr[:, k])) <= tol, (nrhs, k)
    assert H.status() == 0


def test_device_status_clean(case, gpu):
    """No bounded device wait expires in a product, plain or compensated."""
    import ctypes as C
    import torch
    _, _, Ho = case
    for comp in (False, True):
        H = hmgpu.HMatrix.from_flat(**_flat(Ho), precision="f32", compensated=comp)
        x = torch.arange(Ho.n, device=gpu, dtype=torch.float32).sin()
        y = H * x
        st = C.c_int(-1)
        assert hmgpu._lib.lib().hmgpu_hmatrix_status(H._h, C.byref(st)) == 0 and st.value == 0
        assert torch.isfinite(y).all()


def test_mixed_tensor_core_many_rhs(case, gpu):
    """HMGPU_MIXED with 32+ right-hand sides runs on the tensor cores (scaled
    FP16 hi/lo pairs, FP32 accumulation). Its error against the FP64 product
    of the same H-matrix is held to twice the plain FP32 form's (each column
    against its own oracle product), with a floor of 1e-6."""
    import ctypes as C
    import torch
    _, _, Ho = case
    H = hmgpu.HMatrix.from_flat(**_flat(Ho), precision="mixed")
    H32 = hmgpu.HMatrix.from_flat(**_flat(Ho), precision="f32")
    # 32: one 32-wide pass; 40, 64: one 64-wide pass; 70: a 64-wide and a 32-wide pass
    for nr in (32, 40, 64, 70, 3):
        X = np.random.default_rng(nr).standard_normal((Ho.n, nr))
        Xd = torch.tensor(X, dtype=torch.float32, device=gpu).t().contiguous().t()
        Y = (H * Xd).double().cpu().numpy()
        Y32 = np.stack([(H32 * Xd[:, k].contiguous()).double().cpu().numpy() for k in range(nr)], 1)
        Xr = X.astype(np.float32).astype(np.float64)
        ref = np.stack([Ho.mul(Xr[:, k]) for k in range(nr)], 1)
        err = max(rel(Y[:, k], ref[:, k]) for k in range(nr))
        err32 = max(rel(Y32[:, k], ref[:, k]) for k in range(nr))
        assert err <= max(2.0 * err32, 1e-6), (nr, err, err32)
    st = C.c_int(-1)
    assert hmgpu._lib.lib().hmgpu_hmatrix_status(H._h, C.byref(st)) == 0 and st.value == 0


def test_mixed_scales_follow_the_data(case, gpu):
    """The FP16 pairs carry power-of-two scales per right-hand side, per panel
    row and per rank row, so the product is invariant to the magnitude of x
    and of each column of X: columns of 1e-30, 1 and 1e30 (and a zero column)
    give the same relative error as unscaled ones, and scaling a column by a
    power of two scales its product exactly."""
    import torch
    _, _, Ho = case
    H = hmgpu.HMatrix.from_flat(**_flat(Ho), precision="mixed")
    rng = np.random.default_rng(23)
    X = rng.standard_normal((Ho.n, 32)).astype(np.float32)
    X[:, 1] = 0.0
    scale = np.ones(32, np.float32)
    scale[2], scale[3], scale[4] = 1e-30, 1e30, 2.0 ** 40
    Xs = X * scale
    Xd = torch.tensor(Xs, device=gpu).t().contiguous().t()
    Y = (H * Xd).double().cpu().numpy()
    assert np.all(Y[:, 1] == 0.0)
    for k in (0, 2, 3, 4, 5):
        ref = Ho.mul(Xs[:, k].astype(np.float64))
        assert rel(Y[:, k], ref) <= 1e-5, k
    # a power-of-two column scale passes through exactly
    Xd2 = torch.tensor(X, device=gpu).t().contiguous().t()
    Y2 = (H * Xd2).double().cpu().numpy()
    assert np.array_equal(Y[:, 4], Y2[:, 4] * 2.0 ** 40)
    assert H.status() == 0
