"""User kernels on the device: a matrix K[i, j] = f(x_i, y_j) whose entry
function the caller writes (the reference builds an HMatrix from any K it can
index, src/hmatrix.jl:183,195-196).

  * Laplace written as a user kernel, with the built-in kernel's arithmetic,
    gives the oracle's H-matrix: the same partition, every rank and every
    recompressed factor bitwise, products at 1e-12 (FP64);
  * a Gaussian with its width as a parameter: H x against the dense K x at the
    tolerance (the reference's test: isapprox(K*x, H*x)), in FP64 and FP32;
  * sparsify_hmatrix of a user kernel equals the built-in kernel's triplets."""
import numpy as np
import pytest

import hmgpu
from tests import geometry
from tests.test_build_gpu import _oracle_h, rel
from tests.test_user_kernel import LAPLACE

pytestmark = pytest.mark.gpu

GAUSS = """__device__ double hmgpu_entry(const double *x, const double *y, const double *p, int a, int b) {
  double dx = x[0] - y[0], dy = x[1] - y[1], dz = x[2] - y[2];
  return exp(-(dx * dx + dy * dy + dz * dz) / (2.0 * p[0] * p[0]));
}
"""


def test_user_laplace_is_the_oracles_hmatrix(gpu):
    import torch
    P = geometry.cube(4096, seed=0)
    _, Ho = _oracle_h("laplace", P, 32, 2.0, 1e-6)
    T = hmgpu.ClusterTree(P, max_points_per_leaf=32)
    H = hmgpu.HMatrix(hmgpu.Kernel("user", P, user=LAPLACE), T, T, eta=2.0, eps=1e-6, precision="f64",
                      keep_factors=True)
    d, a = H.blocks()
    np.testing.assert_array_equal(d, Ho.dense_block_indices[:, :4])
    np.testing.assert_array_equal(a[:, :2], Ho.U_block_indices[:, :2])
    np.testing.assert_array_equal(a[:, 4], Ho.U_block_indices[:, 3] - Ho.U_block_indices[:, 2] + 1)
    for b in range(0, len(a), 5):
        U, V = H.block_factors(b)
        uo = Ho.U_block_indices[b, 4]
        vo = Ho.V_block_indices[Ho.U_block_indices[b, 2] - 1, 2] if a[b, 4] else 0
        np.testing.assert_array_equal(U, Ho.U_matrices[uo:uo + U.size].reshape(U.shape))
        np.testing.assert_array_equal(V, Ho.V_matrices[vo:vo + V.size].reshape(V.shape))
    x = np.random.default_rng(1).standard_normal(Ho.n)
    assert rel((H * torch.tensor(x, device=gpu)).cpu().numpy(), Ho.mul(x)) <= 1e-12
    # and bitwise the built-in kernel's H-matrix
    Hb = hmgpu.HMatrix(hmgpu.Kernel("laplace", P), T, T, eta=2.0, eps=1e-6, precision="f64")
    xt = torch.tensor(x, device=gpu)
    assert torch.equal(H * xt, Hb * xt)


@pytest.mark.parametrize("precision,tol", [("f64", 1e-6), ("f32", 1e-5)])
def test_user_gaussian_with_a_parameter(gpu, precision, tol):
    import torch
    P = geometry.sphere(3000, seed=4)
    s = 0.3
    T = hmgpu.ClusterTree(P, max_points_per_leaf=32)
    uk = hmgpu.UserKernel(GAUSS)
    H = hmgpu.HMatrix(hmgpu.Kernel("user", P, user=uk, params=[s]), T, T, eta=1.5, eps=1e-6, precision=precision)
    info = H.info()
    assert info["admissible_leaves"] > 0 and info["compression_ratio"] > 1.5, info
    d2 = ((P[:, :, None] - P[:, None, :]) ** 2).sum(axis=0)
    K = np.exp(-d2 / (2 * s * s))
    x = np.random.default_rng(2).standard_normal(P.shape[1])
    dt = torch.float64 if precision == "f64" else torch.float32
    y = (H * torch.tensor(x, dtype=dt, device=gpu)).double().cpu().numpy()
    assert rel(y, K @ x) <= tol
    # another width through the same compiled function: a different matrix
    H2 = hmgpu.HMatrix(hmgpu.Kernel("user", P, user=uk, params=[0.1]), T, T, eta=1.5, eps=1e-6, precision="f64")
    y2 = (H2 * torch.tensor(x, device=gpu)).cpu().numpy()
    assert rel(y2, np.exp(-d2 / (2 * 0.01)) @ x) <= 1e-6


def test_user_sparsify_equals_builtin(gpu):
    P = geometry.cube(1200, seed=3)
    X = hmgpu.ClusterTree(P, max_points_per_leaf=32)
    I, J, V = hmgpu.sparsify_hmatrix(hmgpu.Kernel("user", P, user=LAPLACE), X, X, eta=2.0, triplets=True)
    Ib, Jb, Vb = hmgpu.sparsify_hmatrix(hmgpu.Kernel("laplace", P), X, X, eta=2.0, triplets=True)
    assert np.array_equal(I, Ib) and np.array_equal(J, Jb) and np.array_equal(V, Vb)


def test_bad_user_kernel_arguments(gpu):
    P = geometry.cube(500, seed=1)
    T = hmgpu.ClusterTree(P, max_points_per_leaf=32)
    K = hmgpu.Kernel("user", P, user=GAUSS, params=np.ones(65))
    with pytest.raises(hmgpu.HMGPUError, match="parameters"):
        hmgpu.HMatrix(K, T, T, eta=1.5, eps=1e-6)


# the demagnetising tensor of the reference's example (examples/hmatrix_vector.jl:12-80),
# written as a user kernel with the built-in kernel's operation order
DIPOLAR = """
__device__ double dxx(double x, double y, double z) {
  double R = x * x + y * y + z * z;
  if (R == 0.0) return 0.0;
  double num = 2.0 * x * x - y * y - z * z;
  return -num / (R * R * sqrt(R)) / (4.0 * 3.141592653589793);
}
__device__ double dxy(double x, double y, double z) {
  double R = x * x + y * y + z * z;
  if (R == 0.0) return 0.0;
  return -3.0 * x * y / (R * R * sqrt(R)) / (4.0 * 3.141592653589793);
}
__device__ double hmgpu_entry(const double *p, const double *q, const double *prm, int a, int b) {
  double x = p[0] - q[0], y = p[1] - q[1], z = p[2] - q[2];
  switch (a < b ? a * 3 + b : b * 3 + a) {
    case 0: return dxx(x, y, z);
    case 1: return dxy(x, y, z);
    case 2: return dxy(x, z, y);
    case 4: return dxx(y, x, z);
    case 5: return dxy(y, z, x);
    default: return dxx(z, y, x);
  }
}
"""


def test_user_tensor_kernel_equals_builtin_dipolar(gpu):
    """A 3 x 3 block per point pair over trees of dims 3: component a of target
    point i / 3 is row i, component b of source point j / 3 is column j."""
    import torch
    P = geometry.cube(1200, seed=3)
    T = hmgpu.ClusterTree(P, max_points_per_leaf=16, dims=3)
    Hu = hmgpu.HMatrix(hmgpu.Kernel("user", P, user=DIPOLAR), T, T, eta=1.0, eps=1e-6, precision="f64",
                       keep_factors=True)
    Hb = hmgpu.HMatrix(hmgpu.Kernel("dipolar", P), T, T, eta=1.0, eps=1e-6, precision="f64", keep_factors=True)
    assert Hu.shape == Hb.shape == (3600, 3600)
    du, au = Hu.blocks()
    db, ab = Hb.blocks()
    np.testing.assert_array_equal(du, db)
    np.testing.assert_array_equal(au, ab)
    for b in range(0, len(au), 3):
        Uu, Vu = Hu.block_factors(b)
        Ub, Vb = Hb.block_factors(b)
        np.testing.assert_array_equal(Uu, Ub)
        np.testing.assert_array_equal(Vu, Vb)
    x = torch.randn(3600, dtype=torch.float64, device=gpu)
    assert torch.equal(Hu * x, Hb * x)
    S = hmgpu.sparsify_hmatrix(hmgpu.Kernel("user", P, user=DIPOLAR), T, T, eta=1.0)
    assert S.shape == (3600, 3600)
