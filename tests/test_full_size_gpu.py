"""Parity at the headline size, where the oracle cannot assemble the matrix:
N = 2^20 thin-film cell centres (1024 x 1024 x 1, spacing 1, jitter 0.05),
Laplace 1/(4 pi r), leaf 64, eta 2, tol 1e-4, assembled on the device.

Size-independent checks:
  * exact rows: for 64 random targets i, sum_j G(x_i, x_j) x_j computed
    directly in FP64 on the host agrees with the FP64 H-matrix product within
    the assembly tolerance (relative 1e-3 on those rows);
  * repeatability: two products are bitwise equal;
  * linearity: H(a x + b z) = a H x + b H z to FP64 rounding;
  * precision modes: FP32 within 1e-5 and mixed precision (32 right-hand sides
    on the tensor cores) within 1e-6 of the FP64 product of the same matrix
    (the plain FP32 form's error there is about 5.6e-7)."""
import numpy as np
import pytest

import hmgpu
from tests import geometry

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def film(gpu):
    P = geometry.film(1024, 1024, spacing=1.0, jitter=0.05, seed=1)
    T = hmgpu.ClusterTree(P, max_points_per_leaf=64)
    H64 = hmgpu.HMatrix(hmgpu.Kernel("laplace", P), T, T, eta=2.0, eps=1e-4, precision="f64")
    return P, T, H64


def test_exact_rows(film, gpu):
    import torch
    P, T, H = film
    n = P.shape[1]
    x = np.random.default_rng(3).standard_normal(n)
    y = (H * torch.tensor(x, device=gpu)).cpu().numpy()
    rows = np.random.default_rng(4).choice(n, 64, replace=False)
    exact = np.empty(len(rows))
    for k, i in enumerate(rows):  # one row at a time: 2^20 distances each
        d = np.sqrt(((P - P[:, i:i + 1]) ** 2).sum(axis=0))
        with np.errstate(divide="ignore"):
            exact[k] = np.where(d > 0, 1.0 / (4.0 * np.pi * d), 0.0) @ x
    assert np.linalg.norm(y[rows] - exact) / np.linalg.norm(exact) < 1e-3


def test_repeatable_and_linear(film, gpu):
    import torch
    _, _, H = film
    n = H.shape[1]
    g = torch.Generator(device=gpu).manual_seed(5)
    x = torch.randn(n, dtype=torch.float64, device=gpu, generator=g)
    z = torch.randn(n, dtype=torch.float64, device=gpu, generator=g)
    hx, hz = H * x, H * z
    assert torch.equal(H * x, hx)
    lin = H * (0.75 * x - 2.0 * z)
    ref = 0.75 * hx - 2.0 * hz
    assert float((lin - ref).norm() / ref.norm()) < 1e-13
    assert H.status() == 0


def test_precision_modes(film, gpu):
    import torch
    P, T, H64 = film
    n = P.shape[1]
    K = hmgpu.Kernel("laplace", P)
    X = torch.randn(32, n, dtype=torch.float32, device=gpu,
                    generator=torch.Generator(device=gpu).manual_seed(6)).t()
    Y64 = torch.empty(32, n, dtype=torch.float64, device=gpu).t()
    hmgpu.mul_(Y64, H64, X.double())
    H32 = hmgpu.HMatrix(K, T, T, eta=2.0, eps=1e-4, precision="f32")
    y32 = H32 * X[:, 0].contiguous()
    assert float((y32.double() - Y64[:, 0]).norm() / Y64[:, 0].norm()) < 1e-5
    del H32
    Hm = hmgpu.HMatrix(K, T, T, eta=2.0, eps=1e-4, precision="mixed")
    Ym = Hm * X
    err = ((Ym.double() - Y64).norm(dim=0) / Y64.norm(dim=0)).max()
    assert float(err) < 1e-6, float(err)
    assert Hm.status() == 0
