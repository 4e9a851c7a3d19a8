"""Lean mixed precision (hmgpu_options.lean): only the tensor-core copy of the
H-matrix stays on the device, so it takes half the memory of the mixed handle,
and every product, one and two right-hand sides too, runs on the tensor cores.
Products are held to the mixed-precision bar against the oracle's FP64 mul!
(twice the plain FP32 form's error, floor 1e-6), equal the mixed handle's
bitwise from three right-hand sides on, and the entry points that need the
FP32 layout refuse a lean handle."""
import numpy as np
import pytest

import hmgpu
from oracle import oracle as O
from tests import geometry
from tests.test_matvec_gpu import _flat, rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def film():
    f = geometry.film(96, 80)
    K = O.Kernel("laplace", f.T, f.T)
    return O.HMatrix(K, O.Tree(f.T, 64), O.Tree(f.T, 64), eta=2.0, eps=1e-5, nthreads=8)


def test_lean_products_and_memory(film, gpu):
    import torch
    Ho = film
    Hm = hmgpu.HMatrix.from_flat(**_flat(Ho), precision="mixed")
    Hl = hmgpu.HMatrix.from_flat(**_flat(Ho), precision="mixed", lean=True)
    H32 = hmgpu.HMatrix.from_flat(**_flat(Ho), precision="f32")
    im, il = Hm.info(), Hl.info()
    assert il["device_bytes"] < 0.6 * im["device_bytes"], (il["device_bytes"], im["device_bytes"])
    for nr in (1, 2, 3, 32, 40):
        X = np.random.default_rng(nr).standard_normal((Ho.n, nr))
        Xd = torch.tensor(X, dtype=torch.float32, device=gpu).t().contiguous().t()
        Xr = X.astype(np.float32).astype(np.float64)
        ref = np.stack([Ho.mul(Xr[:, k]) for k in range(nr)], 1)
        Yl = (Hl * (Xd[:, 0].contiguous() if nr == 1 else Xd)).double().cpu().numpy().reshape(Ho.m, nr)
        Y32 = np.stack([(H32 * Xd[:, k].contiguous()).double().cpu().numpy() for k in range(nr)], 1)
        err = max(rel(Yl[:, k], ref[:, k]) for k in range(nr))
        err32 = max(rel(Y32[:, k], ref[:, k]) for k in range(nr))
        assert err <= max(2.0 * err32, 1e-6), (nr, err, err32)
        if nr >= 3:
            assert torch.equal(Hl * Xd, Hm * Xd), nr
    assert Hl.status() == 0


def test_lean_refusals(film, gpu, tmp_path):
    Hl = hmgpu.HMatrix.from_flat(**_flat(film), precision="mixed", lean=True)
    with pytest.raises(hmgpu.HMGPUError, match="lean"):
        Hl.save(tmp_path / "l.hmgpu")
    with pytest.raises(hmgpu.HMGPUError, match="lean"):
        Hl.shard(0, 2)
    with pytest.raises(hmgpu.HMGPUError, match="lean"):
        hmgpu.batch([Hl, Hl])
    with pytest.raises(hmgpu.HMGPUError, match="lean"):
        Hl.set_tuning(16, 64, 3, 0)
    t = Hl.autotune()  # nothing to tune: the handle stays as it is
    assert t["multi_rhs_from"] == 1


def test_lean_device_build(gpu):
    import torch
    P = geometry.cube(3000, seed=7)
    T = hmgpu.ClusterTree(P, max_points_per_leaf=32)
    K = hmgpu.Kernel("laplace", P)
    Hm = hmgpu.HMatrix(K, T, T, eta=2.0, eps=1e-6, precision="mixed")
    Hl = hmgpu.HMatrix(K, T, T, eta=2.0, eps=1e-6, precision="mixed", lean=True)
    X = torch.randn(32, P.shape[1], device=gpu).t()
    assert torch.equal(Hl * X, Hm * X)
    assert Hl.info()["matrix_bytes"] > 0
