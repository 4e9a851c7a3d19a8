"""Assembled H-matrices on disk (hmgpu_hmatrix_save / hmgpu_hmatrix_load):
a loaded matrix multiplies bit for bit like the saved one, and damaged files
are refused before anything reaches the device."""
import numpy as np
import pytest

import hmgpu
from tests import geometry

pytestmark = pytest.mark.gpu


def _h(precision, n=4000, seed=3):
    P = geometry.cube(n, seed=seed)
    T = hmgpu.ClusterTree(P, max_points_per_leaf=32)
    return hmgpu.HMatrix(hmgpu.Kernel("laplace", P), T, T, eta=2.0, eps=1e-5, precision=precision)


@pytest.mark.parametrize("precision,nrhs", [("f64", 1), ("f32", 1), ("f32", 33), ("mixed", 32)])
def test_round_trip_bitwise(gpu, tmp_path, precision, nrhs):
    import torch
    H = _h(precision)
    path = tmp_path / "h.hmgpu"
    H.save(path)
    G = hmgpu.HMatrix.load(path)
    assert G.shape == H.shape and G.info()["admissible_leaves"] == H.info()["admissible_leaves"]
    a, b = H.blocks(), G.blocks()
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    dt = torch.float64 if precision == "f64" else torch.float32
    g = torch.Generator(device=gpu).manual_seed(nrhs)
    x = torch.randn(H.shape[1], device=gpu, dtype=dt, generator=g) if nrhs == 1 else \
        torch.randn(nrhs, H.shape[1], device=gpu, dtype=dt, generator=g).t()
    assert torch.equal(H * x, G * x)
    assert G.status() == 0


def test_batch_round_trip(gpu, tmp_path):
    import torch
    B = hmgpu.batch([_h("f32", 3000, 1), _h("f32", 2000, 2)])
    path = tmp_path / "b.hmgpu"
    B.save(path)
    G = hmgpu.HMatrix.load(path)
    x = torch.randn(B.shape[1], device=gpu)
    assert torch.equal(B * x, G * x)


def test_damaged_files_are_refused(gpu, tmp_path):
    H = _h("f32", 1500, 4)
    path = tmp_path / "h.hmgpu"
    H.save(path)
    raw = path.read_bytes()
    cut = tmp_path / "cut.hmgpu"
    cut.write_bytes(raw[: len(raw) // 2])
    with pytest.raises(hmgpu.HMGPUError, match="truncated"):
        hmgpu.HMatrix.load(cut)
    flip = bytearray(raw)
    flip[-100] ^= 0x40  # inside the V rows
    bad = tmp_path / "bad.hmgpu"
    bad.write_bytes(bytes(flip))
    with pytest.raises(hmgpu.HMGPUError, match="checksum"):
        hmgpu.HMatrix.load(bad)


@pytest.mark.parametrize("unit_rows", [32, 64])
def test_tuned_round_trip(gpu, tmp_path, unit_rows):
    """A matrix saved after tuning keeps its tuning: every unit size the tuner
    may choose loads back (near/U units of 8, 16, 32 or 64 rows)."""
    import torch
    H = _h("f32", 3000, 5)
    H.set_tuning(unit_rows, 64, 8, 1)
    path = tmp_path / "t.hmgpu"
    H.save(path)
    G = hmgpu.HMatrix.load(path)
    assert G.tuning() == H.tuning()
    x = torch.randn(H.shape[1], device=gpu)
    assert torch.equal(H * x, G * x)
