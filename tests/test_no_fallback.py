"""Without a GPU the library does not fall back to anything: assembly, import
and products raise with the CUDA error, and the oracle is never called."""
import numpy as np
import pytest

import hmgpu
from tests import geometry
from tests.conftest import has_gpu

pytestmark = pytest.mark.skipif(has_gpu(), reason="checks the behaviour on a host without a GPU")


def test_device_assembly_raises():
    P = geometry.cube(500, seed=1)
    T = hmgpu.ClusterTree(P, max_points_per_leaf=32)  # the host tree needs no GPU
    with pytest.raises(hmgpu.HMGPUError) as e:
        hmgpu.HMatrix(hmgpu.Kernel("laplace", P), T, T, eta=2.0, eps=1e-6)
    assert e.value.code in (-2, -3), e.value  # a CUDA or allocation error, not a result


def test_import_raises():
    n = 4
    with pytest.raises(hmgpu.HMGPUError) as e:
        hmgpu.HMatrix.from_flat(n, n, np.arange(1, n + 1), np.arange(1, n + 1),
                                np.array([[1, n, 1, n, 1]]), np.ones(n * n),
                                np.zeros((0, 5), np.int64), np.zeros(0),
                                np.zeros((0, 3), np.int64), np.zeros(0))
    assert e.value.code == -2, e.value  # the CUDA error: the tables themselves are valid
