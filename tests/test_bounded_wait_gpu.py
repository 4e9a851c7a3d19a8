"""Failure detection of the tensor-core product's bounded device-side waits,
without a GPU fault: the same wait runs against a barrier that nothing
completes, with a short limit. It must give up, record its status code, and
leave the context usable, so that the next product runs with a clean status."""
import numpy as np
import pytest

import hmgpu
from oracle import oracle as O
from tests import geometry

pytestmark = pytest.mark.gpu


def test_wait_expires_and_reports(gpu):
    code, waited = hmgpu.selftest_bounded_wait(20.0)
    assert code == 90, code
    # the limit is read from the device's global timer; the loop stops at the
    # first check after it
    assert 20.0 <= waited < 1000.0, waited


def test_limit_is_validated(gpu):
    for bad in (0.0, 0.5, 5000.0):
        with pytest.raises(hmgpu.HMGPUError):
            hmgpu.selftest_bounded_wait(bad)


def test_context_usable_after_expired_wait(gpu):
    import torch
    assert hmgpu.selftest_bounded_wait(5.0)[0] == 90
    p = geometry.cube(2048, seed=4)
    K = O.Kernel("laplace", p.T, p.T)
    Ho = O.HMatrix(K, O.Tree(p.T, 32), O.Tree(p.T, 32), eta=2.0, eps=1e-5, nthreads=8)
    H = hmgpu.HMatrix.from_flat(m=Ho.m, n=Ho.n, target_index_map=Ho.target_index_map,
                                source_index_map=Ho.source_index_map,
                                dense_block_indices=Ho.dense_block_indices,
                                dense_blocks=Ho.dense_blocks, U_block_indices=Ho.U_block_indices,
                                U_matrices=Ho.U_matrices, V_block_indices=Ho.V_block_indices,
                                V_matrices=Ho.V_matrices, precision="mixed")
    X = np.random.default_rng(1).standard_normal((Ho.n, 32))
    Xd = torch.tensor(X, dtype=torch.float32, device=gpu).t().contiguous().t()
    Y = (H * Xd).double().cpu().numpy()
    Xr = X.astype(np.float32).astype(np.float64)
    for k in (0, 31):
        ref = Ho.mul(Xr[:, k])
        assert np.linalg.norm(Y[:, k] - ref) <= 2e-4 * np.linalg.norm(ref)
    assert H.status() == 0
