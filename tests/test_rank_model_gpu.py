"""The learned ACA-rank predictor: its forward and backward kernels against an
FP64 NumPy restatement (oracle/mlp.py), training on ranks the device ACA
produced, and what it buys the assembly while leaving the H-matrix unchanged."""
import numpy as np
import pytest

import hmgpu
from oracle import mlp as M
from tests import geometry

pytestmark = pytest.mark.gpu


def test_forward_and_gradients_match_fp64(gpu):
    rng = np.random.default_rng(0)
    model = hmgpu.RankModel(seed=3)
    p = (rng.standard_normal(M.NPARAMS) * 0.2).astype(np.float32)
    norm = np.concatenate([rng.standard_normal(8), rng.uniform(0.5, 2.0, 8)]).astype(np.float32)
    model.params(set_params=p, set_norm=norm)
    X = rng.standard_normal((777, 8)).astype(np.float32) * norm[8:] + norm[:8]
    y = rng.uniform(1, 30, 777).astype(np.float32)
    out = model.predict(X)
    ref, _ = M.forward(p, norm.astype(np.float64), X)
    np.testing.assert_allclose(out, ref, rtol=2e-4, atol=2e-4 * np.abs(ref).max())
    g, loss = model.gradients(X, y)
    lref, gref = M.loss_and_grad(p, norm.astype(np.float64), X, y)
    assert abs(loss - lref) <= 1e-4 * lref
    assert np.linalg.norm(g - gref) <= 1e-4 * np.linalg.norm(gref)
    # each parameter block separately, so that a small block cannot hide
    off = 0
    for name, shape in M.SIZES:
        k = int(np.prod(shape))
        gb, rb = g[off:off + k], gref[off:off + k]
        assert np.linalg.norm(gb - rb) <= 1e-3 * max(np.linalg.norm(rb), 1e-6), name
        off += k


def _training_set(eps_list=(1e-4, 1e-6)):
    feats, ranks = [], []
    geoms = [geometry.cube(6000, seed=1), geometry.film(80, 80), geometry.sphere(6000, seed=2)]
    for P in geoms:
        T = hmgpu.ClusterTree(P, max_points_per_leaf=32)
        for eps in eps_list:
            H = hmgpu.HMatrix(hmgpu.Kernel("laplace", P), T, T, eta=2.0, eps=eps, precision="f32")
            f = hmgpu.block_features(T, T, 2.0, eps)
            a, _ = H.aca_ranks(len(f))
            feats.append(f)
            ranks.append(a.astype(np.float32))
    return np.concatenate(feats), np.concatenate(ranks)


def test_training_and_learned_bucketing(gpu):
    import torch
    X, y = _training_set()
    assert len(y) > 5000 and y.min() >= 1
    model = hmgpu.RankModel(seed=1)
    loss0 = model.gradients(X, y)[1]
    loss = model.train(X, y, epochs=60, batch=512, lr=2e-3, seed=1)
    assert loss < 0.05 * loss0, (loss0, loss)
    pred = model.predict(X)
    mae = float(np.mean(np.abs(pred - y)))
    assert mae < 0.25 * float(np.mean(y)), mae
    # geometries the network has not seen: a larger film at the headline
    # tolerance (low ranks: the fixed 48-term workspace is mostly idle) and a
    # denser cube at a tight tolerance (high ranks)
    for P, eps, gain in [(geometry.film(150, 120, seed=4), 1e-4, 0.5),
                         (geometry.cube(12000, seed=9), 1e-5, 0.95)]:
        T = hmgpu.ClusterTree(P, max_points_per_leaf=32)
        K = hmgpu.Kernel("laplace", P)
        plain = hmgpu.HMatrix(K, T, T, eta=2.0, eps=eps, precision="f32")
        learned = hmgpu.HMatrix(K, T, T, eta=2.0, eps=eps, precision="f32", rank_model=model)
        x = torch.randn(P.shape[1], device=gpu)
        assert torch.equal(plain * x, learned * x)  # the network never changes the matrix
        ip, il = plain.info(), learned.info()
        nblocks = len(hmgpu.block_features(T, T, 2.0, eps))
        assert il["aca_workspace_bytes"] < gain * ip["aca_workspace_bytes"], (eps, ip, il)
        assert il["aca_reruns"] <= 0.05 * nblocks, (eps, il["aca_reruns"], nblocks)


def test_outgrown_caps_continue_bitwise(gpu):
    """A network that predicts far too low (untrained, caps near 4 terms) makes
    most blocks outgrow their workspace. Each continues from its state in the
    same batch (the first terms, the last residual row and column, the used
    pivots), so the H-matrix is bitwise the one built without the network."""
    import torch
    P = geometry.film(90, 70, seed=5)
    T = hmgpu.ClusterTree(P, max_points_per_leaf=32)
    K = hmgpu.Kernel("laplace", P)
    plain = hmgpu.HMatrix(K, T, T, eta=2.0, eps=1e-6, precision="f64", keep_factors=True)
    low = hmgpu.RankModel(seed=3)
    low.params(set_params=np.zeros(hmgpu.RankModel.NPARAMS, np.float32))  # predicts 0 everywhere
    learned = hmgpu.HMatrix(K, T, T, eta=2.0, eps=1e-6, precision="f64", keep_factors=True, rank_model=low)
    il = learned.info()
    nblocks = len(hmgpu.block_features(T, T, 2.0, 1e-6))
    assert il["aca_continued"] > 0.5 * nblocks, (il["aca_continued"], nblocks)
    a_p, _ = plain.aca_ranks(nblocks)
    a_l, _ = learned.aca_ranks(nblocks)
    np.testing.assert_array_equal(a_p, a_l)
    for b in range(0, plain.info()["admissible_leaves"], 7):
        Up, Vp = plain.block_factors(b)
        Ul, Vl = learned.block_factors(b)
        np.testing.assert_array_equal(Up, Ul)
        np.testing.assert_array_equal(Vp, Vl)
    x = torch.randn(P.shape[1], dtype=torch.float64, device=gpu)
    assert torch.equal(plain * x, learned * x)
