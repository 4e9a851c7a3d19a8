"""The library's host-side cluster tree and block partition against the oracle,
bit for bit (CPU only; no GPU call)."""
import numpy as np
import pytest

import hmgpu
from oracle import oracle as O
from tests import geometry

CASES = [
    ("square_z0", 1000, 10, 1, 1.5),
    ("cube", 4096, 32, 1, 2.0),
    ("circle", 1000, 64, 1, 1.5),
    ("circle", 1000, 64, 3, 1.5),
    ("film", 64 * 64, 64, 1, 2.0),
    ("sphere", 5000, 16, 1, 1.0),
    ("cube", 37, 4, 1, 0.5),
    ("cube", 1, 32, 1, 2.0),
    ("cube", 65536, 64, 1, 2.0),
]


def _points(kind, N):
    if kind == "circle":
        return geometry.circle(N)
    if kind == "film":
        return geometry.film(64, 64)
    if kind == "sphere":
        return geometry.sphere(N, seed=3)
    if kind == "square_z0":
        return geometry.square_z0(N)
    return geometry.cube(N, seed=N)


@pytest.mark.parametrize("kind,N,leaf,dims,eta", CASES)
def test_tree_and_partition_bit_exact(kind, N, leaf, dims, eta):
    P = _points(kind, N)
    T = hmgpu.ClusterTree(P, max_points_per_leaf=leaf, dims=dims)
    R = O.Tree(P.T, leaf, dims)
    assert np.array_equal(T.index_map, R.index_map)
    assert np.array_equal(T._start, R.start) and np.array_equal(T._end, R.end)
    assert np.array_equal(T._leaf, R.is_leaf)
    assert np.array_equal(T._left, R.left) and np.array_equal(T._right, R.right)
    assert np.array_equal(T._center.view(np.uint64), R.center.view(np.uint64))
    assert np.array_equal(T._radius.view(np.uint64), R.radius.view(np.uint64))
    Ts = hmgpu.ClusterTree(P, max_points_per_leaf=leaf)
    Rs = O.Tree(P.T, leaf)
    for merge in (False, True):
        B = hmgpu.BlockTree(T, Ts, eta=eta, merge=merge)
        BR = O.Blocks(R, Rs, eta=eta, merge=merge)
        assert np.array_equal(B._dense_pairs, BR.dense)
        assert np.array_equal(B._approx_pairs, BR.approx)
        assert np.array_equal(B._adm, BR.node_adm) and np.array_equal(B._dense, BR.node_dense)
        assert np.array_equal(B._left, BR.node_left)


def test_tree_info_and_errors():
    P = geometry.square_z0(1000)
    T = hmgpu.ClusterTree(P, max_points_per_leaf=10)
    s = hmgpu.info(T)
    assert s["max_points"] <= 10 and s["min_points"] >= 3 and s["depth"] > 1
    with pytest.raises(ValueError):
        hmgpu.ClusterTree(P, dims=0)
    with pytest.raises(hmgpu.HMGPUError):  # coincident points cannot be bisected
        hmgpu.ClusterTree(np.zeros((3, 50)), max_points_per_leaf=10)
    with pytest.raises(ValueError):
        hmgpu.ClusterTree(np.zeros((2, 50)))


def test_block_tree_views():
    """test/test_block.jl:20-70 on the library's block tree."""
    P = geometry.square_z0(32, seed=11)
    S = hmgpu.ClusterTree(P, max_points_per_leaf=4)
    T = hmgpu.ClusterTree(P, max_points_per_leaf=8)
    bt = hmgpu.BlockTree(T, S, eta=1.5)
    assert bt.root.left is not None and bt.root.right is not None

    def check(node, eta):
        if node.is_dense or node.is_admissible:
            assert node.left is None and node.right is None
        if node.is_admissible:
            d = np.linalg.norm(node.target_tree.center - node.source_tree.center)
            assert d > eta * (node.target_tree.radius + node.source_tree.radius)
        if node.left is not None:
            check(node.left, eta)
            check(node.right, eta)

    check(bt.root, 1.5)
    check(hmgpu.BlockTree(T, S, eta=0.5).root, 0.5)
    direct, approx = hmgpu.traverse(bt)
    assert len(direct) > 0 and len(approx) > 0
