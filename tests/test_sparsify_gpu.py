"""sparsify_hmatrix on the device (hmgpu_sparsify) against the oracle's
restatement of src/hmatrix.jl:234-274: the same (I, J) indices in the same
order, and the same values: bit for bit where an entry is built from +, -, *,
/ and sqrt (all correctly rounded on both sides), within 2 ulp where it takes
a log or an exp (the device's and the host library's differ in the last bit)."""
import ctypes as C

import numpy as np
import pytest

import hmgpu
from oracle import oracle as O
from tests import geometry

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind,geom,leaf,eta,dims", [
    ("log2d", "circle", 64, 1.5, 1),      # test/test_hmatrix.jl:102-108
    ("vector_r", "circle", 64, 1.5, 3),
    ("laplace", "cube", 32, 2.0, 1),
    ("yukawa", "sphere", 16, 1.0, 1),
    ("dipolar", "cube", 16, 1.0, 3),
])
def test_triplets_equal_oracle(gpu, kind, geom, leaf, eta, dims):
    P = {"circle": geometry.circle(1000), "sphere": geometry.sphere(2000, seed=2),
         "cube": geometry.cube(1200, seed=3)}[geom]
    xd = 3 if kind == "dipolar" else 1
    Ko = O.Kernel(kind, P.T, P.T)
    Io, Jo, Vo = O.sparsify(Ko, O.Tree(P.T, leaf, xd), O.Tree(P.T, leaf, dims), eta)
    X = hmgpu.ClusterTree(P, max_points_per_leaf=leaf, dims=xd)
    Y = hmgpu.ClusterTree(P, max_points_per_leaf=leaf, dims=dims)
    I, J, V = hmgpu.sparsify_hmatrix(hmgpu.Kernel(kind, P), X, Y, eta=eta, triplets=True)
    assert np.array_equal(I, Io) and np.array_equal(J, Jo)
    if kind in ("log2d", "yukawa"):
        assert np.all(np.abs(V - Vo) <= 2 * np.spacing(np.abs(Vo))), float(np.max(np.abs(V - Vo)))
    else:
        assert np.array_equal(V, Vo), float(np.max(np.abs(V - Vo)))
    S = hmgpu.sparsify_hmatrix(hmgpu.Kernel(kind, P), X, Y, eta=eta)
    assert S.shape == Ko.shape and S.nnz == len(I)


def test_explicit_matrix(gpu):
    P = geometry.cube(800, seed=5)
    A = O.Kernel("laplace", P.T, P.T).dense()
    T = hmgpu.ClusterTree(P, max_points_per_leaf=32)
    I, J, V = hmgpu.sparsify_hmatrix(A, T, T, eta=2.0, triplets=True)
    assert np.array_equal(V, A[I - 1, J - 1])
    x = np.random.default_rng(1).standard_normal(800)
    S = hmgpu.sparsify_hmatrix(A, T, T, eta=2.0)
    dense, _ = hmgpu.BlockTree(T, T, eta=2.0, merge=True).traverse()  # src/block.jl:98-155
    tm = T.index_map
    yd = np.zeros(800)
    for a, b in dense:
        rows, cols = tm[a.start_idx - 1:a.end_idx - 1] - 1, tm[b.start_idx - 1:b.end_idx - 1] - 1
        yd[rows] += A[np.ix_(rows, cols)] @ x[cols]
    assert np.max(np.abs(S @ x - yd)) < 1e-12


def test_count_and_argument_checks(gpu):
    P = geometry.cube(300, seed=6)
    T = hmgpu.ClusterTree(P, max_points_per_leaf=16)
    d = hmgpu.Kernel("laplace", P).desc()
    L = hmgpu._lib.lib()
    nnz = C.c_int64(-1)
    assert L.hmgpu_sparsify(C.byref(d), T._h, T._h, 1.0, None, None, None, C.byref(nnz)) == 0
    assert nnz.value > 0
    I = np.empty(nnz.value, np.int64)
    assert L.hmgpu_sparsify(C.byref(d), T._h, T._h, 1.0, hmgpu.ptr(I, hmgpu._lib.I64P), None, None,
                            C.byref(nnz)) == -1
    assert b"all be given" in L.hmgpu_last_error()
