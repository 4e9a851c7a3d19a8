"""The oracle against the reference's own known-answer tests (CPU only).

Each test restates one assertion block of the reference's test suite on the
oracle, so that the checker used by the GPU parity tests is itself pinned."""
import numpy as np
import pytest

from oracle import oracle as O
from tests import geometry


def _inv_sq_block():
    # test/test_aca.jl:7-16: K[i,j] = N/(i-j)^2 off the diagonal, last 30 rows x first 30 cols
    N = 100
    i = np.arange(1, N + 1, dtype=np.float64)
    d = i[:, None] - i[None, :]
    with np.errstate(divide="ignore"):
        K = np.where(d != 0, N / d ** 2, 0.0)
    return K[N - 30:, :30]


def test_aca_known_answer():
    """test/test_aca.jl:17-42."""
    blk = _inv_sq_block()
    eps = 1e-6
    K = O.Kernel("explicit", A=blk)
    U, V = O.aca_plus(K, np.arange(1, 31), np.arange(1, 31), eps / 10.0)
    x = np.random.default_rng(10).random(30)
    assert U.shape[1] < 30
    assert np.linalg.norm(U @ V - blk, 2) < eps / 100
    assert np.max(np.abs(U @ (V @ x) - blk @ x)) < eps / 100
    Us, Vs = O.svd_recompress(U, V, eps / 10)
    assert np.max(np.abs(Us @ (Vs @ x) - blk @ x)) < eps / 100
    assert np.linalg.norm(Us @ Vs - blk, 2) < eps / 100
    assert U.shape[1] >= Us.shape[1]


def test_aca_pivot_rules_small():
    """First step: row pivot from column 1, then the pivot row; ties to the lowest index."""
    A = np.array([[1.0, 2.0, 3.0], [4.0, 5.0, 6.0], [7.0, 8.0, 10.0]])
    K = O.Kernel("explicit", A=A)
    U, V = O.aca_plus(K, np.arange(1, 4), np.arange(1, 4), 0.0)
    # k=1: column 1 -> row pivot 3 (|7| largest) -> row 3 -> column pivot 3 (|10|)
    np.testing.assert_allclose(U[:, 0], A[:, 0])
    np.testing.assert_allclose(V[0], A[2] / A[2, 0])
    assert U.shape[1] == 3
    np.testing.assert_allclose(U @ V, A, rtol=0, atol=1e-12)


def test_qr_and_svd_against_numpy():
    rng = np.random.default_rng(3)
    for m, k in [(40, 7), (12, 12), (100, 1), (5, 3)]:
        U = rng.standard_normal((m, k))
        V = rng.standard_normal((k, 23 if k <= 23 else k))
        s_ref = np.linalg.svd(U @ V, compute_uv=False)
        Us, Vs = O.svd_recompress(U, V, 0.0)
        assert Us.shape[1] == k
        np.testing.assert_allclose(Us @ Vs, U @ V, rtol=0, atol=1e-12 * np.abs(U @ V).max())
        s = np.linalg.svd(Us @ Vs, compute_uv=False)
        np.testing.assert_allclose(s[:k], s_ref[:k], rtol=1e-12, atol=1e-13 * s_ref[0])


def test_svd_truncation_rule():
    """rank = first i with sqrt(sum_{j>=i} s_j^2) < eps, minus one (src/aca.jl:132-136)."""
    rng = np.random.default_rng(4)
    Q1, _ = np.linalg.qr(rng.standard_normal((30, 6)))
    Q2, _ = np.linalg.qr(rng.standard_normal((25, 6)))
    s = np.array([1.0, 0.5, 1e-3, 4e-4, 3e-4, 1e-9])
    U, V = Q1 * s, Q2.T
    tails = np.sqrt(np.cumsum((s ** 2)[::-1]))[::-1]
    for eps in [2.0, 0.6, 1e-3, 5.1e-4, 1e-8, 1e-12]:
        hit = np.nonzero(tails < eps)[0]
        want = int(hit[0]) if len(hit) else 6
        Us, Vs = O.svd_recompress(U, V, eps)
        assert Us.shape[1] == want, (eps, Us.shape)


@pytest.fixture(scope="module")
def circle_h():
    pts = geometry.circle(1000)
    T = O.Tree(pts.T, 64)
    K = O.Kernel("log2d", pts.T, pts.T)
    return K, T, O.HMatrix(K, T, T, eta=1.5, eps=1e-6)


def test_hmatrix_circle_known_answers(circle_h):
    """test/test_hmatrix.jl:27-55 and :106-155 on the oracle."""
    K, T, H = circle_h
    assert H.info()["compression_ratio"] > 3
    assert not np.isnan(H.dense_blocks).any()
    assert not np.isnan(H.U_matrices).any() and not np.isnan(H.V_matrices).any()
    x = np.random.default_rng(10).random(1000)
    y = H.mul(x)
    assert np.max(np.abs(K.matvec(x) - y)) < 1e-5  # isapprox(K*x, H*x; atol=1e-5)
    # V-table consistency: max over columns of offset + (col_end - col_start + 1)
    vi = H.V_block_indices
    assert np.max(vi[:, 2] + vi[:, 1] - vi[:, 0] + 1) == len(H.V_matrices)
    # flattened semantics == CPU mul! (the reference compares parts at 1e-12 / 1e-10)
    yf, vx = H.mul_flat(x)
    assert np.max(np.abs(yf - y)) < 1e-12
    xo = x[H.source_index_map - 1]
    vx_cpu = []
    off = 0
    for rs, re, vs, ve, uoff in H.U_block_indices:
        r = ve - vs + 1
        cs, ce = H.V_block_indices[vs - 1, :2]
        n = ce - cs + 1
        V = H.V_matrices[H.V_block_indices[vs - 1, 2]:][: r * n].reshape(r, n)
        vx_cpu.append(V @ xo[cs - 1:ce])
    assert np.max(np.abs(np.concatenate(vx_cpu) - vx)) < 1e-10


def test_hmatrix_vector_dofs():
    """test/test_hmatrix_vector.jl:27-60 on the oracle."""
    pts = geometry.circle(1000)
    Tt = O.Tree(pts.T, 64)
    Ts = O.Tree(pts.T, 64, dims=3)
    assert sorted(Ts.index_map) == list(range(1, 3001))
    K = O.Kernel("vector_r", pts.T, pts.T)
    H = O.HMatrix(K, Tt, Ts, eta=1.5, eps=1e-6)
    assert H.info()["compression_ratio"] > 3
    x = np.random.default_rng(10).random(3000)
    assert np.max(np.abs(K.matvec(x) - H.mul(x))) < 1e-5
    vi = H.V_block_indices
    assert np.max(vi[:, 2] + vi[:, 1] - vi[:, 0] + 1) == len(H.V_matrices)


def test_tree_properties():
    """test/test_tree.jl: 1000 points with z = 0, leaf 10."""
    pts = geometry.square_z0(1000)
    T = O.Tree(pts.T, 10)
    leaves = T.is_leaf == 1
    counts = (T.end - T.start)[leaves]
    assert counts.max() <= 10 and counts.min() >= 3
    assert sorted(T.index_map) == list(range(1, 1001))


def test_block_tree_properties():
    """test/test_block.jl: 32 points, source leaf 4, target leaf 8."""
    pts = geometry.square_z0(32, seed=11)
    S = O.Tree(pts.T, 4)
    Tt = O.Tree(pts.T, 8)
    for eta in (1.5, 0.5):
        B = O.Blocks(Tt, S, eta=eta, merge=False)
        flagged = (B.node_adm == 1) | (B.node_dense == 1)
        assert np.all(B.node_left[flagged] == -1) and np.all(B.node_right[flagged] == -1)
        for k in np.nonzero(B.node_adm)[0]:
            a, b = B.node_target[k], B.node_source[k]
            dist = np.linalg.norm(Tt.center[a] - S.center[b])
            assert dist > eta * (Tt.radius[a] + S.radius[b])
    B = O.Blocks(Tt, S, eta=1.5, merge=False)
    assert len(B.dense) > 0 and len(B.approx) > 0
    rng = np.random.default_rng(12)
    Km = rng.random((32, 32))
    x = rng.random(32)
    y = np.zeros(32)
    for a, b in np.concatenate([B.dense, B.approx]):
        ia = Tt.index_map[Tt.start[a] - 1:Tt.end[a] - 1] - 1
        ib = S.index_map[S.start[b] - 1:S.end[b] - 1] - 1
        y[ia] += Km[np.ix_(ia, ib)] @ x[ib]
    np.testing.assert_allclose(y, Km @ x, rtol=0, atol=1e-10)


def test_mul_cpu_threads_match():
    pts = geometry.cube(2000, seed=5)
    T = O.Tree(pts.T, 32)
    K = O.Kernel("laplace", pts.T, pts.T)
    H = O.HMatrix(K, T, T, eta=2.0, eps=1e-6, nthreads=4)
    x = np.random.default_rng(6).standard_normal(2000)
    y1 = H.mul(x, 1)
    y4 = H.mul(x, 4)
    assert np.max(np.abs(y1 - y4)) <= 1e-13 * np.max(np.abs(y1))
    yd = K.matvec(x)
    assert np.linalg.norm(y1 - yd) / np.linalg.norm(yd) < 1e-5


def _dense_multiply(H, x):
    # test/test_hmatrix.jl:79-100: the dense blocks of the flattened HMatrix alone
    y = np.zeros(H.m)
    for rs, re, cs, ce, off in H.dense_block_indices:
        m, n = re - rs + 1, ce - cs + 1
        D = H.dense_blocks[off:off + m * n].reshape(m, n)
        y[H.target_index_map[rs - 1:re] - 1] += D @ x[H.source_index_map[cs - 1:ce] - 1]
    return y


def test_sparsify_against_dense_part(circle_h):
    """test/test_hmatrix.jl:102-108: sparsify_hmatrix(K, X, X; eta=1.5) * x equals
    the product with the HMatrix's dense blocks (atol 1e-12)."""
    K, T, H = circle_h
    I, J, V = O.sparsify(K, T, T, eta=1.5)
    assert len(I) == len(J) == len(V) > 0
    assert (I >= 1).all() and (I <= H.m).all() and (J >= 1).all() and (J <= H.n).all()
    x = np.random.default_rng(10).random(H.n)
    c = np.zeros(H.m)
    np.add.at(c, I - 1, V * x[J - 1])
    assert np.max(np.abs(_dense_multiply(H, x) - c)) < 1e-12
    # every entry is K[I, J]
    for k in range(0, len(I), 997):
        assert V[k] == K.entry(I[k], J[k])
