"""Writes the golden fixtures of tests/golden/ from the oracle.

The reference ships no data files and cannot run here (no Julia), so the
fixtures are the oracle's outputs on the reference's own RNG-free test inputs
(test/test_aca.jl:7-16, test/test_hmatrix.jl:10-28,
test/test_hmatrix_vector.jl:9-31). They anchor regressions of the oracle and of
the library; the oracle itself is pinned by the reference's known-answer
assertions (tests/test_oracle.py).

    python tests/golden/gen_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from oracle import oracle as O  # noqa: E402
from tests import geometry  # noqa: E402


def inv_sq_block():
    N = 100
    i = np.arange(1, N + 1, dtype=np.float64)
    d = i[:, None] - i[None, :]
    with np.errstate(divide="ignore"):
        K = np.where(d != 0, N / d ** 2, 0.0)
    return K[N - 30:, :30]


def main():
    blk = inv_sq_block()
    U, V = O.aca_plus(O.Kernel("explicit", A=blk), np.arange(1, 31), np.arange(1, 31), 1e-7)
    Us, Vs = O.svd_recompress(U, V, 1e-7)
    np.savez_compressed(os.path.join(HERE, "aca_inv_sq.npz"), block=blk, U=U, V=V, U_svd=Us, V_svd=Vs)

    pts = geometry.circle(1000)
    x = np.sin(np.arange(1, 1001, dtype=np.float64))
    for name, kind, dims in [("circle_log2d", "log2d", 1), ("circle_vector_r", "vector_r", 3)]:
        K = O.Kernel(kind, pts.T, pts.T)
        X = O.Tree(pts.T, 64)
        Y = O.Tree(pts.T, 64, dims)
        H = O.HMatrix(K, X, Y, eta=1.5, eps=1e-6)
        xv = np.sin(np.arange(1, H.n + 1, dtype=np.float64))
        np.savez_compressed(
            os.path.join(HERE, name + ".npz"),
            target_index_map=X.index_map, source_index_map=Y.index_map,
            dense_block_indices=H.dense_block_indices, U_block_indices=H.U_block_indices,
            aca_ranks=H.aca_ranks, final_ranks=H.final_ranks, x=xv, y=H.mul(xv),
            y_dense=K.matvec(xv), compression_ratio=H.info()["compression_ratio"])
    print("wrote", sorted(f for f in os.listdir(HERE) if f.endswith(".npz")))


if __name__ == "__main__":
    main()
