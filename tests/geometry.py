"""Seeded synthetic point sets used by the tests and the benchmark.

The reference's own fixtures that need no random numbers are restated exactly
(unit circle, test/test_hmatrix.jl:10-11); the ones seeded with Julia's
Random.seed!(10) cannot be regenerated without Julia and are replaced by seeded
NumPy points of the same shape and distribution."""
import numpy as np


def circle(N=1000):
    """pts[:, i] = (sin(2 pi i/N), cos(2 pi i/N), 0), i = 1..N (test/test_hmatrix.jl:10-11)."""
    i = np.arange(1, N + 1, dtype=np.float64)
    return np.stack([np.sin(i * 2 * np.pi / N), np.cos(i * 2 * np.pi / N), np.zeros(N)])


def cube(N, seed=0):
    """N points i.i.d. uniform in [0,1]^3, 3 x N."""
    return np.random.default_rng(seed).random((N, 3)).T.copy()


def square_z0(N, seed=10):
    """N uniform points in [0,1]^2 x {0} (the shape of test/test_tree.jl and test_block.jl)."""
    p = np.random.default_rng(seed).random((N, 3))
    p[:, 2] = 0
    return p.T.copy()


def film(nx=1024, ny=1024, spacing=1.0, jitter=0.05, seed=1):
    """Thin-film cell centres: nx x ny x 1 grid with `spacing` plus Gaussian jitter of
    `jitter` spacings on every coordinate, 3 x (nx*ny)."""
    g = np.stack(np.meshgrid(np.arange(nx, dtype=np.float64), np.arange(ny, dtype=np.float64),
                             [0.0], indexing="ij"), 0).reshape(3, -1)
    return spacing * (g + jitter * np.random.default_rng(seed).standard_normal(g.shape))


def sphere(N, seed=0):
    """N points uniform on the unit sphere surface, 3 x N."""
    v = np.random.default_rng(seed).standard_normal((3, N))
    return v / np.linalg.norm(v, axis=0)
