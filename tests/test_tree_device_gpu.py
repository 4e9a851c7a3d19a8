"""Cluster and block trees built on the GPU (hmgpu_tree_build_device,
hmgpu_blocks_build_device) against the host builds, which follow ClusterTree
(src/tree.jl:45-137) and BlockTree + merge + traverse (src/block.jl:31-155).

The two builds must agree bit for bit: index map, ranges, children in
pre-order, leaf flags, centers and radii; block-tree node numbers, flags,
children and both traverse lists; and they must fail alike."""
import ctypes as C
import time

import numpy as np
import pytest

import hmgpu
from hmgpu._lib import lib
from tests import geometry

pytestmark = pytest.mark.gpu


def _same(a, b):
    for name in ("index_map", "_start", "_end", "_leaf", "_left", "_right"):
        np.testing.assert_array_equal(getattr(a, name), getattr(b, name), err_msg=name)
    for name in ("_center", "_radius"):  # bitwise, NaN included
        np.testing.assert_array_equal(getattr(a, name).view(np.int64), getattr(b, name).view(np.int64),
                                      err_msg=name)
    assert a.info() == b.info()


def _lattice(n, seed):
    """Integer lattice points with many coordinates equal to a node centroid."""
    rng = np.random.default_rng(seed)
    return rng.integers(0, 7, size=(3, n)).astype(np.float64) + np.arange(n) * 1e-9


CASES = [
    ("sphere", lambda: geometry.sphere(3000, seed=1), 32, 1),
    ("cube_dims3", lambda: geometry.cube(20000, seed=2), 16, 3),
    ("film_lattice", lambda: geometry.film(256, 256, jitter=0.0, seed=3), 64, 1),
    ("film_jitter", lambda: geometry.film(300, 200, seed=4), 50, 2),
    ("lattice_ties", lambda: _lattice(5000, 5), 8, 1),
    ("leaf1", lambda: geometry.cube(4097, seed=6), 1, 1),
    ("one_point", lambda: np.array([[0.5], [0.25], [-1.0]]), 32, 1),
    ("two_points", lambda: np.array([[0.0, 1.0], [0.0, 0.0], [0.0, 0.0]]), 1, 1),
    ("flat_plane", lambda: geometry.square_z0(3000), 24, 1),
    ("huge_offsets", lambda: geometry.cube(2000, seed=8) * 1e150 + 1e160, 16, 1),
    ("tiny_scale", lambda: geometry.cube(2000, seed=9) * 1e-160, 16, 1),
    # centroid sums with exact ties at half units, sign changes and wide ranges
    ("half_units", lambda: np.round(np.random.default_rng(10).uniform(-50, 50, (3, 30000)) * 2) / 2, 20, 1),
    ("mixed_scales", lambda: np.random.default_rng(11).standard_normal((3, 30000))
     * np.exp2(np.random.default_rng(12).integers(-30, 30, (3, 30000))), 20, 1),
    ("small_then_large", lambda: np.concatenate([np.random.default_rng(13).uniform(0, 4, (3, 20000)),
                                                 np.random.default_rng(14).uniform(500, 520, (3, 20000))], 1), 32, 1),
]


@pytest.mark.parametrize("name,pts,leaf,dims", CASES, ids=[c[0] for c in CASES])
def test_device_tree_matches_host(gpu, name, pts, leaf, dims):
    P = pts()
    host = hmgpu.ClusterTree(P, max_points_per_leaf=leaf, dims=dims)
    dev = hmgpu.ClusterTree(P, max_points_per_leaf=leaf, dims=dims, gpu=True)
    _same(host, dev)


def test_device_tree_full_size(gpu):
    """The 2^20-point film of the product benchmark; the GPU build is timed
    beside the host build."""
    P = geometry.film(1024, 1024, seed=1)
    t0 = time.perf_counter()
    dev = hmgpu.ClusterTree(P, max_points_per_leaf=64, gpu=True)
    t1 = time.perf_counter()
    host = hmgpu.ClusterTree(P, max_points_per_leaf=64)
    t2 = time.perf_counter()
    _same(host, dev)
    print(f"\ncluster tree of 2^20 points: device {1e3 * (t1 - t0):.1f} ms, host {1e3 * (t2 - t1):.1f} ms")


def test_device_tree_from_device_memory(gpu):
    import torch
    P = geometry.cube(10000, seed=11)
    host = hmgpu.ClusterTree(P, max_points_per_leaf=32)
    d = torch.from_numpy(np.ascontiguousarray(P.T)).to(gpu)  # point-major, as coordinates[:, i]
    h = C.c_void_p()
    L = lib()
    assert L.hmgpu_tree_build_device(d.data_ptr(), P.shape[1], 32, 1, C.byref(h)) == 0
    n = C.c_int64()
    assert L.hmgpu_tree_info(h, C.byref(n), None, None, None, None) == 0
    imap = np.empty(P.shape[1], np.int64)
    center = np.empty((n.value, 3))
    assert L.hmgpu_tree_export(h, imap.ctypes.data_as(C.POINTER(C.c_int64)), None, None, None, None,
                               None, center.ctypes.data_as(C.POINTER(C.c_double)), None) == 0
    L.hmgpu_tree_free(h)
    np.testing.assert_array_equal(imap, host.index_map)
    np.testing.assert_array_equal(center.view(np.int64), host._center.view(np.int64))


@pytest.mark.parametrize("bad", ["coincident", "nan"])
def test_device_tree_fails_like_host(gpu, bad):
    P = geometry.cube(500, seed=12)
    if bad == "coincident":
        P[:, 100:200] = P[:, [7]]  # 101 equal points, more than a leaf holds
    else:
        P[1, 33] = np.nan
    codes = []
    for gpu_build in (False, True):
        with pytest.raises(hmgpu.HMGPUError) as e:
            hmgpu.ClusterTree(P, max_points_per_leaf=16, gpu=gpu_build)
        codes.append(e.value.code)
    assert codes[0] == codes[1] == -4  # HMGPU_ERR_TREE


def test_device_tree_rejects_bad_arguments(gpu):
    P = geometry.cube(100, seed=13)
    with pytest.raises(hmgpu.HMGPUError):
        hmgpu.ClusterTree(P, max_points_per_leaf=0, gpu=True)
    with pytest.raises(ValueError):
        hmgpu.ClusterTree(P, max_points_per_leaf=8, dims=0, gpu=True)


def test_device_tree_hmatrix_identical(gpu):
    """An H-matrix over the device-built tree is the same operator, bit for bit."""
    import torch
    P = geometry.sphere(4000, seed=14)
    Th = hmgpu.ClusterTree(P, max_points_per_leaf=32)
    Td = hmgpu.ClusterTree(P, max_points_per_leaf=32, gpu=True)
    K = hmgpu.Kernel("laplace", P)
    Hh = hmgpu.HMatrix(K, Th, Th, eta=1.5, eps=1e-6, precision="f64")
    Hd = hmgpu.HMatrix(K, Td, Td, eta=1.5, eps=1e-6, precision="f64")
    x = torch.randn(P.shape[1], device=gpu, dtype=torch.float64)
    assert torch.equal(Hh * x, Hd * x)


def _same_blocks(a, b):
    for name in ("_target", "_source", "_adm", "_dense", "_left", "_right", "_dense_pairs", "_approx_pairs"):
        np.testing.assert_array_equal(getattr(a, name), getattr(b, name), err_msg=name)


BLOCK_CASES = [
    ("sphere_square", lambda: geometry.sphere(3000, seed=1), None, 32, 1.5),
    ("cube_eta1", lambda: geometry.cube(8000, seed=2), None, 16, 1.0),
    ("cube_eta3", lambda: geometry.cube(8000, seed=2), None, 16, 3.0),
    ("film_lattice", lambda: geometry.film(128, 128, jitter=0.0, seed=3), None, 64, 2.0),
    ("rect_cube_sphere", lambda: geometry.cube(5000, seed=4), lambda: geometry.sphere(3000, seed=5), 24, 1.5),
    ("rect_small_big", lambda: geometry.cube(100, seed=6), lambda: geometry.cube(9000, seed=7), 8, 1.0),
    ("single_leaf", lambda: geometry.cube(20, seed=8), None, 32, 1.5),
    ("eta0", lambda: geometry.sphere(1500, seed=9), None, 16, 0.0),
]


@pytest.mark.parametrize("merge", [False, True])
@pytest.mark.parametrize("name,px,py,leaf,eta", BLOCK_CASES, ids=[c[0] for c in BLOCK_CASES])
def test_device_blocks_match_host(gpu, name, px, py, leaf, eta, merge):
    X = hmgpu.ClusterTree(px(), max_points_per_leaf=leaf)
    Y = X if py is None else hmgpu.ClusterTree(py(), max_points_per_leaf=leaf)
    host = hmgpu.BlockTree(X, Y, eta=eta, merge=merge)
    dev = hmgpu.BlockTree(X, Y, eta=eta, merge=merge, gpu=True)
    _same_blocks(host, dev)


def test_device_blocks_full_size(gpu):
    """Block tree of the 2^20-point film (eta 2, merged, as the H-matrix build
    uses it), timed beside the host build."""
    P = geometry.film(1024, 1024, seed=1)
    T = hmgpu.ClusterTree(P, max_points_per_leaf=64, gpu=True)
    hmgpu.BlockTree(T, T, eta=2.0, merge=True, gpu=True)  # first use of the kernels
    t0 = time.perf_counter()
    dev = hmgpu.BlockTree(T, T, eta=2.0, merge=True, gpu=True)
    t1 = time.perf_counter()
    host = hmgpu.BlockTree(T, T, eta=2.0, merge=True)
    t2 = time.perf_counter()
    _same_blocks(host, dev)
    print(f"\nblock tree of 2^20 points ({len(dev._target)} nodes): device {1e3 * (t1 - t0):.1f} ms, "
          f"host {1e3 * (t2 - t1):.1f} ms")
