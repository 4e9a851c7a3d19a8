"""ctypes wrapper of the oracle -- TEST INFRASTRUCTURE ONLY.

The oracle is a CPU FP64 restatement of HMatrixGPU.jl's H-matrix path
(src/tree.jl, src/block.jl, src/aca.jl, src/hmatrix.jl, src/mult.jl).  Only
tests, the smoke check and bench.py's CPU-baseline legs use it, as the checker
or as the timed CPU baseline; the product never imports it.

Parity: pinned by the reference's own known-answer tests (restated in tests/);
bit-level agreement with Julia's LAPACK/BLAS calls is not claimed.
"""
import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

I64P = C.POINTER(C.c_int64)
F64P = C.POINTER(C.c_double)
I8P = C.POINTER(C.c_int8)

KERNELS = {"explicit": 0, "laplace": 1, "yukawa": 2, "log2d": 3, "vector_r": 4, "dipolar": 5}


class _Kernel(C.Structure):
    _fields_ = [("type", C.c_int32), ("nrows", C.c_int64), ("ncols", C.c_int64),
                ("X", F64P), ("Y", F64P), ("A", F64P), ("lda", C.c_int64)]


def build():
    """Compile liboracle.so with the committed Makefile."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        L = C.CDLL(path)
        L.or_cluster_tree.argtypes = [F64P, C.c_int64, C.c_int64, C.c_int64, C.POINTER(C.c_void_p)]
        L.or_tree_num_nodes.argtypes = [C.c_void_p]
        L.or_tree_num_nodes.restype = C.c_int64
        L.or_tree_index_len.argtypes = [C.c_void_p]
        L.or_tree_index_len.restype = C.c_int64
        L.or_tree_export.argtypes = [C.c_void_p, I64P, I64P, I64P, I8P, I64P, I64P, F64P, F64P]
        L.or_tree_free.argtypes = [C.c_void_p]
        L.or_block_tree.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_int, C.POINTER(C.c_void_p)]
        for f in ("or_blocks_num_dense", "or_blocks_num_approx", "or_blocks_num_nodes"):
            getattr(L, f).argtypes = [C.c_void_p]
            getattr(L, f).restype = C.c_int64
        L.or_blocks_export.argtypes = [C.c_void_p, I64P, I64P]
        L.or_blocks_export_nodes.argtypes = [C.c_void_p, I64P, I64P, I8P, I8P, I64P, I64P]
        L.or_blocks_free.argtypes = [C.c_void_p]
        L.or_kernel_entry.argtypes = [C.POINTER(_Kernel), C.c_int64, C.c_int64]
        L.or_kernel_entry.restype = C.c_double
        L.or_kernel_matvec.argtypes = [C.POINTER(_Kernel), F64P, F64P]
        L.or_sparsify.argtypes = [C.POINTER(_Kernel), C.c_void_p, C.c_void_p, C.c_double, I64P, I64P, F64P]
        L.or_sparsify.restype = C.c_int64
        L.or_aca_plus.argtypes = [C.POINTER(_Kernel), I64P, C.c_int64, I64P, C.c_int64, C.c_double,
                                  C.c_int64, C.c_int64, F64P, F64P, I64P]
        L.or_svd_recompress.argtypes = [C.c_int64, C.c_int64, C.c_int64, F64P, F64P, C.c_double,
                                        F64P, F64P, I64P]
        L.or_qr.argtypes = [C.c_int64, C.c_int64, F64P, F64P, F64P, C.c_int]
        L.or_jacobi_svd.argtypes = [C.c_int64, F64P, F64P, F64P, I64P]
        L.or_hmatrix_build.argtypes = [C.POINTER(_Kernel), C.c_void_p, C.c_void_p, C.c_double,
                                       C.c_double, C.c_int, C.c_int64, C.c_int, C.POINTER(C.c_void_p)]
        L.or_hmatrix_sizes.argtypes = [C.c_void_p] + [I64P] * 8
        L.or_hmatrix_export.argtypes = [C.c_void_p, I64P, I64P, I64P, I64P, I64P, F64P, F64P, F64P]
        L.or_hmatrix_aca_ranks.argtypes = [C.c_void_p, I64P, I64P]
        L.or_hmatrix_num_approx_candidates.argtypes = [C.c_void_p]
        L.or_hmatrix_num_approx_candidates.restype = C.c_int64
        L.or_hmatrix_free.argtypes = [C.c_void_p]
        L.or_mul_cpu.argtypes = [C.c_void_p, F64P, F64P, C.c_int]
        L.or_mul_cpu_timed.argtypes = [C.c_void_p, F64P, F64P, C.c_int, C.c_int]
        L.or_mul_cpu_timed.restype = C.c_double
        L.or_mul_flat.argtypes = [C.c_void_p, F64P, F64P, F64P]
        L.or_cpu_mul_plan.argtypes = [C.c_void_p, C.c_int]
        L.or_cpu_mul_plan.restype = C.c_void_p
        L.or_cpu_mul_run.argtypes = [C.c_void_p, F64P, F64P, C.c_int]
        L.or_cpu_mul_run.restype = C.c_double
        L.or_cpu_mul_free.argtypes = [C.c_void_p]
        L.or_hmatrix_stored_entries.argtypes = [C.c_void_p]
        L.or_hmatrix_stored_entries.restype = C.c_int64
        _LIB = L
    return _LIB


def _p(a, t=F64P):
    return a.ctypes.data_as(t)


class Kernel:
    """Matrix entry source: a named kernel over target/source points, or an explicit matrix."""

    def __init__(self, kind, X=None, Y=None, A=None):
        self.kind = kind
        if kind == "explicit":
            self.A = np.asfortranarray(A, dtype=np.float64)
            self.shape = self.A.shape
            self.X = self.Y = None
        else:
            # (N, 3) C-contiguous == Julia's 3 x N column-major coordinates
            self.X = np.ascontiguousarray(np.asarray(X, dtype=np.float64))
            self.Y = np.ascontiguousarray(np.asarray(Y if Y is not None else X, dtype=np.float64))
            nx, ny = self.X.shape[0], self.Y.shape[0]
            if kind == "vector_r":
                self.shape = (nx, 3 * ny)
            elif kind == "dipolar":
                self.shape = (3 * nx, 3 * ny)
            else:
                self.shape = (nx, ny)
            self.A = None
        k = _Kernel()
        k.type = KERNELS[kind]
        k.nrows, k.ncols = self.shape
        if self.A is not None:
            k.A = _p(self.A)
            k.lda = self.shape[0]
        else:
            k.X = _p(self.X)
            k.Y = _p(self.Y)
        self._k = k

    def entry(self, i, j):
        """K[i, j] with 1-based indices."""
        return lib().or_kernel_entry(C.byref(self._k), int(i), int(j))

    def dense(self):
        m, n = self.shape
        return np.array([[self.entry(i, j) for j in range(1, n + 1)] for i in range(1, m + 1)])

    def matvec(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty(self.shape[0])
        lib().or_kernel_matvec(C.byref(self._k), _p(x), _p(y))
        return y


class Tree:
    """ClusterTree (src/tree.jl:45-67). `points` is (N, 3)."""

    def __init__(self, points, max_points_per_leaf=32, dims=1):
        pts = np.ascontiguousarray(np.asarray(points, dtype=np.float64))
        assert pts.ndim == 2 and pts.shape[1] == 3
        h = C.c_void_p()
        rc = lib().or_cluster_tree(_p(pts), pts.shape[0], max_points_per_leaf, dims, C.byref(h))
        if rc != 0:
            raise ValueError(f"or_cluster_tree failed ({rc})")
        self._h = h
        self._pts = pts
        L = lib()
        nn = L.or_tree_num_nodes(h)
        il = L.or_tree_index_len(h)
        self.index_map = np.empty(il, np.int64)
        self.start = np.empty(nn, np.int64)
        self.end = np.empty(nn, np.int64)
        self.is_leaf = np.empty(nn, np.int8)
        self.left = np.empty(nn, np.int64)
        self.right = np.empty(nn, np.int64)
        self.center = np.empty((nn, 3))
        self.radius = np.empty(nn)
        L.or_tree_export(h, _p(self.index_map, I64P), _p(self.start, I64P), _p(self.end, I64P),
                         _p(self.is_leaf, I8P), _p(self.left, I64P), _p(self.right, I64P),
                         _p(self.center), _p(self.radius))

    def __del__(self):
        if getattr(self, "_h", None) and _LIB is not None:
            _LIB.or_tree_free(self._h)
            self._h = None


class Blocks:
    """BlockTree + merge_dense_matrices! + traverse (src/block.jl)."""

    def __init__(self, X, Y, eta=1.5, merge=True):
        L = lib()
        h = C.c_void_p()
        L.or_block_tree(X._h, Y._h, eta, int(merge), C.byref(h))
        nd, na, nn = L.or_blocks_num_dense(h), L.or_blocks_num_approx(h), L.or_blocks_num_nodes(h)
        self.dense = np.empty((nd, 2), np.int64)
        self.approx = np.empty((na, 2), np.int64)
        L.or_blocks_export(h, _p(self.dense, I64P), _p(self.approx, I64P))
        self.node_target = np.empty(nn, np.int64)
        self.node_source = np.empty(nn, np.int64)
        self.node_adm = np.empty(nn, np.int8)
        self.node_dense = np.empty(nn, np.int8)
        self.node_left = np.empty(nn, np.int64)
        self.node_right = np.empty(nn, np.int64)
        L.or_blocks_export_nodes(h, _p(self.node_target, I64P), _p(self.node_source, I64P),
                                 _p(self.node_adm, I8P), _p(self.node_dense, I8P),
                                 _p(self.node_left, I64P), _p(self.node_right, I64P))
        L.or_blocks_free(h)


def sparsify(K, X, Y, eta=1.5):
    """sparsify_hmatrix (src/hmatrix.jl:234-274) as its (I, J, V) triplets:
    1-based original indices and K entries of every dense leaf, in the order
    the reference pushes them."""
    L = lib()
    n = L.or_sparsify(C.byref(K._k), X._h, Y._h, float(eta), None, None, None)
    I = np.empty(n, np.int64)
    J = np.empty(n, np.int64)
    V = np.empty(n)
    L.or_sparsify(C.byref(K._k), X._h, Y._h, float(eta), _p(I, I64P), _p(J, I64P), _p(V))
    return I, J, V


def aca_plus(K, rows, cols, eps, max_iter=0):
    """ACA_plus on K[rows, cols] (1-based original indices). Returns (U m x k, V k x n)."""
    rows = np.ascontiguousarray(rows, dtype=np.int64)
    cols = np.ascontiguousarray(cols, dtype=np.int64)
    m, n = len(rows), len(cols)
    cap = min(m, n)
    U = np.zeros((m, cap), order="F")
    V = np.zeros((cap, n), order="F")
    k = C.c_int64()
    rc = lib().or_aca_plus(C.byref(K._k), _p(rows, I64P), m, _p(cols, I64P), n, eps, max_iter,
                           cap, _p(U), _p(V), C.byref(k))
    assert rc == 0
    return np.array(U[:, :k.value]), np.array(V[:k.value, :])


def svd_recompress(U, V, eps):
    """SVD_recompress (src/aca.jl:123-143)."""
    U = np.asfortranarray(U, dtype=np.float64)
    V = np.asfortranarray(V, dtype=np.float64)
    m, k = U.shape
    n = V.shape[1]
    Uo = np.zeros((m, max(k, 1)), order="F")
    Vo = np.zeros((max(k, 1), n), order="F")
    r = C.c_int64()
    rc = lib().or_svd_recompress(m, n, k, _p(U), _p(V), eps, _p(Uo), _p(Vo), C.byref(r))
    assert rc == 0
    r = r.value
    Vo = np.asfortranarray(Vo.reshape(-1, order="F")[: r * n].reshape(r, n, order="F"))
    return np.array(Uo[:, :r]), np.array(Vo)


class HMatrix:
    """HMatrix assembly (src/hmatrix.jl:72-217) with the flattened fields of
    HMatrix{T} (src/hmatrix.jl:46-57) exported as numpy arrays (1-based)."""

    def __init__(self, K, X, Y, eta=1.5, eps=1e-5, svd_recompress=True, sample_stride=1,
                 nthreads=1):
        L = lib()
        h = C.c_void_p()
        L.or_hmatrix_build(C.byref(K._k), X._h, Y._h, eta, eps, int(svd_recompress),
                           sample_stride, nthreads, C.byref(h))
        self._h = h
        self.K = K
        s = [C.c_int64() for _ in range(8)]
        L.or_hmatrix_sizes(h, *[C.byref(v) for v in s])
        self.m, self.n, self.nD, self.nA, self.R, dl, ul, vl = [v.value for v in s]
        self.target_index_map = np.empty(len(X.index_map), np.int64)
        self.source_index_map = np.empty(len(Y.index_map), np.int64)
        self.dense_block_indices = np.zeros((self.nD, 5), np.int64)
        self.U_block_indices = np.zeros((self.nA, 5), np.int64)
        self.V_block_indices = np.zeros((self.R, 3), np.int64)
        self.dense_blocks = np.zeros(dl)
        self.U_matrices = np.zeros(ul)
        self.V_matrices = np.zeros(vl)
        L.or_hmatrix_export(h, _p(self.target_index_map, I64P), _p(self.source_index_map, I64P),
                            _p(self.dense_block_indices, I64P), _p(self.U_block_indices, I64P),
                            _p(self.V_block_indices, I64P), _p(self.dense_blocks),
                            _p(self.U_matrices), _p(self.V_matrices))
        nc = L.or_hmatrix_num_approx_candidates(h)
        self.aca_ranks = np.empty(nc, np.int64)
        self.final_ranks = np.empty(nc, np.int64)
        L.or_hmatrix_aca_ranks(h, _p(self.aca_ranks, I64P), _p(self.final_ranks, I64P))

    def __del__(self):
        if getattr(self, "_h", None) and _LIB is not None:
            _LIB.or_hmatrix_free(self._h)
            self._h = None

    def mul(self, x, nthreads=1):
        """CPU mul! (src/mult.jl:6-32)."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty(self.m)
        lib().or_mul_cpu(self._h, _p(x), _p(y), nthreads)
        return y

    def mul_timed(self, x, nthreads=1, reps=1):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty(self.m)
        return lib().or_mul_cpu_timed(self._h, _p(x), _p(y), nthreads, reps)

    def stored_entries(self):
        """FP64 entries stored in all blocks (each read once per product)."""
        return lib().or_hmatrix_stored_entries(self._h)

    def timed_product(self, nthreads=1):
        """A CpuProduct: the timed CPU baseline on this matrix (cpu_mul.c)."""
        return CpuProduct(self, nthreads)

    def mul_flat(self, x):
        """Flattened mul! semantics (src/mult.jl:41-146); returns (y, Vx)."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty(self.m)
        vx = np.empty(max(self.R, 1))
        lib().or_mul_flat(self._h, _p(x), _p(y), _p(vx))
        return y, vx[: self.R]

    def info(self):
        """info(::HMatrixCPU) (src/hmatrix.jl:289-330)."""
        d = self.dense_block_indices
        dsz = (d[:, 1] - d[:, 0] + 1) * (d[:, 3] - d[:, 2] + 1)
        u = self.U_block_indices
        ranks = u[:, 3] - u[:, 2] + 1 if self.nA else np.zeros(0, np.int64)
        comp = dsz.sum() + len(self.U_matrices) + len(self.V_matrices)
        return {"size": (self.m, self.n), "leaves": self.nD + self.nA,
                "admissible_leaves": self.nA, "full_leaves": self.nD,
                "min_rank": int(ranks.min()) if len(ranks) else 0,
                "max_rank": int(ranks.max()) if len(ranks) else 0,
                "min_dense_size": int(dsz.min()), "max_dense_size": int(dsz.max()),
                "compression_ratio": self.m * self.n / comp}


class CpuProduct:
    """The reference's CPU mul! (src/mult.jl:6-32) shaped as Julia runs it, with
    BLAS-like dot products, on `nthreads` threads (cpu_mul.c). Timing only: the
    checker is HMatrix.mul."""

    def __init__(self, H, nthreads=1):
        self.H = H
        self.nthreads = int(nthreads)
        self._p = lib().or_cpu_mul_plan(H._h, self.nthreads)

    def run(self, x, reps=1):
        """(seconds for `reps` whole products, y of the last one)."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty(self.H.m)
        dt = lib().or_cpu_mul_run(self._p, _p(x), _p(y), int(reps))
        return dt, y

    def __del__(self):
        if getattr(self, "_p", None) and _LIB is not None:
            _LIB.or_cpu_mul_free(self._p)
            self._p = None
