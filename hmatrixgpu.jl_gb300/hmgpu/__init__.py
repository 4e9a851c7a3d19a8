"""hmgpu -- Python face of libhmgpu, mirroring HMatrixGPU.jl's API.

    ClusterTree(coordinates; max_points_per_leaf=32, dims=1)   src/tree.jl:45
    info(tree)                                                  src/tree.jl:153
    BlockTree(X, Y; eta=1.5)                                    src/block.jl:31
    traverse(block_tree)                                        src/block.jl:127
    ACA_plus(n_rows, n_cols, calc_rows, calc_cols, eps)         src/aca.jl:36
    SVD_recompress(U, V, eps)                                   src/aca.jl:123
    HMatrix(K, X, Y; eta=1.5, eps=1e-5, ...)                    src/hmatrix.jl:72
    info(hmatrix)                                               src/hmatrix.jl:289
    mul_(y, H, x)   == mul!(y, H, x)                            src/mult.jl:159
    H * x, H @ x                                                src/mult.jl:203

Coordinates are 3 x N arrays (one column per point) as in the reference.  All
compute runs in libhmgpu (CUDA, sm_103a); the tree and partition are the
library's host code.  Nothing here falls back to another implementation: if
the library cannot be loaded or a GPU is missing, the call raises.
"""
import ctypes as C

import numpy as np

from ._lib import (F64, F32, MIXED, PRECISIONS, KERNEL_IDS, HMGPUError, Info, KernelDesc,
                   Options, I64P, I8P, F32P, F64P, check, lib, ptr)
from . import _build

__all__ = ["ClusterTree", "BlockTree", "ACA_plus", "SVD_recompress", "HMatrix", "Kernel", "info",
           "traverse", "mul_", "HMGPUError", "build", "RankModel", "block_features", "batch", "Graph",
           "sparsify_hmatrix"]


def build(verbose=False):
    """Compiles libhmgpu.so (sm_103a) in-tree."""
    return _build.build(verbose=verbose)


def _coords(coordinates):
    a = np.asarray(coordinates, dtype=np.float64)
    if a.ndim != 2 or a.shape[0] != 3:
        raise ValueError("coordinates must be a 3 x N array (one column per point)")
    return np.asfortranarray(a)


class ClusterNode:
    """View of one node of a ClusterTree (src/tree.jl:6-14)."""

    __slots__ = ("tree", "id")

    def __init__(self, tree, i):
        self.tree, self.id = tree, int(i)

    is_leaf = property(lambda s: bool(s.tree._leaf[s.id]))
    start_idx = property(lambda s: int(s.tree._start[s.id]))
    end_idx = property(lambda s: int(s.tree._end[s.id]))
    center = property(lambda s: s.tree._center[s.id].copy())
    radius = property(lambda s: float(s.tree._radius[s.id]))
    left = property(lambda s: ClusterNode(s.tree, s.tree._left[s.id]) if s.tree._left[s.id] >= 0 else None)
    right = property(lambda s: ClusterNode(s.tree, s.tree._right[s.id]) if s.tree._right[s.id] >= 0 else None)


class ClusterTree:
    """ClusterTree(coordinates; max_points_per_leaf=32, dims=1) (src/tree.jl:45-67).

    gpu=True builds the same tree (bit for bit) on the current CUDA device."""

    def __init__(self, coordinates, max_points_per_leaf=32, dims=1, gpu=False):
        if dims <= 0:
            raise ValueError("Parameter `dims` must be a positive integer.")
        self.coordinates = _coords(coordinates)
        L = lib()
        h = C.c_void_p()
        if gpu:
            check(L.hmgpu_tree_build_device(self.coordinates.ctypes.data, self.coordinates.shape[1],
                                            int(max_points_per_leaf), int(dims), C.byref(h)))
        else:
            check(L.hmgpu_tree_build(ptr(self.coordinates), self.coordinates.shape[1],
                                     int(max_points_per_leaf), int(dims), C.byref(h)))
        self._h = h
        self.dims = dims
        self.max_points_per_leaf = max_points_per_leaf
        v = [C.c_int64() for _ in range(5)]
        check(L.hmgpu_tree_info(h, *[C.byref(x) for x in v]))
        nn, il, self._depth, self._maxp, self._minp = [x.value for x in v]
        self.index_map = np.empty(il, np.int64)
        self._start = np.empty(nn, np.int64)
        self._end = np.empty(nn, np.int64)
        self._leaf = np.empty(nn, np.int8)
        self._left = np.empty(nn, np.int64)
        self._right = np.empty(nn, np.int64)
        self._center = np.empty((nn, 3))
        self._radius = np.empty(nn)
        check(L.hmgpu_tree_export(h, ptr(self.index_map, I64P), ptr(self._start, I64P),
                                  ptr(self._end, I64P), ptr(self._leaf, I8P), ptr(self._left, I64P),
                                  ptr(self._right, I64P), ptr(self._center), ptr(self._radius)))

    @property
    def root(self):
        return ClusterNode(self, 0)

    @property
    def num_nodes(self):
        return len(self._start)

    def info(self):
        """info(::ClusterTree) (src/tree.jl:153-187)."""
        return {"depth": self._depth, "max_points": self._maxp, "min_points": self._minp}

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().hmgpu_tree_free(h)
            self._h = None


class BlockTreeNode:
    """View of one node of a BlockTree (src/block.jl:2-9)."""

    __slots__ = ("bt", "id")

    def __init__(self, bt, i):
        self.bt, self.id = bt, int(i)

    target_tree = property(lambda s: ClusterNode(s.bt.X, s.bt._target[s.id]))
    source_tree = property(lambda s: ClusterNode(s.bt.Y, s.bt._source[s.id]))
    is_admissible = property(lambda s: bool(s.bt._adm[s.id]))
    is_dense = property(lambda s: bool(s.bt._dense[s.id]))
    left = property(lambda s: BlockTreeNode(s.bt, s.bt._left[s.id]) if s.bt._left[s.id] >= 0 else None)
    right = property(lambda s: BlockTreeNode(s.bt, s.bt._right[s.id]) if s.bt._right[s.id] >= 0 else None)


class BlockTree:
    """BlockTree(X, Y; eta=1.5) (src/block.jl:31-44). `merge=True` also applies
    merge_dense_matrices! (src/block.jl:98-112) as HMatrix does. gpu=True
    builds the same tree (bit for bit) on the current CUDA device."""

    def __init__(self, X, Y, eta=1.5, merge=False, gpu=False):
        self.X, self.Y, self.eta = X, Y, eta
        L = lib()
        h = C.c_void_p()
        build = L.hmgpu_blocks_build_device if gpu else L.hmgpu_blocks_build
        check(build(X._h, Y._h, float(eta), int(bool(merge)), C.byref(h)))
        try:
            v = [C.c_int64() for _ in range(3)]
            check(L.hmgpu_blocks_counts(h, *[C.byref(x) for x in v]))
            nd, na, nn = [x.value for x in v]
            self._dense_pairs = np.empty((nd, 2), np.int64)
            self._approx_pairs = np.empty((na, 2), np.int64)
            check(L.hmgpu_blocks_export(h, ptr(self._dense_pairs, I64P), ptr(self._approx_pairs, I64P)))
            self._target = np.empty(nn, np.int64)
            self._source = np.empty(nn, np.int64)
            self._adm = np.empty(nn, np.int8)
            self._dense = np.empty(nn, np.int8)
            self._left = np.empty(nn, np.int64)
            self._right = np.empty(nn, np.int64)
            check(L.hmgpu_blocks_export_nodes(h, ptr(self._target, I64P), ptr(self._source, I64P),
                                              ptr(self._adm, I8P), ptr(self._dense, I8P),
                                              ptr(self._left, I64P), ptr(self._right, I64P)))
        finally:
            L.hmgpu_blocks_free(h)
        self.target_index_map = X.index_map
        self.source_index_map = Y.index_map

    @property
    def root(self):
        return BlockTreeNode(self, 0)

    def traverse(self):
        """traverse(block_tree) (src/block.jl:127-155): (direct_list, approx_list)
        of (target ClusterNode, source ClusterNode) pairs."""
        d = [(ClusterNode(self.X, a), ClusterNode(self.Y, b)) for a, b in self._dense_pairs]
        a = [(ClusterNode(self.X, x), ClusterNode(self.Y, y)) for x, y in self._approx_pairs]
        return d, a


def traverse(block_tree):
    return block_tree.traverse()


def ACA_plus(n_rows, n_cols, calc_rows, calc_cols, eps, max_iter=None):
    """ACA_plus(n_rows, n_cols, calc_rows, calc_cols, eps; max_iter=n_rows)
    (src/aca.jl:36-106). The row callbacks are evaluated once per row to place
    the block on the device; the partially pivoted ACA+ then runs in the
    library's batched device kernel. Returns (U n_rows x k, V k x n_cols)."""
    A = np.empty((n_rows, n_cols), order="F")
    for i in range(n_rows):
        A[i, :] = np.asarray(calc_rows(i + 1), dtype=np.float64).reshape(-1)
    mi = int(max_iter) if max_iter is not None else 0
    cap = max(1, min(n_rows, n_cols, mi if mi > 0 else n_rows))
    U = np.zeros((n_rows, cap), order="F")
    V = np.zeros((cap, n_cols), order="F")
    k = C.c_int64()
    check(lib().hmgpu_aca_plus(ptr(A), n_rows, n_rows, n_cols, float(eps), mi, cap, ptr(U), ptr(V),
                               C.byref(k)))
    k = k.value
    return np.array(U[:, :k]), np.array(V[:k, :])


def SVD_recompress(U, V, eps):
    """SVD_recompress(U, V, eps) (src/aca.jl:123-143), FP64 on the device."""
    U = np.asfortranarray(U, dtype=np.float64)
    V = np.asfortranarray(V, dtype=np.float64)
    m, k = U.shape
    n = V.shape[1]
    Uo = np.zeros((m, max(k, 1)), order="F")
    Vo = np.zeros(max(k, 1) * n)
    r = C.c_int64()
    check(lib().hmgpu_svd_recompress(m, n, k, ptr(U), ptr(V), float(eps), ptr(Uo), ptr(Vo), C.byref(r)))
    r = r.value
    return np.array(Uo[:, :r]), np.array(Vo[: r * n].reshape((r, n), order="F"))


class UserKernel:
    """A kernel K[i, j] = f(x_i, y_j) of the caller's own: CUDA C++ source that
    defines ``__device__ double hmgpu_entry(const double *x, const double *y,
    const double *p, int a, int b)`` (target point x, source point y, 3
    coordinates each; p the parameters given to Kernel('user', ...); a, b the
    components of a vector or tensor kernel over trees with dims 3, 0 for a
    scalar kernel), compiled at run time with
    NVRTC into the library's ACA+, dense-block and sparsify kernels
    (hmgpu_user_kernel_compile). A compile error raises HMGPUError with the
    compiler's log in ``.log``."""

    def __init__(self, source):
        self._h = C.c_void_p()
        buf = C.create_string_buffer(1 << 16)
        rc = lib().hmgpu_user_kernel_compile(source.encode(), C.byref(self._h), buf, len(buf))
        self.log = buf.value.decode(errors="replace")
        if rc != 0:
            err = HMGPUError(rc, lib().hmgpu_last_error().decode())
            err.log = self.log
            raise err
        self.source = source

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            lib().hmgpu_user_kernel_free(h)
            self._h = None


_USER_KERNELS = {}  # source -> UserKernel compiled from it


class Kernel:
    """A matrix K generated on the device: kind in {'laplace', 'yukawa', 'log2d',
    'vector_r', 'dipolar'} over target points X and source points Y (3 x N),
    'explicit' with a dense matrix A, or 'user' with a UserKernel (or its
    source) and up to 64 parameters."""

    def __init__(self, kind, X=None, Y=None, A=None, user=None, params=()):
        if kind not in KERNEL_IDS:
            raise ValueError(f"unknown kernel {kind!r}")
        self.kind = kind
        self.user = None
        self.params = np.ascontiguousarray(params, dtype=np.float64).reshape(-1)
        if kind == "user":
            if user is None:
                raise ValueError("a 'user' kernel needs user= (a UserKernel or its source)")
            if not isinstance(user, UserKernel):  # one compilation per source
                if user not in _USER_KERNELS:
                    _USER_KERNELS[user] = UserKernel(user)
                user = _USER_KERNELS[user]
            self.user = user
        if kind == "explicit":
            self.A = np.asfortranarray(A, dtype=np.float64)
            self.X = self.Y = None
            self.shape = self.A.shape
        else:
            self.X = _coords(X)
            self.Y = _coords(X if Y is None else Y)
            nx, ny = self.X.shape[1], self.Y.shape[1]
            # (a user kernel's rows and columns per point come from the trees' dims)
            self.shape = {"vector_r": (nx, 3 * ny), "dipolar": (3 * nx, 3 * ny)}.get(kind, (nx, ny))
            self.A = None

    def desc(self):
        d = KernelDesc()
        d.kind = KERNEL_IDS[self.kind]
        if self.A is not None:
            d.A = ptr(self.A)
            d.lda = self.shape[0]
        else:
            d.X = ptr(self.X)
            d.nX = self.X.shape[1]
            d.Y = ptr(self.Y)
            d.nY = self.Y.shape[1]
        if self.user is not None:
            d.user = self.user._h
            d.params = ptr(self.params) if self.params.size else None
            d.nparams = self.params.size
        return d

    def size(self):
        return self.shape


def _opts(precision, compensated, keep_factors, rank_model=None, lean=False):
    o = Options()
    o.precision = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
    o.compensated = int(bool(compensated))
    o.keep_factors = int(bool(keep_factors))
    o.lean = int(bool(lean))
    o.rank_model = rank_model._h if rank_model is not None else None
    return o


def block_features(X, Y, eta, eps):
    """Rank-predictor features (n, 8) of the admissible leaves of BlockTree(X, Y; eta)
    in traversal order (the order of HMatrix.aca_ranks())."""
    n = C.c_int64()
    check(lib().hmgpu_block_features(X._h, Y._h, float(eta), float(eps), None, C.byref(n)))
    out = np.zeros((n.value, 8), np.float32)
    check(lib().hmgpu_block_features(X._h, Y._h, float(eta), float(eps), ptr(out, F32P), C.byref(n)))
    return out


class RankModel:
    """The learned ACA-rank predictor (8 -> 64 -> 64 -> 1 ReLU MLP, FP32), trained
    and evaluated by libhmgpu's kernels; passed to HMatrix(..., rank_model=M) it
    sizes and batches the ACA work (results never depend on it)."""

    NPARAMS = 4801

    def __init__(self, seed=0):
        h = C.c_void_p()
        check(lib().hmgpu_rank_model_create(int(seed), C.byref(h)))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().hmgpu_rank_model_free(h)
            self._h = None

    def train(self, X, y, epochs=50, batch=1024, lr=1e-3, seed=0):
        X = np.ascontiguousarray(X, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        loss = C.c_float()
        check(lib().hmgpu_rank_model_train(self._h, ptr(X, F32P), ptr(y, F32P), len(y), int(epochs),
                                           int(batch), float(lr), int(seed), C.byref(loss)))
        return loss.value

    def predict(self, X):
        X = np.ascontiguousarray(X, np.float32)
        out = np.zeros(len(X), np.float32)
        check(lib().hmgpu_rank_model_predict(self._h, ptr(X, F32P), len(X), ptr(out, F32P)))
        return out

    def gradients(self, X, y):
        X = np.ascontiguousarray(X, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        g = np.zeros(self.NPARAMS, np.float32)
        loss = C.c_float()
        check(lib().hmgpu_rank_model_gradients(self._h, ptr(X, F32P), ptr(y, F32P), len(y), ptr(g, F32P),
                                               C.byref(loss)))
        return g, loss.value

    def params(self, set_params=None, set_norm=None):
        p = np.zeros(self.NPARAMS, np.float32)
        nm = np.zeros(16, np.float32)
        sp = np.ascontiguousarray(set_params, np.float32) if set_params is not None else None
        sn = np.ascontiguousarray(set_norm, np.float32) if set_norm is not None else None
        check(lib().hmgpu_rank_model_params(self._h, ptr(p, F32P), ptr(sp, F32P) if sp is not None else None,
                                            ptr(nm, F32P), ptr(sn, F32P) if sn is not None else None))
        return p, nm


class HMatrix:
    """HMatrix(K, X, Y; eta=1.5, eps=1e-5, svd_recompress=True) (src/hmatrix.jl:72-148),
    assembled on the device, stored in `precision` ('f64', 'f32' or 'mixed');
    with 'mixed', lean=True keeps only the tensor-core copy (half the memory;
    every product on the tensor cores)."""

    def __init__(self, K, X, Y, eta=1.5, eps=1e-5, svd_recompress=True, precision="f64",
                 compensated=False, keep_factors=False, rank_model=None, lean=False, _handle=None):
        self._h = None
        if _handle is not None:
            self._h = _handle
        else:
            if not isinstance(K, Kernel):
                K = Kernel("explicit", A=K)
            self.K = K
            o = _opts(precision, compensated, keep_factors, rank_model, lean)
            h = C.c_void_p()
            d = K.desc()
            check(lib().hmgpu_hmatrix_build(C.byref(o), C.byref(d), X._h, Y._h, float(eta),
                                             float(eps), int(bool(svd_recompress)), C.byref(h)))
            self._h = h
        self._load_meta()

    @classmethod
    def from_flat(cls, m, n, target_index_map, source_index_map, dense_block_indices, dense_blocks,
                  U_block_indices, U_matrices, V_block_indices, V_matrices, precision="f64",
                  compensated=False, keep_factors=False, lean=False):
        """Imports the reference's flattened HMatrix{Float64} fields
        (src/hmatrix.jl:46-57): index tables as (nblocks, 5) / (R, 3) arrays of
        the 1-based Julia columns."""
        a64 = lambda a: np.ascontiguousarray(a, dtype=np.int64)
        f64 = lambda a: np.ascontiguousarray(a, dtype=np.float64).reshape(-1)
        tm, sm = a64(target_index_map), a64(source_index_map)
        di, ui, vi = a64(dense_block_indices), a64(U_block_indices), a64(V_block_indices)
        dd, ud, vd = f64(dense_blocks), f64(U_matrices), f64(V_matrices)
        o = _opts(precision, compensated, keep_factors, lean=lean)
        h = C.c_void_p()
        check(lib().hmgpu_hmatrix_import_flat(
            C.byref(o), m, n, ptr(tm, I64P), ptr(sm, I64P), ptr(di, I64P), di.shape[0] if di.size else 0,
            ptr(dd), dd.size, ptr(ui, I64P), ui.shape[0] if ui.size else 0, ptr(ud), ud.size,
            ptr(vi, I64P), vi.shape[0] if vi.size else 0, ptr(vd), vd.size, C.byref(h)))
        return cls(None, None, None, _handle=h)

    def _load_meta(self):
        inf = Info()
        check(lib().hmgpu_hmatrix_info(self._h, C.byref(inf)))
        self._info = inf
        self.shape = (inf.m, inf.n)
        self.dtype = np.float64 if inf.precision == F64 else np.float32

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().hmgpu_hmatrix_free(h)
            self._h = None

    # ---- queries ---------------------------------------------------------------------
    def info(self):
        """info(::HMatrixCPU) (src/hmatrix.jl:289-330) plus storage figures."""
        i = self._info
        return {"data_type": self.dtype, "size": (i.m, i.n), "leaves": i.n_dense + i.n_approx,
                "admissible_leaves": i.n_approx, "full_leaves": i.n_dense,
                "min_rank": i.min_rank, "max_rank": i.max_rank,
                "min_dense_size": i.min_dense_size, "max_dense_size": i.max_dense_size,
                "compression_ratio": i.compression_ratio, "total_rank": i.total_rank,
                "dense_entries": i.dense_entries, "far_entries": i.far_entries,
                "matrix_bytes": i.matrix_bytes, "device_bytes": i.device_bytes,
                "n_tiles": i.n_tiles, "hi_only_blocks": i.hi_only_blocks,
                "build_seconds": i.build_seconds, "aca_batches": i.aca_batches,
                "aca_reruns": i.aca_reruns, "aca_workspace_bytes": i.aca_workspace_bytes,
                "aca_continued": i.aca_continued}

    BUILD_PHASES = ("block_tree", "setup", "aca", "gather", "plan", "pack", "tensor_core")

    def build_profile(self):
        """Seconds per phase of the last build (hmgpu_hmatrix_build_profile)."""
        v = (C.c_double * len(self.BUILD_PHASES))()
        check(lib().hmgpu_hmatrix_build_profile(self._h, v, len(self.BUILD_PHASES)))
        return dict(zip(self.BUILD_PHASES, list(v)))

    def blocks(self):
        """(dense (nD, 4), approx (nA, 5)) block tables: 1-based inclusive ranges, rank last."""
        i = self._info
        d = np.empty((i.n_dense, 4), np.int64)
        a = np.empty((i.n_approx, 5), np.int64)
        check(lib().hmgpu_hmatrix_blocks(self._h, ptr(d, I64P), ptr(a, I64P)))
        return d, a

    def index_maps(self):
        t = np.empty(self.shape[0], np.int64)
        s = np.empty(self.shape[1], np.int64)
        check(lib().hmgpu_hmatrix_index_maps(self._h, ptr(t, I64P), ptr(s, I64P)))
        return t, s

    def block_factors(self, b):
        """FP64 (U, V) of low-rank block b (0-based); needs keep_factors=True."""
        _, a = self.blocks()
        rs, re, cs, ce, r = a[b]
        U = np.empty((re - rs + 1, r))
        V = np.empty((r, ce - cs + 1))
        check(lib().hmgpu_hmatrix_block_factors(self._h, int(b), ptr(U), ptr(V)))
        return U, V

    def aca_ranks(self, count):
        """(ACA rank, final rank or -1 if stored dense) per admissible leaf of the
        block tree in traversal order (device builds; `count` = number of leaves)."""
        a = np.full(count, -1, np.int64)
        f = np.full(count, -1, np.int64)
        check(lib().hmgpu_hmatrix_aca_ranks(self._h, ptr(a, I64P), ptr(f, I64P)))
        return a, f

    def save(self, path):
        """Writes the assembled H-matrix to `path` (hmgpu_hmatrix_save)."""
        check(lib().hmgpu_hmatrix_save(self._h, str(path).encode()))

    @classmethod
    def load(cls, path):
        """An H-matrix saved by save(), on the current device, without assembly."""
        h = C.c_void_p()
        check(lib().hmgpu_hmatrix_load(str(path).encode(), C.byref(h)))
        return cls(None, None, None, _handle=h)

    def autotune(self, cache_path=None):
        """Times the product's free parameters on this H-matrix and keeps the
        fastest (hmgpu_hmatrix_autotune); results are bitwise unchanged."""
        r = (C.c_int32 * 4)()
        path = None if cache_path is None else str(cache_path).encode()
        check(lib().hmgpu_hmatrix_autotune(self._h, path, r))
        out = {"unit_rows": r[0], "vunit_kib": r[1], "multi_rhs_from": r[2], "from_cache": bool(r[3])}
        out["v_schedule"] = "dynamic" if self.tuning()["v_dynamic"] else "static"
        return out

    def set_tuning(self, unit_rows, vunit_kib, multi_rhs_from, v_dynamic):
        """Sets the product parameters directly (hmgpu_hmatrix_set_tuning)."""
        v = (C.c_int32 * 4)(int(unit_rows), int(vunit_kib), int(multi_rhs_from), int(v_dynamic))
        check(lib().hmgpu_hmatrix_set_tuning(self._h, v, 4))

    def tuning(self):
        """The product parameters in force (hmgpu_hmatrix_tuning)."""
        v = (C.c_int32 * 4)()
        check(lib().hmgpu_hmatrix_tuning(self._h, v, 4))
        return {"unit_rows": v[0], "vunit_kib": v[1], "multi_rhs_from": v[2], "v_dynamic": bool(v[3])}

    def status(self):
        """Device error word of the products so far (0 = clean; synchronises the
        device). Non-zero values name the bounded wait that ran out."""
        st = C.c_int32(0)
        rc = lib().hmgpu_hmatrix_status(self._h, C.byref(st))
        if rc not in (0, -5):  # HMGPU_ERR_TIMEOUT carries the code in st
            check(rc)
        return st.value

    def shard(self, rank, world):
        """Row shard `rank` of `world` (hmgpu_hmatrix_shard): the H-matrix's
        contiguous range of permuted rows, for products split over GPUs."""
        h = C.c_void_p()
        check(lib().hmgpu_hmatrix_shard(self._h, int(rank), int(world), C.byref(h)))
        return Shard(h, self.shape, self.dtype)

    # ---- products ------------------------------------------------------------------
    def mul(self, y, x, stream=None):
        """mul!(y, H, x): y and x are torch CUDA tensors (stream-ordered on the
        current torch stream unless `stream` is given) or numpy arrays (host,
        synchronous). Vectors or (n, nrhs) column-major/Fortran matrices."""
        return mul_(y, self, x, stream=stream)

    def __mul__(self, x):
        """H * x (src/mult.jl:203-209)."""
        return self.matvec(x)

    __matmul__ = __mul__

    def matvec(self, x):
        m = self.shape[0]
        if _is_torch(x):
            import torch
            shape = (m,) if x.dim() == 1 else (x.shape[1], m)
            y = torch.empty(shape, dtype=x.dtype, device=x.device)
            if x.dim() == 2:
                y = y.t()
            mul_(y, self, x)
            return y
        x = np.asarray(x)
        y = np.empty((m,) + x.shape[1:], dtype=self.dtype, order="F")
        mul_(y, self, x)
        return y


def _is_torch(a):
    return type(a).__module__.startswith("torch")


class Shard:
    """Rows [row_begin, row_end) of an H-matrix in the permuted target order
    (hmgpu_hmatrix_shard). Each owned row of its product is bitwise the row
    the whole H-matrix computes; it reads x in the permuted source order."""

    def __init__(self, handle, shape, dtype):
        self._h = handle
        self.shape = shape
        self.dtype = dtype
        b, e = C.c_int64(), C.c_int64()
        check(lib().hmgpu_shard_rows(self._h, C.byref(b), C.byref(e)))
        self.rows = (b.value, e.value)

    def mul_permuted(self, y_rows, x_perm, stream=None):
        """y_rows[i] = (H x)[target_map[row_begin + i] - 1] for the owned rows,
        from x_perm (all n entries, permuted source order). CUDA tensors of
        the H-matrix's dtype, stream-ordered."""
        import torch
        want = torch.float64 if self.dtype == np.float64 else torch.float32
        if x_perm.dtype != want or y_rows.dtype != want or not (x_perm.is_cuda and y_rows.is_cuda):
            raise TypeError(f"x and y must be CUDA {want} tensors")
        if x_perm.numel() != self.shape[1] or y_rows.numel() != self.rows[1] - self.rows[0]:
            raise ValueError("dimension mismatch")
        if not (x_perm.is_contiguous() and y_rows.is_contiguous()):
            raise ValueError("x and y must be contiguous")
        if stream is None:
            stream = torch.cuda.current_stream(x_perm.device).cuda_stream
        with torch.cuda.device(x_perm.device):
            check(lib().hmgpu_matvec_shard(self._h, C.c_void_p(x_perm.data_ptr()), C.c_void_p(y_rows.data_ptr()),
                                           C.c_void_p(stream)))
        return y_rows

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().hmgpu_hmatrix_free(h)
            self._h = None


def sparsify_hmatrix(K, X, Y, eta=1.5, triplets=False):
    """sparsify_hmatrix(K, X, Y; eta) (src/hmatrix.jl:234-274): the dense leaves
    of the merged block tree as a sparse matrix (scipy CSC, size(K)); with
    triplets=True the 1-based (I, J, V) arrays in the reference's order. The
    entries are generated on the device."""
    if not isinstance(K, Kernel):
        K = Kernel("explicit", A=K)
    d = K.desc()
    nnz = C.c_int64()
    check(lib().hmgpu_sparsify(C.byref(d), X._h, Y._h, float(eta), None, None, None, C.byref(nnz)))
    n = nnz.value
    I = np.empty(n, np.int64)
    J = np.empty(n, np.int64)
    V = np.empty(n)
    check(lib().hmgpu_sparsify(C.byref(d), X._h, Y._h, float(eta), ptr(I, I64P), ptr(J, I64P), ptr(V),
                               C.byref(nnz)))
    if triplets:
        return I, J, V
    import scipy.sparse as sp
    shape = (len(X.index_map), len(Y.index_map)) if K.kind == "user" else K.size()
    return sp.csc_matrix((V, (I - 1, J - 1)), shape=shape)


def batch(members):
    """The block-diagonal H-matrix diag(H_1, ..., H_k) of several H-matrices
    (hmgpu_hmatrix_batch): one product runs every member in the same kernel
    launches; x and y are the members' vectors concatenated."""
    hs = (C.c_void_p * len(members))(*[H._h for H in members])
    h = C.c_void_p()
    check(lib().hmgpu_hmatrix_batch(hs, len(members), C.byref(h)))
    return HMatrix(None, None, None, _handle=h)


class Graph:
    """mul!(y, H, x) captured into a CUDA graph (hmgpu_graph_create) for torch
    CUDA tensors x and y; launch() replays it on the current torch stream."""

    def __init__(self, H, x, y):
        import torch
        nrhs = 1 if x.dim() == 1 else x.shape[1]
        ldx = x.stride(1) if x.dim() == 2 else x.shape[0]
        ldy = y.stride(1) if y.dim() == 2 else y.shape[0]
        self.H, self.x, self.y = H, x, y  # the graph holds their device pointers
        g = C.c_void_p()
        with torch.cuda.device(x.device):
            check(lib().hmgpu_graph_create(H._h, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()),
                                           nrhs, ldx, ldy, C.byref(g)))
        self._g = g

    def launch(self, stream=None):
        import torch
        if stream is None:
            stream = torch.cuda.current_stream(self.x.device).cuda_stream
        check(lib().hmgpu_graph_launch(self._g, C.c_void_p(stream)))
        return self.y

    def __del__(self):
        g = getattr(self, "_g", None)
        if g:
            lib().hmgpu_graph_free(g)
            self._g = None


def mul_(y, H, x, stream=None):
    """mul!(y, H, x) (src/mult.jl:159-189): overwrites y with H x, original ordering."""
    m, n = H.shape
    L = lib()
    if _is_torch(x):
        import torch
        if not (x.is_cuda and y.is_cuda):
            raise ValueError("torch tensors must be CUDA tensors")
        want = torch.float64 if H.dtype == np.float64 else torch.float32
        if x.dtype != want or y.dtype != want:
            raise TypeError(f"x and y must be {want} for this H-matrix")
        nrhs = 1 if x.dim() == 1 else x.shape[1]
        if x.shape[0] != n or y.shape[0] != m or (x.dim() == 2 and y.shape[1] != nrhs):
            raise ValueError("dimension mismatch")
        if x.dim() == 2 and (x.stride(0) != 1 or y.stride(0) != 1):
            raise ValueError("x and y must be column-major (use .t().contiguous().t())")
        ldx = x.stride(1) if x.dim() == 2 else n
        ldy = y.stride(1) if y.dim() == 2 else m
        if stream is None:
            stream = torch.cuda.current_stream(x.device).cuda_stream
        with torch.cuda.device(x.device):
            check(L.hmgpu_matvec(H._h, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), nrhs,
                                 ldx, ldy, C.c_void_p(stream)))
        return y
    xa = np.asarray(x)
    if xa.dtype != H.dtype:
        raise TypeError(f"x must be {np.dtype(H.dtype)} for this H-matrix")
    if not isinstance(y, np.ndarray) or y.dtype != H.dtype:
        raise TypeError(f"y must be a numpy {np.dtype(H.dtype)} array")
    xa = np.asfortranarray(xa)
    nrhs = 1 if xa.ndim == 1 else xa.shape[1]
    if xa.shape[0] != n or y.shape[0] != m:
        raise ValueError("dimension mismatch")
    yb = y if y.flags.f_contiguous else np.empty(y.shape, y.dtype, order="F")
    check(L.hmgpu_matvec_host(H._h, xa.ctypes.data_as(C.c_void_p), yb.ctypes.data_as(C.c_void_p),
                              nrhs, n, m))
    if yb is not y:
        y[...] = yb
    return y


def info(obj):
    """info(tree) / info(hmatrix)."""
    return obj.info()


def selftest_bounded_wait(limit_ms=20.0):
    """Runs the bounded device-side wait of the tensor-core product against a
    barrier that nothing completes, limited to limit_ms. Returns (code, waited_ms):
    code 90 means the wait expired and reported itself, as it must."""
    L = lib()
    code = C.c_int32(0)
    waited = C.c_double(0.0)
    check(L.hmgpu_selftest_bounded_wait(int(limit_ms * 1e6), C.byref(code), C.byref(waited)))
    return code.value, waited.value
