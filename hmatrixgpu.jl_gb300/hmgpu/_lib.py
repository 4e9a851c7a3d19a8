"""ctypes binding of libhmgpu.so (the C ABI declared in include/hmgpu.h)."""
import ctypes as C
import os
import threading

from . import _build

I64P = C.POINTER(C.c_int64)
F64P = C.POINTER(C.c_double)
F32P = C.POINTER(C.c_float)
I8P = C.POINTER(C.c_int8)
VP = C.c_void_p

F64, F32, MIXED = 0, 1, 2
PRECISIONS = {"f64": F64, "float64": F64, "f32": F32, "float32": F32, "mixed": MIXED}

KERNEL_IDS = {"explicit": 0, "laplace": 1, "yukawa": 2, "log2d": 3, "vector_r": 4, "dipolar": 5, "user": 6}

_lock = threading.Lock()
_LIB = None


class HMGPUError(RuntimeError):
    """A libhmgpu call returned a non-zero status."""

    def __init__(self, code, msg):
        super().__init__(f"libhmgpu error {code}: {msg}")
        self.code = code


class Options(C.Structure):
    _fields_ = [("precision", C.c_int32), ("compensated", C.c_int32),
                ("keep_factors", C.c_int32), ("lean", C.c_int32), ("rank_model", C.c_void_p)]


class KernelDesc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("reserved", C.c_int32), ("X", F64P), ("nX", C.c_int64),
                ("Y", F64P), ("nY", C.c_int64), ("A", F64P), ("lda", C.c_int64),
                ("user", C.c_void_p), ("params", F64P), ("nparams", C.c_int64)]


class Info(C.Structure):
    _fields_ = [("m", C.c_int64), ("n", C.c_int64), ("n_dense", C.c_int64),
                ("n_approx", C.c_int64), ("min_rank", C.c_int64), ("max_rank", C.c_int64),
                ("min_dense_size", C.c_int64), ("max_dense_size", C.c_int64),
                ("total_rank", C.c_int64), ("dense_entries", C.c_int64),
                ("far_entries", C.c_int64), ("compression_ratio", C.c_double),
                ("matrix_bytes", C.c_int64), ("device_bytes", C.c_int64),
                ("n_tiles", C.c_int64), ("precision", C.c_int32), ("hi_only_blocks", C.c_int32),
                ("build_seconds", C.c_double), ("aca_batches", C.c_int64),
                ("aca_reruns", C.c_int64), ("aca_workspace_bytes", C.c_int64),
                ("aca_continued", C.c_int64)]


# name -> (restype, argtypes); every entry point returns an int status unless noted
SIGNATURES = {
    "hmgpu_last_error": (C.c_char_p, []),
    "hmgpu_abi_version": (C.c_int, []),
    "hmgpu_tree_build": (C.c_int, [F64P, C.c_int64, C.c_int64, C.c_int64, C.POINTER(VP)]),
    "hmgpu_tree_build_device": (C.c_int, [VP, C.c_int64, C.c_int64, C.c_int64, C.POINTER(VP)]),
    "hmgpu_tree_info": (C.c_int, [VP, I64P, I64P, I64P, I64P, I64P]),
    "hmgpu_tree_export": (C.c_int, [VP, I64P, I64P, I64P, I8P, I64P, I64P, F64P, F64P]),
    "hmgpu_tree_free": (C.c_int, [VP]),
    "hmgpu_blocks_build": (C.c_int, [VP, VP, C.c_double, C.c_int, C.POINTER(VP)]),
    "hmgpu_blocks_build_device": (C.c_int, [VP, VP, C.c_double, C.c_int, C.POINTER(VP)]),
    "hmgpu_blocks_counts": (C.c_int, [VP, I64P, I64P, I64P]),
    "hmgpu_blocks_export": (C.c_int, [VP, I64P, I64P]),
    "hmgpu_blocks_export_nodes": (C.c_int, [VP, I64P, I64P, I8P, I8P, I64P, I64P]),
    "hmgpu_blocks_free": (C.c_int, [VP]),
    "hmgpu_hmatrix_import_flat": (C.c_int, [C.POINTER(Options), C.c_int64, C.c_int64, I64P, I64P,
                                            I64P, C.c_int64, F64P, C.c_int64, I64P, C.c_int64,
                                            F64P, C.c_int64, I64P, C.c_int64, F64P, C.c_int64,
                                            C.POINTER(VP)]),
    "hmgpu_hmatrix_build": (C.c_int, [C.POINTER(Options), C.POINTER(KernelDesc), VP, VP,
                                      C.c_double, C.c_double, C.c_int, C.POINTER(VP)]),
    "hmgpu_matvec": (C.c_int, [VP, VP, VP, C.c_int64, C.c_int64, C.c_int64, VP]),
    "hmgpu_matvec_host": (C.c_int, [VP, VP, VP, C.c_int64, C.c_int64, C.c_int64]),
    "hmgpu_matvec_noalloc": (C.c_int, [VP, VP, VP, VP]),
    "hmgpu_hmatrix_shard": (C.c_int, [VP, C.c_int32, C.c_int32, C.POINTER(VP)]),
    "hmgpu_shard_rows": (C.c_int, [VP, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "hmgpu_matvec_shard": (C.c_int, [VP, VP, VP, VP]),
    "hmgpu_hmatrix_info": (C.c_int, [VP, C.POINTER(Info)]),
    "hmgpu_hmatrix_build_profile": (C.c_int, [VP, C.POINTER(C.c_double), C.c_int32]),
    "hmgpu_hmatrix_status": (C.c_int, [VP, C.POINTER(C.c_int)]),
    "hmgpu_hmatrix_set_profiling": (C.c_int, [VP, C.c_int]),
    "hmgpu_hmatrix_phase_times": (C.c_int, [VP, F64P, I64P, I64P]),
    "hmgpu_hmatrix_blocks": (C.c_int, [VP, I64P, I64P]),
    "hmgpu_hmatrix_index_maps": (C.c_int, [VP, I64P, I64P]),
    "hmgpu_hmatrix_block_factors": (C.c_int, [VP, C.c_int64, F64P, F64P]),
    "hmgpu_hmatrix_aca_ranks": (C.c_int, [VP, I64P, I64P]),
    "hmgpu_hmatrix_free": (C.c_int, [VP]),
    "hmgpu_aca_plus": (C.c_int, [F64P, C.c_int64, C.c_int64, C.c_int64, C.c_double, C.c_int64,
                                 C.c_int64, F64P, F64P, I64P]),
    "hmgpu_svd_recompress": (C.c_int, [C.c_int64, C.c_int64, C.c_int64, F64P, F64P, C.c_double,
                                       F64P, F64P, I64P]),
    "hmgpu_rank_model_create": (C.c_int, [C.c_uint64, C.POINTER(VP)]),
    "hmgpu_rank_model_train": (C.c_int, [VP, F32P, F32P, C.c_int64, C.c_int64, C.c_int64, C.c_float,
                                         C.c_uint64, F32P]),
    "hmgpu_rank_model_predict": (C.c_int, [VP, F32P, C.c_int64, F32P]),
    "hmgpu_rank_model_gradients": (C.c_int, [VP, F32P, F32P, C.c_int64, F32P, F32P]),
    "hmgpu_rank_model_params": (C.c_int, [VP, F32P, F32P, F32P, F32P]),
    "hmgpu_rank_model_free": (C.c_int, [VP]),
    "hmgpu_block_features": (C.c_int, [VP, VP, C.c_double, C.c_double, F32P, I64P]),
    "hmgpu_sparsify": (C.c_int, [C.POINTER(KernelDesc), VP, VP, C.c_double, I64P, I64P, F64P, I64P]),
    "hmgpu_user_kernel_compile": (C.c_int, [C.c_char_p, C.POINTER(VP), C.c_char_p, C.c_int64]),
    "hmgpu_user_kernel_free": (C.c_int, [VP]),
    "hmgpu_hmatrix_batch": (C.c_int, [C.POINTER(VP), C.c_int32, C.POINTER(VP)]),
    "hmgpu_graph_create": (C.c_int, [VP, VP, VP, C.c_int64, C.c_int64, C.c_int64, C.POINTER(VP)]),
    "hmgpu_graph_launch": (C.c_int, [VP, VP]),
    "hmgpu_graph_free": (C.c_int, [VP]),
    "hmgpu_hmatrix_autotune": (C.c_int, [VP, C.c_char_p, C.POINTER(C.c_int32)]),
    "hmgpu_hmatrix_tuning": (C.c_int, [VP, C.POINTER(C.c_int32), C.c_int32]),
    "hmgpu_hmatrix_set_tuning": (C.c_int, [VP, C.POINTER(C.c_int32), C.c_int32]),
    "hmgpu_selftest_bounded_wait": (C.c_int, [C.c_int64, C.POINTER(C.c_int32), F64P]),
    "hmgpu_hmatrix_save": (C.c_int, [VP, C.c_char_p]),
    "hmgpu_hmatrix_load": (C.c_int, [C.c_char_p, C.POINTER(VP)]),
}


def _stale():
    if not os.path.exists(_build.LIB):
        return True
    t = os.path.getmtime(_build.LIB)
    srcs = [os.path.join(_build.CSRC, s) for s in os.listdir(_build.CSRC)]
    srcs.append(os.path.join(_build.REPO, "include", "hmgpu.h"))
    return any(os.path.getmtime(s) > t for s in srcs)


def lib():
    """Loads libhmgpu.so, compiling it first if it is missing or older than its sources."""
    global _LIB
    with _lock:
        if _LIB is None:
            if _stale():
                _build.build()
            L = C.CDLL(_build.LIB)
            for name, (res, args) in SIGNATURES.items():
                f = getattr(L, name)
                f.restype = res
                f.argtypes = args
            _LIB = L
    return _LIB


def check(rc):
    if rc != 0:
        raise HMGPUError(rc, lib().hmgpu_last_error().decode(errors="replace"))
    return rc


def ptr(a, t=F64P):
    """ctypes pointer to a numpy array's data."""
    return a.ctypes.data_as(t)
