"""The C ABI library loads and exports every entry point include/hmgpu.h declares."""
import ctypes
import os
import re

import hmgpu
from hmgpu import _lib

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    src = open(os.path.join(REPO, "include", "hmgpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(hmgpu_[a-z0-9_]+)\s*\(", src)))


def test_every_declared_symbol_is_exported():
    L = _lib.lib()
    names = declared()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert set(names) == set(_lib.SIGNATURES), set(names) ^ set(_lib.SIGNATURES)


def test_abi_version_and_errors():
    L = _lib.lib()
    assert L.hmgpu_abi_version() == 2
    rc = L.hmgpu_tree_build(None, 10, 4, 1, ctypes.byref(ctypes.c_void_p()))
    assert rc == -1 and b"NULL" in L.hmgpu_last_error()


def test_library_is_in_tree():
    path = _lib._build.LIB
    assert os.path.commonpath([path, REPO]) == REPO
    assert os.path.exists(path)


def test_julia_binding_calls_only_declared_symbols():
    """The Julia binding (julia/HMatrixGB.jl; Julia itself is not installed
    here) binds only entry points the header declares, by their names."""
    jl = open(os.path.join(REPO, "hmatrixgpu.jl_gb300", "julia", "HMatrixGB.jl")).read()
    called = set(re.findall(r"ccall\(\(:(hmgpu_[a-z0-9_]+)", jl))
    assert len(called) >= 15
    assert called <= set(declared()), called - set(declared())
