"""
    HMatrixGB

Julia binding of libhmgpu (include/hmgpu.h): the H-matrix path of HMatrixGPU.jl
— ClusterTree, BlockTree, HMatrix assembly and mul!(y, H, x) / H * x — running
on a GB300 (sm_103a) through a C ABI. The API keeps the reference's names,
keyword arguments and semantics (src/tree.jl:45, src/block.jl:31,
src/hmatrix.jl:72, src/mult.jl:159, :203).

Two ways in:
  * `HMatrixGB.HMatrix(kernel, X, Y; eta, eps, precision)` assembles on the
    device (batched ACA+ and QR/SVD recompression) for a named kernel;
  * `HMatrixGB.HMatrix(H::HMatrixGPU.HMatrix{Float64})` imports a matrix the
    reference already assembled, in its flattened layout, unchanged.

`mul!(y::CuArray, H, x::CuArray)` is stream-ordered on CUDA.jl's task-local
stream and returns without synchronising, as the reference's device mul! does.
"""
module HMatrixGB

using LinearAlgebra
import SparseArrays
import LinearAlgebra: mul!
import Base: *

const libhmgpu = get(ENV, "HMGPU_LIB",
                     joinpath(@__DIR__, "..", "lib", "libhmgpu.so"))

const HMGPU_F64 = Int32(0)
const HMGPU_F32 = Int32(1)
const HMGPU_MIXED = Int32(2)

const KERNELS = Dict(:explicit => Int32(0), :laplace => Int32(1), :yukawa => Int32(2),
                     :log2d => Int32(3), :vector_r => Int32(4), :dipolar => Int32(5))

struct Options            # hmgpu_options
    precision::Int32
    compensated::Int32
    keep_factors::Int32
    lean::Int32            # mixed precision: 1 = keep only the tensor-core copy
    rank_model::Ptr{Cvoid} # const hmgpu_rank_model* (C_NULL: fixed ACA workspace)
end
Options(precision, compensated, keep_factors, lean) =
    Options(precision, compensated, keep_factors, lean, C_NULL)

struct KernelDesc
    kind::Int32
    reserved::Int32
    X::Ptr{Float64}
    nX::Int64
    Y::Ptr{Float64}
    nY::Int64
    A::Ptr{Float64}
    lda::Int64
    user::Ptr{Cvoid}        # const hmgpu_user_kernel* (HMGPU_KERNEL_USER)
    params::Ptr{Float64}
    nparams::Int64
end
KernelDesc(kind, reserved, X, nX, Y, nY, A, lda) =
    KernelDesc(kind, reserved, X, nX, Y, nY, A, lda, C_NULL, C_NULL, 0)

"""
    UserKernel(source)

A kernel K[i, j] = f(x_i, y_j) of the caller's own, for `HMatrix(uk, ...)`: the
reference builds an HMatrix from any K it can index (src/hmatrix.jl:183). The
CUDA C++ `source` defines
`__device__ double hmgpu_entry(const double *x, const double *y, const double *p, int a, int b)`
and is compiled at run time (NVRTC) into the library's assembly kernels.
"""
mutable struct UserKernel
    handle::Ptr{Cvoid}
    function UserKernel(source::AbstractString)
        h = Ref{Ptr{Cvoid}}(C_NULL)
        log = zeros(UInt8, 1 << 16)
        rc = ccall((:hmgpu_user_kernel_compile, libhmgpu), Cint,
                   (Cstring, Ref{Ptr{Cvoid}}, Ptr{UInt8}, Int64), source, h, log, length(log))
        rc == 0 || throw(HMGPUError(rc, unsafe_string(ccall((:hmgpu_last_error, libhmgpu), Cstring, ())) *
                                        "\n" * unsafe_string(pointer(log))))
        uk = new(h[])
        finalizer(u -> ccall((:hmgpu_user_kernel_free, libhmgpu), Cint, (Ptr{Cvoid},), u.handle), uk)
        return uk
    end
end

struct HMGPUError <: Exception
    code::Int
    msg::String
end

function check(rc)
    if rc != 0
        msg = unsafe_string(ccall((:hmgpu_last_error, libhmgpu), Cstring, ()))
        throw(HMGPUError(rc, msg))
    end
    return nothing
end

# ---------------------------------------------------------------------------
# ClusterTree(coordinates; max_points_per_leaf=32, dims=1)   (src/tree.jl:45)
# ---------------------------------------------------------------------------
mutable struct ClusterTree
    handle::Ptr{Cvoid}
    index_map::Vector{Int}
    coordinates::Matrix{Float64}
end

# gpu=true builds the same tree (bit for bit) on the current CUDA device
# (hmgpu_tree_build_device).
function ClusterTree(coordinates::AbstractMatrix; max_points_per_leaf::Int=32, dims::Int=1,
                     gpu::Bool=false)
    dims <= 0 && error("Parameter `dims` must be a positive integer.")
    c = Matrix{Float64}(coordinates)
    size(c, 1) == 3 || error("coordinates must be 3 x N")
    h = Ref{Ptr{Cvoid}}(C_NULL)
    if gpu
        check(ccall((:hmgpu_tree_build_device, libhmgpu), Cint,
                    (Ptr{Float64}, Int64, Int64, Int64, Ref{Ptr{Cvoid}}),
                    c, size(c, 2), max_points_per_leaf, dims, h))
    else
        check(ccall((:hmgpu_tree_build, libhmgpu), Cint,
                    (Ptr{Float64}, Int64, Int64, Int64, Ref{Ptr{Cvoid}}),
                    c, size(c, 2), max_points_per_leaf, dims, h))
    end
    nn, il = Ref{Int64}(0), Ref{Int64}(0)
    check(ccall((:hmgpu_tree_info, libhmgpu), Cint,
                (Ptr{Cvoid}, Ref{Int64}, Ref{Int64}, Ptr{Int64}, Ptr{Int64}, Ptr{Int64}),
                h[], nn, il, C_NULL, C_NULL, C_NULL))
    imap = Vector{Int}(undef, il[])
    check(ccall((:hmgpu_tree_export, libhmgpu), Cint,
                (Ptr{Cvoid}, Ptr{Int64}, Ptr{Int64}, Ptr{Int64}, Ptr{Int8}, Ptr{Int64},
                 Ptr{Int64}, Ptr{Float64}, Ptr{Float64}),
                h[], imap, C_NULL, C_NULL, C_NULL, C_NULL, C_NULL, C_NULL, C_NULL))
    t = ClusterTree(h[], imap, c)
    finalizer(t) do t
        ccall((:hmgpu_tree_free, libhmgpu), Cint, (Ptr{Cvoid},), t.handle)
    end
    return t
end

"""info(tree) (src/tree.jl:153-187)"""
function info(t::ClusterTree)
    d, mx, mn = Ref{Int64}(0), Ref{Int64}(0), Ref{Int64}(0)
    check(ccall((:hmgpu_tree_info, libhmgpu), Cint,
                (Ptr{Cvoid}, Ptr{Int64}, Ptr{Int64}, Ref{Int64}, Ref{Int64}, Ref{Int64}),
                t.handle, C_NULL, C_NULL, d, mx, mn))
    return Dict(:depth => d[], :max_points => mx[], :min_points => mn[])
end

# ---------------------------------------------------------------------------
# HMatrix
# ---------------------------------------------------------------------------
mutable struct HMatrix{T<:AbstractFloat}
    handle::Ptr{Cvoid}
    m::Int
    n::Int
end

Base.size(H::HMatrix) = (H.m, H.n)
Base.size(H::HMatrix, d) = size(H)[d]
Base.eltype(::HMatrix{T}) where {T} = T

_T(precision) = precision == :f64 ? Float64 : Float32
_mode(precision) = precision == :f64 ? HMGPU_F64 : precision == :f32 ? HMGPU_F32 : HMGPU_MIXED

function _wrap(::Type{T}, h) where {T}
    info_buf = zeros(UInt8, 256)
    check(ccall((:hmgpu_hmatrix_info, libhmgpu), Cint, (Ptr{Cvoid}, Ptr{UInt8}), h, info_buf))
    m = reinterpret(Int64, info_buf[1:8])[1]
    n = reinterpret(Int64, info_buf[9:16])[1]
    H = HMatrix{T}(h, m, n)
    finalizer(H) do H
        ccall((:hmgpu_hmatrix_free, libhmgpu), Cint, (Ptr{Cvoid},), H.handle)
    end
    return H
end

"""
    HMatrix(kind::Symbol, Xpts, Ypts, X::ClusterTree, Y::ClusterTree;
            eta=1.5, eps=1e-5, svd_recompress=true, precision=:f64)

HMatrix(K, X, Y; eta, eps) (src/hmatrix.jl:72) with K the named kernel over
the target points `Xpts` and source points `Ypts` (3 x N), assembled on the GPU.
"""
function HMatrix(kind::Symbol, Xpts::AbstractMatrix, Ypts::AbstractMatrix, X::ClusterTree,
                 Y::ClusterTree; eta=1.5, eps=1e-5, svd_recompress=true, precision=:f64)
    xp, yp = Matrix{Float64}(Xpts), Matrix{Float64}(Ypts)
    o = Ref(Options(_mode(precision), 0, 0, 0))
    k = Ref(KernelDesc(KERNELS[kind], 0, pointer(xp), size(xp, 2), pointer(yp), size(yp, 2),
                       C_NULL, 0))
    h = Ref{Ptr{Cvoid}}(C_NULL)
    GC.@preserve xp yp check(ccall((:hmgpu_hmatrix_build, libhmgpu), Cint,
                                   (Ref{Options}, Ref{KernelDesc}, Ptr{Cvoid}, Ptr{Cvoid}, Float64,
                                    Float64, Cint, Ref{Ptr{Cvoid}}),
                                   o, k, X.handle, Y.handle, eta, eps, svd_recompress, h))
    return _wrap(_T(precision), h[])
end

"""
    HMatrix(uk::UserKernel, Xpts, Ypts, X::ClusterTree, Y::ClusterTree;
            params=Float64[], eta=1.5, eps=1e-5, svd_recompress=true, precision=:f64)

HMatrix(K, X, Y; eta, eps) with K[i, j] = f(Xpts[:, i], Ypts[:, j]) from the
caller's compiled entry function and its parameters `params` (at most 64).
"""
function HMatrix(uk::UserKernel, Xpts::AbstractMatrix, Ypts::AbstractMatrix, X::ClusterTree,
                 Y::ClusterTree; params=Float64[], eta=1.5, eps=1e-5, svd_recompress=true, precision=:f64)
    xp, yp, pp = Matrix{Float64}(Xpts), Matrix{Float64}(Ypts), Vector{Float64}(params)
    o = Ref(Options(_mode(precision), 0, 0, 0))
    k = Ref(KernelDesc(Int32(6), 0, pointer(xp), size(xp, 2), pointer(yp), size(yp, 2), C_NULL, 0,
                       uk.handle, isempty(pp) ? C_NULL : pointer(pp), length(pp)))
    h = Ref{Ptr{Cvoid}}(C_NULL)
    GC.@preserve xp yp pp uk check(ccall((:hmgpu_hmatrix_build, libhmgpu), Cint,
                                         (Ref{Options}, Ref{KernelDesc}, Ptr{Cvoid}, Ptr{Cvoid}, Float64,
                                          Float64, Cint, Ref{Ptr{Cvoid}}),
                                         o, k, X.handle, Y.handle, eta, eps, svd_recompress, h))
    return _wrap(_T(precision), h[])
end

"""
    HMatrix(Hf; precision=:f64)

Imports a flattened `HMatrixGPU.HMatrix{Float64}` (src/hmatrix.jl:46-57) as it
is: index maps, dense/U/V tables and data (CPU or device arrays).
"""
function HMatrix(Hf; precision=:f64)
    m, n = size(Hf.K)
    A(x) = Array(x)
    tm, sm = A(Hf.target_index_map), A(Hf.source_index_map)
    di, ui, vi = A(Hf.dense_block_indices), A(Hf.U_block_indices), A(Hf.V_block_indices)
    dd, ud, vd = A(Hf.dense_blocks), A(Hf.U_matrices), A(Hf.V_matrices)
    o = Ref(Options(_mode(precision), 0, 0, 0))
    h = Ref{Ptr{Cvoid}}(C_NULL)
    nA = size(ui, 1) == 5 ? size(ui, 2) : 0
    R = size(vi, 1) == 3 ? size(vi, 2) : 0
    check(ccall((:hmgpu_hmatrix_import_flat, libhmgpu), Cint,
                (Ref{Options}, Int64, Int64, Ptr{Int64}, Ptr{Int64}, Ptr{Int64}, Int64,
                 Ptr{Float64}, Int64, Ptr{Int64}, Int64, Ptr{Float64}, Int64, Ptr{Int64}, Int64,
                 Ptr{Float64}, Int64, Ref{Ptr{Cvoid}}),
                o, m, n, tm, sm, di, size(di, 2), dd, length(dd), ui, nA, ud, length(ud), vi, R,
                vd, length(vd), h))
    return _wrap(_T(precision), h[])
end

# ---------------------------------------------------------------------------
# mul!(y, H, x) and H * x   (src/mult.jl:159-209)
# ---------------------------------------------------------------------------
# Device arrays: any array type whose `pointer` is a device address (CuArray
# via CUDA.jl's `CuPtr`); the stream is CUDA.jl's task-local stream.
function mul!(y::AbstractVecOrMat{T}, H::HMatrix{T}, x::AbstractVecOrMat{T}) where {T}
    nrhs = size(x, 2)
    size(x, 1) == H.n && size(y, 1) == H.m && size(y, 2) == nrhs ||
        throw(DimensionMismatch("H is $(size(H)), x is $(size(x)), y is $(size(y))"))
    if y isa Array
        check(ccall((:hmgpu_matvec_host, libhmgpu), Cint,
                    (Ptr{Cvoid}, Ptr{T}, Ptr{T}, Int64, Int64, Int64),
                    H.handle, x, y, nrhs, stride(x, 2), stride(y, 2)))
    else
        stream = _stream()
        check(ccall((:hmgpu_matvec, libhmgpu), Cint,
                    (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Int64, Int64, Int64, Ptr{Cvoid}),
                    H.handle, _devptr(x), _devptr(y), nrhs, stride(x, 2), stride(y, 2), stream))
    end
    return y
end

function *(H::HMatrix{T}, x::AbstractVecOrMat{T}) where {T}
    y = similar(x, T, size(x, 2) == 1 && x isa AbstractVector ? (H.m,) : (H.m, size(x, 2)))
    return mul!(y, H, x)
end

# ---------------------------------------------------------------------------
# sparsify_hmatrix (src/hmatrix.jl:234-274), batches, files, tuning
# ---------------------------------------------------------------------------
# A handle of either storage precision, typed from hmgpu_info.precision.
function _wrap_auto(h)
    info_buf = zeros(UInt8, 256)
    check(ccall((:hmgpu_hmatrix_info, libhmgpu), Cint, (Ptr{Cvoid}, Ptr{UInt8}), h, info_buf))
    p = reinterpret(Int32, info_buf[121:124])[1]
    return _wrap(p == HMGPU_F64 ? Float64 : Float32, h)
end

"""
    sparsify_hmatrix(kind::Symbol, Xpts, Ypts, X::ClusterTree, Y::ClusterTree; eta=1.5)

sparsify_hmatrix(K, X, Y; eta) (src/hmatrix.jl:234-274) for the named kernel
over `Xpts`/`Ypts`: the near field as a `SparseMatrixCSC`, entries generated on
the GPU.
"""
function sparsify_hmatrix(kind::Symbol, Xpts::AbstractMatrix, Ypts::AbstractMatrix, X::ClusterTree,
                          Y::ClusterTree; eta=1.5)
    xp, yp = Matrix{Float64}(Xpts), Matrix{Float64}(Ypts)
    k = Ref(KernelDesc(KERNELS[kind], 0, pointer(xp), size(xp, 2), pointer(yp), size(yp, 2), C_NULL, 0))
    nnz = Ref{Int64}(0)
    GC.@preserve xp yp begin
        check(ccall((:hmgpu_sparsify, libhmgpu), Cint,
                    (Ref{KernelDesc}, Ptr{Cvoid}, Ptr{Cvoid}, Float64, Ptr{Int64}, Ptr{Int64},
                     Ptr{Float64}, Ref{Int64}), k, X.handle, Y.handle, eta, C_NULL, C_NULL, C_NULL, nnz))
        I, J, V = Vector{Int64}(undef, nnz[]), Vector{Int64}(undef, nnz[]), Vector{Float64}(undef, nnz[])
        check(ccall((:hmgpu_sparsify, libhmgpu), Cint,
                    (Ref{KernelDesc}, Ptr{Cvoid}, Ptr{Cvoid}, Float64, Ptr{Int64}, Ptr{Int64},
                     Ptr{Float64}, Ref{Int64}), k, X.handle, Y.handle, eta, I, J, V, nnz))
    end
    m = kind == :dipolar ? 3 * size(xp, 2) : size(xp, 2)
    n = kind in (:vector_r, :dipolar) ? 3 * size(yp, 2) : size(yp, 2)
    return SparseArrays.sparse(I, J, V, m, n)
end

"""
    batch(Hs) -> HMatrix

diag(H_1, ..., H_k) as one H-matrix: x and y are the members' vectors
concatenated, and one product runs every member in the same kernel launches.
"""
function batch(Hs::AbstractVector{<:HMatrix})
    hs = Ptr{Cvoid}[H.handle for H in Hs]
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:hmgpu_hmatrix_batch, libhmgpu), Cint, (Ptr{Ptr{Cvoid}}, Int32, Ref{Ptr{Cvoid}}),
                hs, length(hs), h))
    return _wrap_auto(h[])
end

"""save(H, path): the assembled H-matrix on disk; load(path) reads it back without assembly."""
save(H::HMatrix, path::AbstractString) =
    check(ccall((:hmgpu_hmatrix_save, libhmgpu), Cint, (Ptr{Cvoid}, Cstring), H.handle, path))

function load(path::AbstractString)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:hmgpu_hmatrix_load, libhmgpu), Cint, (Cstring, Ref{Ptr{Cvoid}}), path, h))
    return _wrap_auto(h[])
end

"""autotune!(H; cache=nothing): times and keeps the product's work-partition
parameters (results are unchanged); `cache` names a file for the choices."""
function autotune!(H::HMatrix; cache::Union{Nothing,AbstractString}=nothing)
    r = zeros(Int32, 4)
    check(ccall((:hmgpu_hmatrix_autotune, libhmgpu), Cint, (Ptr{Cvoid}, Cstring, Ptr{Int32}),
                H.handle, cache === nothing ? C_NULL : cache, r))
    return (unit_rows=r[1], vunit_kib=r[2], multi_rhs_from=r[3], from_cache=r[4] != 0)
end

"""status(H): the device error word of the products so far (0 = clean)."""
function status(H::HMatrix)
    st = Ref{Cint}(0)
    rc = ccall((:hmgpu_hmatrix_status, libhmgpu), Cint, (Ptr{Cvoid}, Ref{Cint}), H.handle, st)
    rc in (0, -5) || check(rc)
    return Int(st[])
end

# ---------------------------------------------------------------------------
# Row shards for products over several GPUs (row ownership of src/mult.jl:144)
# ---------------------------------------------------------------------------
mutable struct Shard{T<:AbstractFloat}
    handle::Ptr{Cvoid}
    rows::UnitRange{Int}   # owned rows, 1-based, in the permuted target order
    n::Int
end

"""
    shard(H, rank, world) -> Shard

Shard `rank` (0-based) of `world`: a contiguous range of H's permuted rows with
the panels and V rows it needs, on the current device. `mul_shard!(y_rows, S,
x_perm)` computes those rows of H x from x in the permuted source order (all n
entries, gathered from the ranks first); every row is bitwise H's own.
"""
function shard(H::HMatrix{T}, rank::Integer, world::Integer) where {T}
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:hmgpu_hmatrix_shard, libhmgpu), Cint, (Ptr{Cvoid}, Int32, Int32, Ref{Ptr{Cvoid}}),
                H.handle, rank, world, h))
    b, e = Ref{Int64}(0), Ref{Int64}(0)
    check(ccall((:hmgpu_shard_rows, libhmgpu), Cint, (Ptr{Cvoid}, Ref{Int64}, Ref{Int64}), h[], b, e))
    S = Shard{T}(h[], (b[] + 1):e[], H.n)
    finalizer(S) do S
        ccall((:hmgpu_hmatrix_free, libhmgpu), Cint, (Ptr{Cvoid},), S.handle)
    end
    return S
end

function mul_shard!(y_rows::AbstractVector{T}, S::Shard{T}, x_perm::AbstractVector{T}) where {T}
    length(x_perm) == S.n && length(y_rows) == length(S.rows) ||
        throw(DimensionMismatch("x_perm has $(length(x_perm)) entries (need $(S.n)), y_rows $(length(y_rows)) (need $(length(S.rows)))"))
    check(ccall((:hmgpu_matvec_shard, libhmgpu), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}),
                S.handle, _devptr(x_perm), _devptr(y_rows), _stream()))
    return y_rows
end

# CUDA.jl hooks, resolved at run time so that this file loads without CUDA.jl.
_devptr(a) = reinterpret(Ptr{Cvoid}, UInt(Base.unsafe_convert(Main.CUDA.CuPtr{eltype(a)}, a)))
_stream() = reinterpret(Ptr{Cvoid}, Main.CUDA.stream().handle)

export ClusterTree, HMatrix, UserKernel, info, sparsify_hmatrix, batch, save, load, autotune!, status, shard, mul_shard!

end # module
