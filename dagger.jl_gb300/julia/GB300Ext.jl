# GB300Ext: a Dagger.jl package extension binding libdaggergb300 through its
# C ABI (include/dagger_gb300.h), with no CUDA.jl, CUBLAS or CUSOLVER on the
# Cholesky path.  It follows the shape of Dagger's own CUDA extension
# (ext/CUDAExt.jl:25-65 processor and memory space, :131-154 moves,
# :309-327 execute!, :329-348 the BLAS/LAPACK substitution table):
#
#   * GB300Array{T,N}: a device buffer allocated through dg_device_alloc;
#   * GB300Proc / GB300MemorySpace: the processor and memory space Dagger's
#     scheduler and datadeps planner place tasks and chunks on;
#   * Dagger.move(::CPUProc, ::GB300Proc, ::typeof(f)) for LAPACK.potrf!,
#     BLAS.trsm!, syrk!, gemm!, trsv!, gemv!: each returns a ccall wrapper, so
#     Dagger's unchanged _chol! (src/array/cholesky.jl) and trsm!/trsv!
#     (src/array/trsm.jl) run their tile tasks on the GB300 kernels;
#   * cholesky_gb300! / ldiv_gb300! (and the engine-2 forms cholesky_gb300_winv!
#     / ldiv_gb300!(C, winv, B)): the whole datadeps region of a DArray
#     handed to the library in one call (dg_cholesky_tiled /
#     dg_cholesky_solve_tiled), issued as one cached multi-stream CUDA graph.
#
# This file is not exercised in this repository's tests (no Julia toolchain
# here); the Python package dagger_gb300 drives the same ABI and is tested.
module GB300Ext

using Dagger
using Distributed
using LinearAlgebra
import LinearAlgebra: BLAS, LAPACK

const libdg = get(ENV, "DAGGER_GB300_LIB",
                  joinpath(@__DIR__, "..", "dagger_gb300", "libdaggergb300.so"))

dgcheck(rc::Integer) = rc < 0 ?
    error("libdaggergb300 error $rc: " * unsafe_string(ccall((:dg_last_error, libdg), Cstring, ()))) : rc

# ---------------------------------------------------------------------------
# device arrays
# ---------------------------------------------------------------------------
mutable struct GB300Array{T,N} <: DenseArray{T,N}
    ptr::Ptr{T}
    dims::NTuple{N,Int}
    device::Int
    function GB300Array{T,N}(::UndefInitializer, dims::NTuple{N,Int}; device::Int=0) where {T,N}
        out = Ref{Ptr{Cvoid}}(C_NULL)
        dgcheck(ccall((:dg_set_device, libdg), Cint, (Cint,), device))
        dgcheck(ccall((:dg_device_alloc, libdg), Cint, (Csize_t, Ptr{Ptr{Cvoid}}),
                      sizeof(T) * prod(dims), out))
        x = new{T,N}(Ptr{T}(out[]), dims, device)
        finalizer(x) do a
            ccall((:dg_device_free, libdg), Cint, (Ptr{Cvoid},), a.ptr)
        end
        return x
    end
end
Base.size(x::GB300Array) = x.dims
Base.pointer(x::GB300Array) = x.ptr
Base.unsafe_convert(::Type{Ptr{T}}, x::GB300Array{T}) where T = x.ptr
Base.strides(x::GB300Array{T,2}) where T = (1, x.dims[1])
Base.stride(x::GB300Array{T,2}, i::Int) where T = i == 1 ? 1 : x.dims[1]

# One library stream per device, created on first use (Dagger's tasks may
# ask for it from several threads at once, hence the lock).  A caller that
# runs whole-region calls from concurrent tasks passes each task its own
# stream (`new_stream`): the library gives every stream its own workspace,
# so such calls run side by side.
const STREAMS = Dict{Int,Ptr{Cvoid}}()
const STREAMS_LOCK = ReentrantLock()
function new_stream()
    s = Ref{Ptr{Cvoid}}(C_NULL)
    dgcheck(ccall((:dg_stream_create, libdg), Cint, (Ptr{Ptr{Cvoid}},), s))
    return s[]
end
function device_stream(device::Int)
    lock(STREAMS_LOCK) do
        get!(new_stream, STREAMS, device)
    end
end
synchronize(device::Int) = dgcheck(ccall((:dg_stream_synchronize, libdg), Cint, (Ptr{Cvoid},), device_stream(device)))

function GB300Array(x::Array{T,N}; device::Int=0) where {T,N}
    y = GB300Array{T,N}(undef, size(x); device)
    dgcheck(ccall((:dg_copy, libdg), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Csize_t, Cint, Ptr{Cvoid}),
                  y.ptr, pointer(x), sizeof(x), 0, device_stream(device)))
    synchronize(device)
    return y
end
function Base.Array(x::GB300Array{T,N}) where {T,N}
    y = Array{T,N}(undef, x.dims)
    dgcheck(ccall((:dg_copy, libdg), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Csize_t, Cint, Ptr{Cvoid}),
                  pointer(y), x.ptr, sizeof(y), 1, device_stream(x.device)))
    synchronize(x.device)
    return y
end

# ---------------------------------------------------------------------------
# processor and memory space (ext/CUDAExt.jl:25-65)
# ---------------------------------------------------------------------------
struct GB300Proc <: Dagger.Processor
    owner::Int
    device::Int
end
Dagger.get_parent(proc::GB300Proc) = Dagger.OSProc(proc.owner)
Dagger.root_worker_id(proc::GB300Proc) = proc.owner
Dagger.short_name(proc::GB300Proc) = "W: $(proc.owner), GB300: $(proc.device)"
Dagger.@gpuproc(GB300Proc, GB300Array)

struct GB300MemorySpace <: Dagger.MemorySpace
    owner::Int
    device::Int
end
Dagger.root_worker_id(space::GB300MemorySpace) = space.owner
Dagger.memory_space(x::GB300Array) = GB300MemorySpace(myid(), x.device)
Dagger.memory_spaces(proc::GB300Proc) = Set([GB300MemorySpace(proc.owner, proc.device)])
Dagger.processors(space::GB300MemorySpace) = Set([GB300Proc(space.owner, space.device)])
function Dagger.aliasing(x::GB300Array{T}) where T
    space = Dagger.memory_space(x)
    rptr = Dagger.RemotePtr{Cvoid}(UInt64(x.ptr), space)
    return Dagger.ContiguousAliasing(Dagger.MemorySpan{GB300MemorySpace}(rptr, sizeof(T) * length(x)))
end
Dagger.unsafe_free!(x::GB300Array) = (finalize(x); nothing)

# moves between host and device (ext/CUDAExt.jl:131-154)
function Dagger.move!(::GB300MemorySpace, ::Dagger.CPURAMMemorySpace, to::GB300Array{T}, from::Array{T}) where T
    dgcheck(ccall((:dg_copy, libdg), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Csize_t, Cint, Ptr{Cvoid}),
                  to.ptr, pointer(from), sizeof(from), 0, device_stream(to.device)))
    return
end
function Dagger.move!(::Dagger.CPURAMMemorySpace, ::GB300MemorySpace, to::Array{T}, from::GB300Array{T}) where T
    dgcheck(ccall((:dg_copy, libdg), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Csize_t, Cint, Ptr{Cvoid}),
                  pointer(to), from.ptr, sizeof(to), 1, device_stream(from.device)))
    synchronize(from.device)
    return
end
Dagger.move(::Dagger.CPUProc, to_proc::GB300Proc, x::Array) = GB300Array(x; device=to_proc.device)
Dagger.move(::GB300Proc, ::Dagger.CPUProc, x::GB300Array) = Array(x)

# execute! on the device's stream (ext/CUDAExt.jl:309-327); kernels are
# stream-ordered, so no synchronisation here
function Dagger.execute!(proc::GB300Proc, f, args...; kwargs...)
    dgcheck(ccall((:dg_set_device, libdg), Cint, (Cint,), proc.device))
    return f(args...; kwargs...)
end

# ---------------------------------------------------------------------------
# tile calls: the substitution table (ext/CUDAExt.jl:329-348)
# ---------------------------------------------------------------------------
ld(A::GB300Array{T,2}) where T = max(1, size(A, 1))

function gb300_potrf!(uplo::AbstractChar, A::GB300Array{Float64,2})
    info = Ref{Cint}(0)
    rc = ccall((:dg_potrf, libdg), Cint, (Cchar, Cint, Ptr{Float64}, Cint, Ptr{Cint}, Ptr{Cvoid}),
               uplo, size(A, 1), A, ld(A), info, device_stream(A.device))
    dgcheck(rc)
    return A, Int(info[])
end
function gb300_trsm!(side, uplo, transa, diag, alpha::Float64, A::GB300Array{Float64,2}, B::GB300Array{Float64,2})
    dgcheck(ccall((:dg_trsm, libdg), Cint,
                  (Cchar, Cchar, Cchar, Cchar, Cint, Cint, Cdouble, Ptr{Float64}, Cint, Ptr{Float64}, Cint, Ptr{Cvoid}),
                  side, uplo, transa, diag, size(B, 1), size(B, 2), alpha, A, ld(A), B, ld(B), device_stream(B.device)))
    return B
end
function gb300_syrk!(uplo, trans, alpha::Float64, A::GB300Array{Float64,2}, beta::Float64, C::GB300Array{Float64,2})
    k = trans == 'N' ? size(A, 2) : size(A, 1)
    dgcheck(ccall((:dg_syrk, libdg), Cint,
                  (Cchar, Cchar, Cint, Cint, Cdouble, Ptr{Float64}, Cint, Cdouble, Ptr{Float64}, Cint, Ptr{Cvoid}),
                  uplo, trans, size(C, 1), k, alpha, A, ld(A), beta, C, ld(C), device_stream(C.device)))
    return C
end
function gb300_gemm!(ta, tb, alpha::Float64, A::GB300Array{Float64,2}, B::GB300Array{Float64,2}, beta::Float64, C::GB300Array{Float64,2})
    k = ta == 'N' ? size(A, 2) : size(A, 1)
    dgcheck(ccall((:dg_gemm, libdg), Cint,
                  (Cchar, Cchar, Cint, Cint, Cint, Cdouble, Ptr{Float64}, Cint, Ptr{Float64}, Cint, Cdouble, Ptr{Float64}, Cint, Ptr{Cvoid}),
                  ta, tb, size(C, 1), size(C, 2), k, alpha, A, ld(A), B, ld(B), beta, C, ld(C), device_stream(C.device)))
    return C
end
function gb300_trsv!(uplo, trans, diag, A::GB300Array{Float64,2}, x::GB300Array{Float64,1})
    dgcheck(ccall((:dg_trsv, libdg), Cint, (Cchar, Cchar, Cchar, Cint, Ptr{Float64}, Cint, Ptr{Float64}, Ptr{Cvoid}),
                  uplo, trans, diag, size(A, 1), A, ld(A), x, device_stream(x.device)))
    return x
end
function gb300_gemv!(trans, alpha::Float64, A::GB300Array{Float64,2}, x::GB300Array{Float64,1}, beta::Float64, y::GB300Array{Float64,1})
    dgcheck(ccall((:dg_gemv, libdg), Cint, (Cchar, Cint, Cint, Cdouble, Ptr{Float64}, Cint, Ptr{Float64}, Cdouble, Ptr{Float64}, Ptr{Cvoid}),
                  trans, size(A, 1), size(A, 2), alpha, A, ld(A), x, beta, y, device_stream(y.device)))
    return y
end

Dagger.move(::Dagger.CPUProc, ::GB300Proc, ::typeof(LAPACK.potrf!)) = gb300_potrf!
Dagger.move(::Dagger.CPUProc, ::GB300Proc, ::typeof(BLAS.trsm!)) = gb300_trsm!
Dagger.move(::Dagger.CPUProc, ::GB300Proc, ::typeof(BLAS.syrk!)) = gb300_syrk!
Dagger.move(::Dagger.CPUProc, ::GB300Proc, ::typeof(BLAS.gemm!)) = gb300_gemm!
Dagger.move(::Dagger.CPUProc, ::GB300Proc, ::typeof(BLAS.trsv!)) = gb300_trsv!
Dagger.move(::Dagger.CPUProc, ::GB300Proc, ::typeof(BLAS.gemv!)) = gb300_gemv!

# ---------------------------------------------------------------------------
# whole-region calls: one ccall per cholesky! / ldiv!
# ---------------------------------------------------------------------------
tile_pointers(A::DArray) = [pointer(fetch(c)::GB300Array{Float64,2}) for c in A.chunks]
# The library reports the global order of the first leading minor that is
# not positive definite; potrf_checked! (src/array/cholesky.jl:2-18) records
# the LAPACK info of the failing diagonal tile, and _chol! returns that
# number, so the binding converts (1-based, tile k starts at k*nb + 1).
tile_local_info(info::Integer, nb::Integer) = info <= 0 ? Int(info) : Int(info - nb * div(info - 1, nb))
# the device holding a DArray's chunks, whose stream a whole-region call uses
# unless the caller passes one
device_of(A::DArray) = (fetch(first(A.chunks))::GB300Array).device

"""
    cholesky_gb300!(A::DArray{Float64,2}, uplo='U') -> Cholesky

The datadeps region of `_chol!` (src/array/cholesky.jl:19-108) run by the
library as one captured multi-stream CUDA graph.  All chunks must be
GB300Arrays with Blocks(nb, nb) partitioning.  Throws PosDefException(info)
with the failing diagonal tile's LAPACK info, as `potrf_checked!` records it.
"""
function cholesky_gb300!(A::DArray{Float64,2}, uplo::Char='U';
                         stream::Ptr{Cvoid}=device_stream(device_of(A)))
    n = size(A, 1)
    nb = A.partitioning.blocksize[1]
    ptrs = tile_pointers(A)
    info = ccall((:dg_cholesky_tiled, libdg), Cint, (Cchar, Cint, Cint, Ptr{Ptr{Float64}}, Ptr{Cvoid}),
                 uplo, n, nb, ptrs, stream)
    dgcheck(info)
    info > 0 && throw(PosDefException(tile_local_info(info, nb)))
    return Cholesky(A, uplo, convert(LinearAlgebra.BlasInt, 0))
end

"""
    ldiv_gb300!(C::Cholesky{Float64,<:DMatrix}, B::DMatrix) -> B

ldiv! (src/array/linalg.jl:352-405) as one library call.
"""
function ldiv_gb300!(C::Cholesky{Float64,<:DArray}, B::DArray{Float64};
                     stream::Ptr{Cvoid}=device_stream(device_of(C.factors)))
    F = C.factors
    n = size(F, 1)
    nb = F.partitioning.blocksize[1]
    nrhs = ndims(B) == 1 ? 1 : size(B, 2)
    dgcheck(ccall((:dg_cholesky_solve_tiled, libdg), Cint,
                  (Cchar, Cint, Cint, Ptr{Ptr{Float64}}, Cint, Ptr{Ptr{Float64}}, Ptr{Cvoid}),
                  C.uplo, n, nb, tile_pointers(F), nrhs, tile_pointers(B), stream))
    return B
end

"""
    cholesky_gb300_winv!(A::DArray{Float64,2}, uplo='U') -> (Cholesky, winv)

cholesky_gb300! with the emulated FP64 engine (engine 2), also keeping the
transposed inverses of the diagonal factor tiles the factorization forms for
its panel products (winv: mt * nb * nb doubles on the device), so that
ldiv_gb300!(C, winv, B) solves each diagonal block as one product.
"""
function cholesky_gb300_winv!(A::DArray{Float64,2}, uplo::Char='U';
                              stream::Ptr{Cvoid}=device_stream(device_of(A)))
    n = size(A, 1)
    nb = A.partitioning.blocksize[1]
    mt = cld(n, nb)
    winv = GB300Array{Float64,1}(undef, (mt * nb * nb,); device=device_of(A))
    info = ccall((:dg_cholesky_tiled_winv, libdg), Cint,
                 (Cchar, Cint, Cint, Ptr{Ptr{Float64}}, Ptr{Float64}, Ptr{Cvoid}),
                 uplo, n, nb, tile_pointers(A), pointer(winv), stream)
    dgcheck(info)
    info > 0 && throw(PosDefException(tile_local_info(info, nb)))
    return Cholesky(A, uplo, convert(LinearAlgebra.BlasInt, 0)), winv
end

"""
    cholesky_gb300_host!(A::DArray{Float64,2}, H::Matrix{Float64}, uplo='U') -> Cholesky

cholesky(distribute(H, Blocks(nb, nb))) for a host matrix H (symmetric, so
its column-major storage reads the same as the row-major source the library
expects), with the chunks' moves to the device as tasks of the factor's graph.
dg_cholesky_tiled_host reads page-locked memory only, so H is copied into a
buffer from dg_host_alloc for the call.  A receives the tiles and then the
factor.
"""
function cholesky_gb300_host!(A::DArray{Float64,2}, H::Matrix{Float64}, uplo::Char='U';
                              stream::Ptr{Cvoid}=device_stream(device_of(A)))
    n = size(A, 1)
    nb = A.partitioning.blocksize[1]
    buf = Ref{Ptr{Cvoid}}(C_NULL)
    dgcheck(ccall((:dg_host_alloc, libdg), Cint, (Csize_t, Ptr{Ptr{Cvoid}}), sizeof(H), buf))
    info = try
        unsafe_copyto!(Ptr{Float64}(buf[]), pointer(H), length(H))
        ccall((:dg_cholesky_tiled_host, libdg), Cint,
              (Cchar, Cint, Cint, Ptr{Float64}, Clonglong, Ptr{Ptr{Float64}}, Ptr{Float64}, Ptr{Cvoid}),
              uplo, n, nb, Ptr{Float64}(buf[]), stride(H, 2), tile_pointers(A), C_NULL, stream)
    finally
        ccall((:dg_host_free, libdg), Cint, (Ptr{Cvoid},), buf[])
    end
    dgcheck(info)
    info > 0 && throw(PosDefException(tile_local_info(info, nb)))
    return Cholesky(A, uplo, convert(LinearAlgebra.BlasInt, 0))
end

function ldiv_gb300!(C::Cholesky{Float64,<:DArray}, winv::GB300Array{Float64,1}, B::DArray{Float64};
                     stream::Ptr{Cvoid}=device_stream(winv.device))
    F = C.factors
    n = size(F, 1)
    nb = F.partitioning.blocksize[1]
    nrhs = ndims(B) == 1 ? 1 : size(B, 2)
    dgcheck(ccall((:dg_cholesky_solve_tiled_winv, libdg), Cint,
                  (Cchar, Cint, Cint, Ptr{Ptr{Float64}}, Ptr{Float64}, Cint, Ptr{Ptr{Float64}}, Ptr{Cvoid}),
                  C.uplo, n, nb, tile_pointers(F), pointer(winv), nrhs, tile_pointers(B), stream))
    return B
end

"""
    mul_gb300!(C::DArray, A::DArray, B::DArray, alpha=1, beta=0, tA='N', tB='N') -> C

mul!(C, op(A), op(B), alpha, beta) on Blocks(nb, nb) DArrays of GB300Arrays,
dispatched as generic_matmatmul! does (src/array/mul.jl:11-41): A === B with
exactly one transposed is syrk_dagger! + copytri!, anything else
gemm_dagger!; each is one library graph (dg_syrk_tiled / dg_gemm_tiled).
"""
function mul_gb300!(C::DArray{Float64,2}, A::DArray{Float64,2}, B::DArray{Float64,2},
                    alpha::Real=1.0, beta::Real=0.0, tA::Char='N', tB::Char='N';
                    stream::Ptr{Cvoid}=device_stream(device_of(C)))
    nb = C.partitioning.blocksize[1]
    m, n = size(C)
    k = tA == 'N' ? size(A, 2) : size(A, 1)
    if A === B && (tA == 'N') != (tB == 'N')
        dgcheck(ccall((:dg_syrk_tiled, libdg), Cint,
                      (Cchar, Cint, Cint, Cint, Cdouble, Ptr{Ptr{Float64}}, Cdouble,
                       Ptr{Ptr{Float64}}, Ptr{Cvoid}),
                      tA == 'N' ? 'N' : 'T', n, k, nb, alpha, tile_pointers(A), beta,
                      tile_pointers(C), stream))
    else
        dgcheck(ccall((:dg_gemm_tiled, libdg), Cint,
                      (Cchar, Cchar, Cint, Cint, Cint, Cint, Cdouble, Ptr{Ptr{Float64}},
                       Ptr{Ptr{Float64}}, Cdouble, Ptr{Ptr{Float64}}, Ptr{Cvoid}),
                      tA, tB, m, n, k, nb, alpha, tile_pointers(A), tile_pointers(B), beta,
                      tile_pointers(C), stream))
    end
    return C
end

"""
    lu_gb300!(A::DArray{Float64,2}, pivot=RowMaximum(); check=true, allowsingular=false) -> LU

lu!(A, RowMaximum()) / lu!(A, NoPivot()) (src/array/lu.jl:5-54, 306-410) as
one library graph (dg_lu_tiled) on Blocks(nb, nb) chunks that are
GB300Arrays.  ipiv stays on the device (GB300Array{Int64,1}); info > 0 is
the first exactly zero pivot, checked as LinearAlgebra._check_lu_success.
"""
function lu_gb300!(A::DArray{Float64,2}, pivot::Union{RowMaximum,NoPivot}=RowMaximum();
                   check::Bool=true, allowsingular::Bool=false,
                   stream::Ptr{Cvoid}=device_stream(device_of(A)))
    m, n = size(A)
    nb = A.partitioning.blocksize[1]
    ipiv = GB300Array{Int64,1}(undef, (max(min(m, n), 1),); device=device_of(A))
    info = ccall((:dg_lu_tiled, libdg), Cint,
                 (Cint, Cint, Cint, Ptr{Ptr{Float64}}, Cint, Ptr{Int64}, Ptr{Cvoid}),
                 m, n, nb, tile_pointers(A), pivot isa RowMaximum ? 1 : 0, pointer(ipiv), stream)
    dgcheck(info)
    check && LinearAlgebra._check_lu_success(Int(info), allowsingular)
    return LU(A, ipiv, convert(LinearAlgebra.BlasInt, info))
end

"""
    ldiv_gb300!(F::LU{Float64,<:DArray}, B::DArray) -> B

ldiv!(F::LU, B) (src/array/linalg.jl:264-308) as one library call
(dg_lu_solve_tiled): B's rows permuted by ipiv, then the unit-lower and the
upper block solves.  B is blocked like the factors.
"""
function ldiv_gb300!(F::LU{Float64,<:DArray}, B::DArray{Float64};
                     stream::Ptr{Cvoid}=device_stream(F.ipiv.device))
    A = F.factors
    n = size(A, 1)
    nb = A.partitioning.blocksize[1]
    nrhs = ndims(B) == 1 ? 1 : size(B, 2)
    dgcheck(ccall((:dg_lu_solve_tiled, libdg), Cint,
                  (Cint, Cint, Ptr{Ptr{Float64}}, Ptr{Int64}, Cint, Ptr{Ptr{Float64}}, Ptr{Cvoid}),
                  n, nb, tile_pointers(A), pointer(F.ipiv), nrhs, tile_pointers(B), stream))
    return B
end

end # module
