"""
    PencilFFTsGB300

`ccall` binding of libpencilfft_gb300 (C ABI in include/pencilfft_gb300.h) for
PencilFFTs.jl at `proc_dims = (1, ..., 1)` on one GB300 GPU.

`GB300Plan(dims, transforms, real_type; permute_dims, extra_dims, fftw_flags,
precision)` is the device counterpart of `PencilFFTPlan(dims, transforms,
proc_dims, comm, real_type; ...)` (reference src/plans.jl:306-320); `mul!`, `ldiv!` and `bmul!` take `CuArray`s
laid out as the reference's `PencilArray` parents: input in natural order,
output with its dimensions reversed when `permute_dims = Val(true)`.

The transforms are the reference's own `Transforms` types; the mapping to the
C ABI codes is `abi_kind`.
"""
module PencilFFTsGB300

using LinearAlgebra
using PencilFFTs: Transforms
using FFTW: FFTW
using CUDA: CuArray, CuPtr, stream as cuda_stream

const LIB = get(ENV, "PENCILFFT_GB300_LIB", joinpath(@__DIR__, "..", "pencilffts_gb300", "_lib",
                                                      "libpencilfft_gb300.so"))

const MAX_DIMS = 8
const MAX_EXTRA = 4

# pfgb_plan_desc (include/pencilfft_gb300.h)
struct PlanDesc
    ndims::Int32
    dims::NTuple{MAX_DIMS,Int64}
    kind::NTuple{MAX_DIMS,Int32}
    inplace::NTuple{MAX_DIMS,Int32}
    r2r_kind::NTuple{MAX_DIMS,Int32}
    brfft_even::NTuple{MAX_DIMS,Int32}
    real_bytes::Int32
    permute_dims::Int32
    n_extra::Int32
    extra_dims::NTuple{MAX_EXTRA,Int64}
    precision_mode::Int32
    autotune::Int32
end

# PFGB_PRECISION_* (include/pencilfft_gb300.h): :default (Float64 power-of-two
# lines in double-float), :native (FP64 everywhere), :tc (Float32 tensor-core
# split form), :fx (Float64 block floating point)
const PRECISION = Dict(:default => Int32(0), :native => Int32(1), :tc => Int32(2), :fx => Int32(3))

# planner measurement, as FFTW measures its candidates for any flag but ESTIMATE
autotune_code(flags) = Int32(flags & FFTW.ESTIMATE == 0)

abi_kind(::Union{Transforms.FFT,Transforms.FFT!}) = Int32(0)
abi_kind(::Union{Transforms.BFFT,Transforms.BFFT!}) = Int32(1)
abi_kind(::Union{Transforms.RFFT,Transforms.RFFT!}) = Int32(2)
abi_kind(::Union{Transforms.BRFFT,Transforms.BRFFT!}) = Int32(3)
abi_kind(::Transforms.AnyR2R) = Int32(4)
abi_kind(::Transforms.AnyNoTransform) = Int32(5)

r2r_code(t::Transforms.AnyR2R) = Int32(Transforms.kind(t))  # FFTW codes are used unchanged
r2r_code(::Transforms.AbstractTransform) = Int32(0)
even_code(t::Union{Transforms.BRFFT,Transforms.BRFFT!}) = Int32(t.even_output)
even_code(::Transforms.AbstractTransform) = Int32(0)

pad(t::Tuple, n, v) = ntuple(i -> i <= length(t) ? t[i] : v, n)

function check(rc::Integer)
    rc == 0 && return nothing
    buf = Vector{UInt8}(undef, 4096)
    ccall((:pfgb_last_error, LIB), Cint, (Ptr{UInt8}, Csize_t), buf, length(buf))
    msg = unsafe_string(pointer(buf))
    rc == -1 && throw(ArgumentError(msg))
    error("libpencilfft_gb300: status $rc: $msg")
end

mutable struct GB300Plan{T,N}
    handle::Ptr{Cvoid}
    transforms::NTuple{N,Transforms.AbstractTransform}
    scale::Float64
    function GB300Plan(dims::Dims{N}, transforms, ::Type{T} = Float64;
                       permute_dims::Val{P} = Val(true), extra_dims::Dims = (),
                       fftw_flags = FFTW.ESTIMATE, precision::Symbol = :default) where {N,T,P}
        haskey(PRECISION, precision) ||
            throw(ArgumentError("precision must be one of $(Tuple(keys(PRECISION)))"))
        trs = transforms isa Transforms.AbstractTransform ?
              Transforms.expand_dims(transforms, Val(N)) : transforms
        desc = PlanDesc(Int32(N), pad(Int64.(dims), MAX_DIMS, 0),
                        pad(map(abi_kind, trs), MAX_DIMS, Int32(0)),
                        pad(map(t -> Int32(Transforms.is_inplace(t)), trs), MAX_DIMS, Int32(0)),
                        pad(map(r2r_code, trs), MAX_DIMS, Int32(0)),
                        pad(map(even_code, trs), MAX_DIMS, Int32(0)),
                        Int32(sizeof(T)), Int32(P), Int32(length(extra_dims)),
                        pad(Int64.(extra_dims), MAX_EXTRA, 0), PRECISION[precision],
                        autotune_code(fftw_flags))
        h = Ref{Ptr{Cvoid}}(C_NULL)
        check(ccall((:pfgb_plan_create, LIB), Cint, (Ref{PlanDesc}, Ref{Ptr{Cvoid}}), desc, h))
        info = Vector{UInt8}(undef, 512)
        check(ccall((:pfgb_plan_info_get, LIB), Cint, (Ptr{Cvoid}, Ptr{UInt8}), h[], info))
        scale = unsafe_load(Ptr{Float64}(pointer(info) + 184))  # pfgb_plan_info.scale_factor (byte offset 184)
        p = new{T,N}(h[], trs, scale)
        finalizer(p) do q
            ccall((:pfgb_plan_destroy, LIB), Cint, (Ptr{Cvoid},), q.handle)
        end
        p
    end
end

scale_factor(p::GB300Plan) = p.scale

stream_ptr() = Ptr{Cvoid}(UInt(cuda_stream().handle))

# reference src/operations.jl:24-31
function LinearAlgebra.mul!(dst::CuArray, p::GB300Plan, src::CuArray)
    check(ccall((:pfgb_forward, LIB), Cint, (Ptr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, Ptr{Cvoid}),
                p.handle, dst, src, stream_ptr()))
    dst
end

# reference src/operations.jl:44-52 (the 1/scale_factor is fused into the last pass)
function LinearAlgebra.ldiv!(dst::CuArray, p::GB300Plan, src::CuArray)
    check(ccall((:pfgb_backward, LIB), Cint,
                (Ptr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, Ptr{Cvoid}, Cint),
                p.handle, dst, src, stream_ptr(), 1))
    dst
end

# reference src/operations.jl:34-41
function bmul!(dst::CuArray, p::GB300Plan, src::CuArray)
    check(ccall((:pfgb_backward, LIB), Cint,
                (Ptr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, Ptr{Cvoid}, Cint),
                p.handle, dst, src, stream_ptr(), 0))
    dst
end

end # module
