"""
    PencilFFTsGB300

`ccall` binding of libpencilfft_gb300 (C ABI in include/pencilfft_gb300.h) for
PencilFFTs.jl at `proc_dims = (1, ..., 1)` on one GB300 GPU.

`GB300Plan(dims, transforms, real_type; permute_dims, extra_dims, fftw_flags,
precision)` is the device counterpart of `PencilFFTPlan(dims, transforms,
proc_dims, comm, real_type; ...)` (reference src/plans.jl:306-320).  The
reference's user API is mirrored on `CuArray`s laid out as the reference's
`PencilArray` parents (input in natural order, output with its dimensions
reversed when `permute_dims = Val(true)`):

- `mul!`, `ldiv!`, `bmul!` (src/operations.jl:24-52), also over tuples and
  arrays of arrays (src/operations.jl:129-152);
- `p * u` and `p \ uF` (src/operations.jl:54-62);
- `allocate_input(p)`, `allocate_output(p)` and their `Val(N)` / dims forms
  (src/allocate.jl:44-122); in-place plans return one buffer holding the
  input and output views (`ManyCuArray`, the counterpart of
  `ManyPencilArray`);
- `scale_factor`, `size`, `is_inplace`, `eltype_input`, `eltype_output`;
- the fused spectral operators of the library: `ldiv_deriv!` (one i k
  multiply), `ldiv_divergence!` and `ldiv_curl!` (test/include/FourierOperations.jl);
- batches: `GB300Batch([(mul!, vF, p, u), (ldiv!, du, p, vF, (dim, L)), ...];
  form = :graph)` records many transforms (any plans and sizes, optional fused
  derivative) for one `launch(batch)` (the collections of
  src/operations.jl:129-152 as one launch): `:graph` one CUDA graph with a
  branch per plan, `:persistent` one work-list kernel, `:auto`, `:measure`.

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

# pfgb_plan_info (include/pencilfft_gb300.h); Julia lays out isbits structs
# with C alignment, so the field order and types are the whole contract
struct PlanInfo
    ndims::Int32
    dims_in::NTuple{MAX_DIMS,Int64}
    dims_out::NTuple{MAX_DIMS,Int64}
    perm_out::NTuple{MAX_DIMS,Int32}
    eltype_in_complex::Int32
    eltype_out_complex::Int32
    real_bytes::Int32
    inplace::Int32
    scale_factor::Float64
    input_bytes::Int64
    output_bytes::Int64
    inplace_bytes::Int64
    scratch_bytes::Int64
    n_passes_forward::Int32
    n_passes_backward::Int32
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
    info::PlanInfo
    extra_dims::Dims
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
        info = Ref{PlanInfo}()
        check(ccall((:pfgb_plan_info_get, LIB), Cint, (Ptr{Cvoid}, Ref{PlanInfo}), h[], info))
        p = new{T,N}(h[], trs, info[].scale_factor, info[], extra_dims)
        finalizer(p) do q
            ccall((:pfgb_plan_destroy, LIB), Cint, (Ptr{Cvoid},), q.handle)
        end
        p
    end
end

scale_factor(p::GB300Plan) = p.scale
is_inplace(p::GB300Plan) = p.info.inplace != 0
Base.size(p::GB300Plan{T,N}) where {T,N} = ntuple(i -> Int(p.info.dims_in[i]), Val(N))
size_out(p::GB300Plan{T,N}) where {T,N} = ntuple(i -> Int(p.info.dims_out[i]), Val(N))
eltype_input(p::GB300Plan{T}) where {T} = p.info.eltype_in_complex != 0 ? Complex{T} : T
eltype_output(p::GB300Plan{T}) where {T} = p.info.eltype_out_complex != 0 ? Complex{T} : T

# memory shapes of the input (natural order) and output (perm_out: fastest
# logical dimension first) arrays, extra dimensions last
input_shape(p::GB300Plan) = (size(p)..., p.extra_dims...)
function output_shape(p::GB300Plan{T,N}) where {T,N}
    (ntuple(i -> Int(p.info.dims_out[p.info.perm_out[i] + 1]), Val(N))..., p.extra_dims...)
end

# In-place plans: one buffer holding the input and output views (the
# counterpart of ManyPencilArray, reference src/multiarrays_r2c.jl)
struct ManyCuArray{Tb}
    buffer::Tb
    input::CuArray
    output::CuArray
end

function _alloc(p::GB300Plan, which::Symbol)
    if is_inplace(p)
        buf = CuArray{UInt8}(undef, Int(p.info.inplace_bytes))
        ti, to = eltype_input(p), eltype_output(p)
        ishape = input_shape(p)
        if ti <: Real && to <: Complex  # RFFT!: real view padded to 2 (n1/2 + 1)
            ishape = (2 * (ishape[1] ÷ 2 + 1), Base.tail(ishape)...)
        end
        vin = reshape(reinterpret(ti, view(buf, 1:(prod(ishape) * sizeof(ti)))), ishape)
        vout = reshape(reinterpret(to, view(buf, 1:(prod(output_shape(p)) * sizeof(to)))), output_shape(p))
        return ManyCuArray(buf, vin, vout)
    end
    which === :in ? CuArray{eltype_input(p)}(undef, input_shape(p)) :
                    CuArray{eltype_output(p)}(undef, output_shape(p))
end

# reference src/allocate.jl:44-122
allocate_input(p::GB300Plan) = _alloc(p, :in)
allocate_output(p::GB300Plan) = _alloc(p, :out)
allocate_input(p::GB300Plan, ::Val{M}) where {M} = ntuple(_ -> allocate_input(p), Val(M))
allocate_output(p::GB300Plan, ::Val{M}) where {M} = ntuple(_ -> allocate_output(p), Val(M))
allocate_input(p::GB300Plan, dims...) = [allocate_input(p) for _ in CartesianIndices(dims)]
allocate_output(p::GB300Plan, dims...) = [allocate_output(p) for _ in CartesianIndices(dims)]

stream_ptr() = Ptr{Cvoid}(UInt(cuda_stream().handle))

_ptr(A::ManyCuArray) = pointer(A.buffer)
_ptr(A::CuArray) = pointer(A)

# reference src/operations.jl:24-31
function LinearAlgebra.mul!(dst::ManyCuArray, p::GB300Plan, src::ManyCuArray)
    dst === src || throw(ArgumentError("input and output arrays for in-place plan must be the same"))
    check(ccall((:pfgb_forward, LIB), Cint, (Ptr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, Ptr{Cvoid}),
                p.handle, _ptr(dst), _ptr(src), stream_ptr()))
    dst
end
function LinearAlgebra.ldiv!(dst::ManyCuArray, p::GB300Plan, src::ManyCuArray)
    dst === src || throw(ArgumentError("input and output arrays for in-place plan must be the same"))
    check(ccall((:pfgb_backward, LIB), Cint,
                (Ptr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, Ptr{Cvoid}, Cint),
                p.handle, _ptr(dst), _ptr(src), stream_ptr(), 1))
    dst
end

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

# reference src/operations.jl:54-62: allocating forms
Base.:*(p::GB300Plan, src::CuArray) = mul!(allocate_output(p), p, src)
Base.:\(p::GB300Plan, src::CuArray) = ldiv!(allocate_input(p), p, src)
Base.:*(p::GB300Plan, A::ManyCuArray) = mul!(A, p, A)
Base.:\(p::GB300Plan, A::ManyCuArray) = ldiv!(A, p, A)

# reference src/operations.jl:129-152: collections of fields
const Collection = Union{Tuple{Vararg{Union{CuArray,ManyCuArray}}},AbstractArray{<:Union{CuArray,ManyCuArray}}}
function _check_lengths(dst, src)
    length(dst) == length(src) || throw(ArgumentError("collections have different lengths"))
end
for f in (:mul!, :ldiv!)
    @eval function LinearAlgebra.$f(dst::Collection, p::GB300Plan, src::Collection)
        _check_lengths(dst, src)
        foreach((d, s) -> $f(d, p, s), dst, src)
        dst
    end
end
function bmul!(dst::Collection, p::GB300Plan, src::Collection)
    _check_lengths(dst, src)
    foreach((d, s) -> bmul!(d, p, s), dst, src)
    dst
end
Base.:*(p::GB300Plan, src::Collection) = map(s -> p * s, src)
Base.:\(p::GB300Plan, src::Collection) = map(s -> p \ s, src)

# Spectral operators fused into the first backward pass (no counterpart in
# the reference API: the reference multiplies by i k in Fourier space, then
# calls ldiv!; examples/gradient.jl, test/include/FourierOperations.jl).
# dims are 1-based, L the domain lengths.
function ldiv_deriv!(dst::CuArray, p::GB300Plan, src::CuArray, dim::Integer, L::Real)
    check(ccall((:pfgb_backward_deriv, LIB), Cint,
                (Ptr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, Ptr{Cvoid}, Cint, Cint, Cdouble),
                p.handle, dst, src, stream_ptr(), 1, dim - 1, L))
    dst
end
function _deriv_sum!(dst::CuArray, p::GB300Plan, terms)
    n = length(terms)
    srcs = Ptr{Cvoid}[Ptr{Cvoid}(UInt(pointer(t[1]))) for t in terms]
    dims = Cint[t[2] - 1 for t in terms]
    coefs = Cdouble[t[3] for t in terms]
    lens = Cdouble[t[4] for t in terms]
    check(ccall((:pfgb_backward_deriv_sum, LIB), Cint,
                (Ptr{Cvoid}, CuPtr{Cvoid}, Ptr{Ptr{Cvoid}}, Cint, Ptr{Cint}, Ptr{Cdouble}, Ptr{Cdouble},
                 Ptr{Cvoid}, Cint),
                p.handle, dst, srcs, n, dims, coefs, lens, stream_ptr(), 1))
    dst
end
# ∇⋅u from the spectra uF (one per dimension)
ldiv_divergence!(dst::CuArray, p::GB300Plan, uF, L) =
    _deriv_sum!(dst, p, [(uF[d], d, 1.0, L[d]) for d in eachindex(uF)])
# ∇×u in 3D, one fused backward transform per component
function ldiv_curl!(ω, p::GB300Plan{T,3}, uF, L) where {T}
    for a in 1:3
        b, c = mod1(a + 1, 3), mod1(a + 2, 3)
        _deriv_sum!(ω[a], p, [(uF[c], b, 1.0, L[b]), (uF[b], c, -1.0, L[c])])
    end
    ω
end

# pfgb_batch_op (include/pencilfft_gb300.h)
struct BatchOp
    plan::Ptr{Cvoid}
    direction::Int32
    normalise::Int32
    dst::Ptr{Cvoid}
    src::Ptr{Cvoid}
    deriv_dim::Int32
    reserved::Int32
    deriv_length::Float64
end

const BATCH_FORMS = Dict(:graph => 0, :persistent => 1, :auto => 2, :measure => 3)

mutable struct GB300Batch
    handle::Ptr{Cvoid}
    keep::Vector{Any}  # the plans and arrays the recorded launches use
end

# ops: (mul!, dst, p, src), (ldiv!, dst, p, src) or (bmul!, dst, p, src), each
# optionally followed by (dim, L) for a fused spectral derivative (1-based dim)
function GB300Batch(ops::AbstractVector; form::Symbol = :graph)
    descs = BatchOp[]
    for op in ops
        f, dst, p, src = op[1], op[2], op[3], op[4]
        dir, norm = f === LinearAlgebra.mul! ? (1, 0) : f === LinearAlgebra.ldiv! ? (-1, 1) :
                    f === bmul! ? (-1, 0) : throw(ArgumentError("batch operations are mul!, ldiv! or bmul!"))
        dd, dl = length(op) >= 5 ? (Int32(op[5][1] - 1), Float64(op[5][2])) : (Int32(-1), 0.0)
        push!(descs, BatchOp(p.handle, dir, norm, Ptr{Cvoid}(UInt(pointer(dst))), Ptr{Cvoid}(UInt(pointer(src))),
                             dd, 0, dl))
    end
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:pfgb_batch_create_ex, LIB), Cint, (Ptr{BatchOp}, Cint, Cint, Ref{Ptr{Cvoid}}),
                descs, length(descs), BATCH_FORMS[form], h))
    b = GB300Batch(h[], collect(Any, ops))
    finalizer(b) do x
        x.handle == C_NULL || ccall((:pfgb_batch_destroy, LIB), Cint, (Ptr{Cvoid},), x.handle)
        x.handle = C_NULL
    end
    b
end

launch(b::GB300Batch) =
    (check(ccall((:pfgb_batch_launch, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), b.handle, stream_ptr())); b)

end # module
