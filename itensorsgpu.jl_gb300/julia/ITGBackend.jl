# Julia glue: ITensorsGPU.jl's storage-level overloads routed to libitg.so.
#
# This file is the drop-in for the reference's tensor layer: it defines the
# CuDense / CuDiag storage types and converters (src/tensor/cudense.jl:1-20,
# src/tensor/cudiag.jl:1-4) and every method the reference adds for them
# (src/ITensorsGPU.jl:32-43 import list; src/tensor/cudense.jl,
# src/tensor/cudiag.jl, src/tensor/culinearalgebra.jl, src/tensor/cutruncate.jl),
# with the cuTENSOR / cuBLAS / cuSOLVER bodies replaced by `ccall`s into the C
# ABI declared in include/itg.h.  Tensor data stays in CUDA.jl `CuVector`s; only
# device pointers cross the boundary.
#
# On top of the storage layer it routes the two-site update of ITensors' dmrg
# to the library: the ProjMPO eigensolve (KrylovKit.eigsolve on a two-site
# ProjMPO) goes to itg_davidson_heff2 and the bond split (replacebond!) to
# itg_factorize_trunc, both at the handle's precision (set_precision!).  Both
# hooks are methods for narrower argument types than ITensors' own and hand
# host tensors, noise terms and swapped sites back to ITensors' generic code.
#
# It cannot be executed in the build environment (no Julia toolchain); every
# ccall's argument list is checked against include/itg.h by
# tests/test_julia_glue_abi.py, and the Python ctypes layer (itg/_lib.py) that
# the GPU tests exercise binds the same symbols.
module ITGBackend

using CUDA
using ITensors
using ITensors.NDTensors
import ITensors.NDTensors: contract!!, contract!, permutedims!!, truncate!, outer!, _contract_scalar!,
                           contraction_output_type, zero_contraction_output, dense,
                           Dense, Diag, DiagTensor, UniformDiag, UniformDiagTensor, NonuniformDiagTensor,
                           Tensor, data, similar_type
import ITensors: replacebond!, cpu, storage
import KrylovKit
import LinearAlgebra

const libitg = joinpath(@__DIR__, "..", "libitg.so")

const ITG_OK = Cint(0)
const ITG_ERR_SHAPE = Cint(2)
const ITG_PREC_FP64 = Cint(0)
const ITG_PREC_SPLIT = Cint(1)

const _handle = Ref{Ptr{Cvoid}}(C_NULL)
const precision = Ref{Cint}(ITG_PREC_FP64)
set_precision!(p::Symbol) = (precision[] = p === :split ? ITG_PREC_SPLIT : ITG_PREC_FP64)

function handle()
    if _handle[] == C_NULL
        h = Ref{Ptr{Cvoid}}(C_NULL)
        st = ccall((:itg_create, libitg), Cint, (Cint, Ref{Ptr{Cvoid}}), CUDA.device().handle, h)
        st == ITG_OK || error("itg_create failed ($st)")
        # share CUDA.jl's task-local stream so ordering with CUDA.jl kernels holds
        st = ccall((:itg_set_stream, libitg), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), h[], CUDA.stream().handle)
        st == ITG_OK || error("itg_set_stream failed ($st)")
        _handle[] = h[]
    end
    return _handle[]
end

function check(st::Cint, what)
    st == ITG_OK && return nothing
    msg = unsafe_string(ccall((:itg_last_error, libitg), Cstring, (Ptr{Cvoid},), handle()))
    st == ITG_ERR_SHAPE && throw(DimensionMismatch("$what: $msg"))
    error("$what: $msg (status $st)")
end

# ------------------------------------------------------------ storage types
# The reference's aliases (cudense.jl:1-2, cudiag.jl:3-4): Dense / Diag
# storage whose data vector lives on the device.
const CuDense{ElT,VecT} = Dense{ElT,VecT} where {VecT<:CuVector}
const CuDenseTensor{ElT,N,StoreT,IndsT} = Tensor{ElT,N,StoreT,IndsT} where {StoreT<:CuDense}
const CuDiag{ElT,VecT} = Diag{ElT,VecT} where {VecT<:CuArray{ElT}}
const NonuniformCuDiagTensor{ElT,N,StoreT,IndsT} = Tensor{ElT,N,StoreT,IndsT} where {StoreT<:CuDiag}

# host <-> device converters (cudense.jl:4-12)
Dense{T,SA}(x::Dense{T,SB}) where {T<:Number,SA<:CuArray,SB<:Array} = Dense{T,SA}(CuArray(data(x)))
Dense{T,SA}(x::Dense{T,SB}) where {T<:Number,SA<:Array,SB<:CuArray} = Dense{T,SA}(Array(data(x)))
Dense{T,S}(size::Integer) where {T,S<:CuArray{<:T}} = Dense{T,S}(CUDA.zeros(T, size))
function Dense{T,S}(x::T, size::Integer) where {T,S<:CuArray{<:T}}
    arr = CuArray{T}(undef, size)
    fill!(arr, x)
    return Dense{T,S}(arr)
end
cpu(x::CuDense{T}) where {T<:Number} = Dense(Array(data(x)))
Base.complex(::Type{Dense{ElT,VT}}) where {ElT,VT<:CuArray} = Dense{complex(ElT),CuVector{complex(ElT)}}
Base.getindex(D::CuDense{<:Number}) = Array(data(D))[]
Base.getindex(D::CuDenseTensor{<:Number,0}) = store(D)[]
function Base.similar(::Type{<:CuDenseTensor{ElT}}, inds) where {ElT}
    return Tensor(Dense(CuVector{ElT}(undef, dim(inds))), inds)
end

# mode labels as int32, dims as int64 (column-major NDTensors layout)
_dims(T) = Int64[dims(inds(T))...]
_labels(l) = Int32[l...]

# element types: ITG_F64 = 0, ITG_C64 = 1 (ComplexF64, interleaved like Julia's own layout)
const ITGElT = Union{Float64,ComplexF64}
_dt(::Type{Float64}) = Cint(0)
_dt(::Type{ComplexF64}) = Cint(1)
_vptr(T) = reinterpret(CuPtr{Cvoid}, pointer(data(store(T))))
_cplx(x) = Cdouble[real(x), imag(x)]

# -------------------------------------------------------------- contraction
# C = alpha * T1 * T2 + beta * C over the shared labels, real, complex or mixed.
function _itg_contract!(R, labelsR, T1, labelsT1, T2, labelsT2, α, β)
    E1 = eltype(T1); E2 = eltype(T2)
    st = ccall((:itg_contract_z, libitg), Cint,
               (Ptr{Cvoid}, Cint, Cint, Ptr{Cdouble},
                CuPtr{Cvoid}, Cint, Ptr{Int64}, Ptr{Int32},
                CuPtr{Cvoid}, Cint, Ptr{Int64}, Ptr{Int32},
                Ptr{Cdouble},
                CuPtr{Cvoid}, Cint, Ptr{Int64}, Ptr{Int32}, Cint),
               handle(), _dt(E1), _dt(E2), _cplx(α),
               _vptr(T1), ndims(T1), _dims(T1), _labels(labelsT1),
               _vptr(T2), ndims(T2), _dims(T2), _labels(labelsT2),
               _cplx(β),
               _vptr(R), ndims(R), _dims(R), _labels(labelsR), precision[])
    check(st, "itg_contract_z")
    return R
end

# contract!! (cudense.jl:83-110): one call covers the scalar, outer-product and
# general cases (R is ComplexF64 when either operand is).
function contract!!(R::CuDenseTensor{<:ITGElT,NR}, labelsR::NTuple{NR},
                    T1::CuDenseTensor{E1,N1}, labelsT1::NTuple{N1},
                    T2::CuDenseTensor{E2,N2}, labelsT2::NTuple{N2}) where {NR,N1,N2,E1<:ITGElT,E2<:ITGElT}
    return _itg_contract!(R, labelsR, T1, labelsT1, T2, labelsT2, 1.0, 0.0)
end

# outer! (cudense.jl:74-81): the same engine with no shared label; R's
# indices are T1's followed by T2's.
function outer!(R::CuDenseTensor{<:ITGElT}, T1::CuDenseTensor{<:ITGElT}, T2::CuDenseTensor{<:ITGElT})
    N1 = ndims(T1); N2 = ndims(T2)
    l1 = ntuple(i -> i, N1); l2 = ntuple(i -> N1 + i, N2)
    return _itg_contract!(R, (l1..., l2...), T1, l1, T2, l2, 1.0, 0.0)
end

# _contract_scalar! (cudense.jl:129-168): two host scalars multiply on the
# host; a one-element tensor times a tensor is a rank-matching contraction.
function _contract_scalar!(R::CuDenseTensor{ElR}, labelsR, T1::Number, labelsT1, T2::Number, labelsT2,
                           α=one(ElR), β=zero(ElR)) where {ElR<:ITGElT}
    v = α * T1 * T2
    if !iszero(β)
        v += β * Array(data(store(R)))[1]
    end
    copyto!(data(store(R)), [ElR(v)])
    return R
end
function _contract_scalar!(R::CuDenseTensor{ElR}, labelsR, T1::CuDenseTensor{<:ITGElT}, labelsT1,
                           T2::CuDenseTensor{<:ITGElT}, labelsT2, α=one(ElR), β=zero(ElR)) where {ElR<:ITGElT}
    (length(data(store(T1))) == 1 || length(data(store(T2))) == 1) ||
        error("In _contract_scalar!, one tensor must be a scalar")
    return _itg_contract!(R, labelsR, T1, labelsT1, T2, labelsT2, α, β)
end

# --------------------------------------------------------------- permutation
# permute! (cudense.jl:447-500): B = A with B's index order.
function Base.permute!(B::CuDenseTensor{ElT,N}, A::CuDenseTensor{ElT,N}) where {ElT<:ITGElT,N}
    ia = inds(A); ib = inds(B)
    la = Int32[1:N...]
    lb = Int32[findfirst(==(i), ia) for i in ib]
    st = ccall((:itg_permute, libitg), Cint,
               (Ptr{Cvoid}, Cint, Cdouble, CuPtr{Cvoid}, Cint, Ptr{Int64}, Ptr{Int32},
                CuPtr{Cvoid}, Ptr{Int32}),
               handle(), _dt(ElT), 1.0, _vptr(A), N, _dims(A), la, _vptr(B), lb)
    check(st, "itg_permute")
    return vec(data(store(B)))
end

# permutedims!! (cudense.jl:52-60,112-127): B = permutedims(A, perm), or with a
# combining function f(b, a) applied elementwise to B and the permuted A.
_overwrite(r, t) = t
function permutedims!!(B::CuDenseTensor{ElT,N}, A::CuDenseTensor{ElT,N}, perm::NTuple{N,Int},
                       f::Function=_overwrite) where {ElT<:ITGElT,N}
    la = Int32[1:N...]
    lb = Int32[perm...]                 # B's index i is A's index perm[i]
    dst = f === _overwrite ? B : Tensor(Dense(CuVector{ElT}(undef, dim(inds(B)))), inds(B))
    st = ccall((:itg_permute, libitg), Cint,
               (Ptr{Cvoid}, Cint, Cdouble, CuPtr{Cvoid}, Cint, Ptr{Int64}, Ptr{Int32},
                CuPtr{Cvoid}, Ptr{Int32}),
               handle(), _dt(ElT), 1.0, _vptr(A), N, _dims(A), la, _vptr(dst), lb)
    check(st, "itg_permute")
    if dst !== B
        data(store(B)) .= f.(data(store(B)), data(store(dst)))
    end
    return B
end

# ------------------------------------------------------------ sums (+ and -)
# B (A's indices permuted to B's order) combined in place: alpha A + beta B.
function _axpby_permuted!(B::CuDenseTensor{ElT,N}, A::CuDenseTensor{ElT,N}, α, β) where {ElT<:ITGElT,N}
    ia = inds(A); ib = inds(B)
    la = Int32[findfirst(==(i), ib) for i in ia]
    lb = Int32[1:N...]
    st = ccall((:itg_axpby_permuted, libitg), Cint,
               (Ptr{Cvoid}, Cint, Cdouble, CuPtr{Cvoid}, Cint, Ptr{Int64}, Ptr{Int32},
                Cdouble, CuPtr{Cvoid}, Ptr{Int32}, CuPtr{Cvoid}),
               handle(), _dt(ElT), α, _vptr(A), N, _dims(A), la, β, _vptr(B), lb, _vptr(B))
    check(st, "itg_axpby_permuted")
    return B
end
# Base.:+ (cudense.jl:333-361): B = A + B, stored in B
Base.:+(B::CuDenseTensor{ElT,N}, A::CuDenseTensor{ElT,N}) where {ElT<:ITGElT,N} = _axpby_permuted!(B, A, 1.0, 1.0)
# Base.:- (cudense.jl:390-418): B = A - B, stored in B (the reference's operand order)
Base.:-(B::CuDenseTensor{ElT,N}, A::CuDenseTensor{ElT,N}) where {ElT<:ITGElT,N} = _axpby_permuted!(B, A, 1.0, -1.0)

# --------------------------------------------------------------- diagonals
_diagvec(D::UniformDiagTensor) = CuVector{Float64}([Float64(data(store(D)))])
_diagvec(D::NonuniformCuDiagTensor{Float64}) = data(store(D))
_isuniform(D::UniformDiagTensor) = Cint(1)
_isuniform(D::NonuniformCuDiagTensor) = Cint(0)
const RealCuDiagT = Union{UniformDiagTensor{<:Real},NonuniformCuDiagTensor{Float64}}

# Diag x Dense (cudiag.jl:105-118, 147-161): one gather / scale kernel; the
# reference densifies the diagonal (and ignores the index permutation for
# UniformDiag, cudiag.jl:105-112).
function _diag_contract!(C::CuDenseTensor{ElC}, Clabels, D::RealCuDiagT, Dlabels,
                         T::CuDenseTensor{ElT}, Tlabels) where {ElC<:ITGElT,ElT<:ITGElT}
    dv = _diagvec(D)
    st = GC.@preserve dv ccall((:itg_diag_contract, libitg), Cint,
               (Ptr{Cvoid}, Cint, Cdouble, CuPtr{Float64}, Cint, Cint, Ptr{Int64}, Ptr{Int32},
                CuPtr{Cvoid}, Cint, Ptr{Int64}, Ptr{Int32}, Cdouble,
                CuPtr{Cvoid}, Cint, Ptr{Int64}, Ptr{Int32}),
               handle(), _dt(ElT), 1.0, pointer(dv), _isuniform(D), ndims(D), _dims(D), _labels(Dlabels),
               _vptr(T), ndims(T), _dims(T), _labels(Tlabels), 0.0,
               _vptr(C), ndims(C), _dims(C), _labels(Clabels))
    check(st, "itg_diag_contract")
    return C
end
contract!(C::CuDenseTensor{<:ITGElT}, Clabels, A::RealCuDiagT, Alabels, B::CuDenseTensor{<:ITGElT}, Blabels) =
    _diag_contract!(C, Clabels, A, Alabels, B, Blabels)
contract!(C::CuDenseTensor{<:ITGElT}, Clabels, A::CuDenseTensor{<:ITGElT}, Alabels, B::RealCuDiagT, Blabels) =
    _diag_contract!(C, Clabels, B, Blabels, A, Alabels)

# Diag x Diag (cudiag.jl:120-145): elementwise product of the stored diagonals.
function contract!(C::NonuniformCuDiagTensor{Float64}, Clabels, A::RealCuDiagT, Alabels,
                   B::RealCuDiagT, Blabels)
    av = _diagvec(A); bv = _diagvec(B)
    n = length(data(store(C)))
    st = GC.@preserve av bv ccall((:itg_diag_diag, libitg), Cint,
               (Ptr{Cvoid}, Int64, Cdouble, CuPtr{Float64}, Cint, CuPtr{Float64}, Cint, CuPtr{Float64}),
               handle(), n, 1.0, pointer(av), _isuniform(A), pointer(bv), _isuniform(B),
               pointer(data(store(C))))
    check(st, "itg_diag_diag")
    return C
end

# dense(::NonuniformCuDiagTensor) (cudiag.jl:8-13)
function dense(T::NonuniformCuDiagTensor{Float64,N}) where {N}
    R = CuVector{Float64}(undef, dim(inds(T)))
    st = ccall((:itg_diag_to_dense, libitg), Cint,
               (Ptr{Cvoid}, CuPtr{Float64}, Cint, Cint, Ptr{Int64}, CuPtr{Float64}),
               handle(), pointer(data(store(T))), Cint(0), N, _dims(T), pointer(R))
    check(st, "itg_diag_to_dense")
    return Tensor(Dense(R), inds(T))
end

# output storage of Diag x CuDense contractions: CuDense of the promoted type
# (the reference's rules, cudiag.jl:44-98)
function contraction_output_type(::Type{<:NonuniformCuDiagTensor{E1}}, ::Type{<:CuDenseTensor{E2}},
                                 IndsR) where {E1,E2}
    E3 = promote_type(E1, E2)
    return Tensor{E3,length(IndsR.parameters),Dense{E3,CuVector{E3}},IndsR}
end
contraction_output_type(T1::Type{<:CuDenseTensor}, T2::Type{<:NonuniformCuDiagTensor}, IndsR) =
    contraction_output_type(T2, T1, IndsR)
function zero_contraction_output(T1::Union{UniformDiagTensor,NonuniformCuDiagTensor}, T2::CuDenseTensor, indsR)
    E3 = promote_type(eltype(T1), eltype(T2))
    return Tensor(Dense(CUDA.zeros(E3, dim(indsR))), indsR)
end
zero_contraction_output(T2::CuDenseTensor, T1::Union{UniformDiagTensor,NonuniformCuDiagTensor}, indsR) =
    zero_contraction_output(T1, T2, indsR)

# --------------------------------------------------------------- truncation
# truncate! (cutruncate.jl:1-93); legacy_gpu = true keeps the reference GPU
# rule, the default is ITensors' CPU rule.
function truncate!(P::CuVector{Float64}; maxdim::Int=length(P), mindim::Int=1,
                   cutoff::Float64=0.0, absoluteCutoff::Bool=false, doRelCutoff::Bool=true,
                   legacy_gpu::Bool=false)
    n = Ref{Int64}(); te = Ref{Cdouble}(); dc = Ref{Cdouble}()
    st = ccall((:itg_truncate, libitg), Cint,
               (Ptr{Cvoid}, CuPtr{Float64}, Int64, Int64, Int64, Cdouble, Cint, Cint, Cint,
                Ref{Int64}, Ref{Cdouble}, Ref{Cdouble}),
               handle(), pointer(P), length(P), maxdim, mindim, cutoff, absoluteCutoff,
               doRelCutoff, legacy_gpu, n, te, dc)
    check(st, "itg_truncate")
    return te[], dc[], P[1:n[]]
end

# ------------------------------------------------------- factorisations
# svd of an order-2 CuDense tensor (culinearalgebra.jl:33-72).  S is returned
# as Diag storage (the reference builds a dense dS x dS matrix).
function LinearAlgebra.svd(T::CuDenseTensor{Float64,2,IndsT}; maxdim::Int=minimum(dims(T)),
                           mindim::Int=1, cutoff::Float64=0.0, absoluteCutoff::Bool=false,
                           doRelCutoff::Bool=true, legacy_gpu::Bool=false, kwargs...) where {IndsT}
    m, n = dims(T); r = min(m, n)
    U = CuVector{Float64}(undef, m * r); S = CuVector{Float64}(undef, r)
    V = CuVector{Float64}(undef, n * r)
    k = Ref{Int64}(); te = Ref{Cdouble}(); dc = Ref{Cdouble}()
    st = ccall((:itg_svd_trunc, libitg), Cint,
               (Ptr{Cvoid}, Int64, Int64, CuPtr{Float64}, Int64, Int64, Int64, Cdouble, Cint,
                Cint, Cint, CuPtr{Float64}, CuPtr{Float64}, CuPtr{Float64}, Ref{Int64},
                Ref{Cdouble}, Ref{Cdouble}),
               handle(), m, n, pointer(data(store(T))), m, maxdim, mindim, cutoff,
               absoluteCutoff, doRelCutoff, legacy_gpu, pointer(U), pointer(S), pointer(V),
               k, te, dc)
    check(st, "itg_svd_trunc")
    dS = k[]
    u = eltype(IndsT)(dS); v = eltype(IndsT)(dS)
    Ut = Tensor(Dense(U[1:m*dS]), IndsT((ind(T, 1), u)))
    St = Tensor(Diag(S[1:dS]), IndsT((u, v)))
    Vt = Tensor(Dense(V[1:n*dS]), IndsT((ind(T, 2), v)))
    return Ut, St, Vt, Spectrum(Array(S[1:dS]) .^ 2, te[])
end

# svd / qr / eigen of order-2 ComplexF64 tensors (itg_svd_trunc_z, itg_qr_z,
# itg_eigh_trunc_z): A = U S V^H, A = Q R, A = U D U^H (Hermitian).
function LinearAlgebra.svd(T::CuDenseTensor{ComplexF64,2,IndsT}; maxdim::Int=minimum(dims(T)),
                           mindim::Int=1, cutoff::Float64=0.0, absoluteCutoff::Bool=false,
                           doRelCutoff::Bool=true, legacy_gpu::Bool=false, kwargs...) where {IndsT}
    m, n = dims(T); r = min(m, n)
    U = CuVector{ComplexF64}(undef, m * r); S = CuVector{Float64}(undef, r)
    V = CuVector{ComplexF64}(undef, n * r)
    k = Ref{Int64}(); te = Ref{Cdouble}(); dc = Ref{Cdouble}()
    st = ccall((:itg_svd_trunc_z, libitg), Cint,
               (Ptr{Cvoid}, Int64, Int64, CuPtr{Cvoid}, Int64, Int64, Int64, Cdouble, Cint,
                Cint, Cint, CuPtr{Cvoid}, CuPtr{Float64}, CuPtr{Cvoid}, Ref{Int64},
                Ref{Cdouble}, Ref{Cdouble}),
               handle(), m, n, _vptr(T), m, maxdim, mindim, cutoff, absoluteCutoff, doRelCutoff,
               legacy_gpu, reinterpret(CuPtr{Cvoid}, pointer(U)), pointer(S),
               reinterpret(CuPtr{Cvoid}, pointer(V)), k, te, dc)
    check(st, "itg_svd_trunc_z")
    dS = k[]
    u = eltype(IndsT)(dS); v = eltype(IndsT)(dS)
    Ut = Tensor(Dense(U[1:m*dS]), IndsT((ind(T, 1), u)))
    St = Tensor(Diag(S[1:dS]), IndsT((u, v)))
    Vt = Tensor(Dense(V[1:n*dS]), IndsT((ind(T, 2), v)))
    return Ut, St, Vt, Spectrum(Array(S[1:dS]) .^ 2, te[])
end

# qr (culinearalgebra.jl:110-121)
function LinearAlgebra.qr(T::CuDenseTensor{ElT,2,IndsT}) where {ElT<:ITGElT,IndsT}
    m, n = dims(T); r = min(m, n)
    Q = CuVector{ElT}(undef, m * r); R = CuVector{ElT}(undef, r * n)
    if ElT === ComplexF64
        st = ccall((:itg_qr_z, libitg), Cint,
                   (Ptr{Cvoid}, Int64, Int64, CuPtr{Cvoid}, Int64, CuPtr{Cvoid}, CuPtr{Cvoid}),
                   handle(), m, n, _vptr(T), m, reinterpret(CuPtr{Cvoid}, pointer(Q)),
                   reinterpret(CuPtr{Cvoid}, pointer(R)))
    else
        st = ccall((:itg_qr, libitg), Cint,
                   (Ptr{Cvoid}, Int64, Int64, CuPtr{Cvoid}, Int64, CuPtr{Cvoid}, CuPtr{Cvoid}),
                   handle(), m, n, _vptr(T), m, reinterpret(CuPtr{Cvoid}, pointer(Q)),
                   reinterpret(CuPtr{Cvoid}, pointer(R)))
    end
    check(st, "itg_qr")
    q = eltype(IndsT)(r)
    return Tensor(Dense(Q), IndsT((ind(T, 1), q))), Tensor(Dense(R), IndsT((q, ind(T, 2))))
end

# eigen(::Hermitian) (culinearalgebra.jl:74-108)
function LinearAlgebra.eigen(T::Hermitian{ElT,<:CuDenseTensor{ElT,2,IndsT}}; maxdim::Int=size(T, 1),
                             mindim::Int=size(T, 1), cutoff::Float64=0.0, kwargs...) where {ElT<:ITGElT,IndsT}
    A = parent(T); n = dims(A)[1]
    D = CuVector{Float64}(undef, n); U = CuVector{ElT}(undef, n * n)
    k = Ref{Int64}(); te = Ref{Cdouble}(); dc = Ref{Cdouble}()
    if ElT === ComplexF64
        st = ccall((:itg_eigh_trunc_z, libitg), Cint,
                   (Ptr{Cvoid}, Int64, CuPtr{Cvoid}, Int64, Int64, Int64, Cdouble, Cint, Cint, Cint,
                    CuPtr{Float64}, CuPtr{Cvoid}, Ref{Int64}, Ref{Cdouble}, Ref{Cdouble}),
                   handle(), n, _vptr(A), n, maxdim, mindim, cutoff, 0, 1, 0, pointer(D),
                   reinterpret(CuPtr{Cvoid}, pointer(U)), k, te, dc)
    else
        st = ccall((:itg_eigh_trunc, libitg), Cint,
                   (Ptr{Cvoid}, Int64, CuPtr{Cvoid}, Int64, Int64, Int64, Cdouble, Cint, Cint, Cint,
                    CuPtr{Float64}, CuPtr{Cvoid}, Ref{Int64}, Ref{Cdouble}, Ref{Cdouble}),
                   handle(), n, _vptr(A), n, maxdim, mindim, cutoff, 0, 1, 0, pointer(D),
                   reinterpret(CuPtr{Cvoid}, pointer(U)), k, te, dc)
    end
    check(st, "itg_eigh_trunc")
    dk = k[]; l = eltype(IndsT)(dk); r = eltype(IndsT)(dk)
    return Tensor(Diag(D[1:dk]), IndsT((l, r))), Tensor(Dense(U[1:n*dk]), IndsT((ind(A, 2), r))),
           Spectrum(Array(D[1:dk]), te[])
end

# factorize of an (m x n) column-major device matrix: the two-site bond split
# of dmrg (ITensors' factorize with which_decomp = "svd").  ortho = :left: L
# (m x k) orthonormal, C = S V^T (k x n); ortho = :right: L (n x k) orthonormal,
# C = U S (m x k).  method: 0 auto, 1 FP64 Jacobi, 2 mixed.
const ITG_ORTHO_LEFT = Cint(0)
const ITG_ORTHO_RIGHT = Cint(1)
function _factorize_trunc(A::CuVector{Float64}, m::Int, n::Int; ortho::Symbol=:left, maxdim::Int=min(m, n),
                          mindim::Int=1, cutoff::Float64=0.0, method::Int=0)
    r = min(m, n); big = max(m, n) * r
    Lb = CuVector{Float64}(undef, big); S = CuVector{Float64}(undef, r); Cb = CuVector{Float64}(undef, big)
    k = Ref{Int64}(); te = Ref{Cdouble}(); dc = Ref{Cdouble}()
    o = ortho === :left ? ITG_ORTHO_LEFT : ITG_ORTHO_RIGHT
    st = ccall((:itg_factorize_trunc, libitg), Cint,
               (Ptr{Cvoid}, Int64, Int64, CuPtr{Float64}, Int64, Int64, Int64, Cdouble, Cint, Cint, Cint,
                Cint, Cint, Cint, CuPtr{Float64}, CuPtr{Float64}, CuPtr{Float64}, Ref{Int64}, Ref{Cdouble},
                Ref{Cdouble}),
               handle(), m, n, pointer(A), m, maxdim, mindim, cutoff, 0, 1, 0, o, method,
               precision[], pointer(Lb), pointer(S), pointer(Cb), k, te, dc)
    check(st, "itg_factorize_trunc")
    return Lb, S, Cb, k[], te[]
end

# -------------------------------------------------------- dmrg two-site hooks
_iscu(T::ITensor) = storage(T) isa CuDense{Float64}
_devdata(T::ITensor) = data(storage(T))

# The kernel's operand layouts: L (a, wL, a'), W1 (wL, s1', s1, wM), W2 (wM,
# s2', s2, wR), R (b, wR, b'), phi (a, s1, s2, b); a missing edge link is a
# dimension of 1.  Each operand is permuted into that order on the device.
function _heff2_operands(PH::ProjMPO, phi::ITensor)
    b = PH.lpos + 1
    W1 = PH.H[b]; W2 = PH.H[b+1]
    s1 = commonind(W1, phi); s2 = commonind(W2, phi); wM = commonind(W1, W2)
    L = PH.lpos >= 1 ? PH.LR[PH.lpos] : nothing
    R = PH.rpos <= length(PH.H) ? PH.LR[PH.rpos] : nothing
    a = L === nothing ? nothing : commonind(L, phi)
    wL = L === nothing ? nothing : commonind(L, W1)
    c = R === nothing ? nothing : commonind(R, phi)
    wR = R === nothing ? nothing : commonind(R, W2)
    keep(xs...) = filter(!isnothing, collect(xs))
    Lp = L === nothing ? nothing : permute(L, a, wL, prime(a))
    W1p = permute(W1, keep(wL, prime(s1), s1, wM)...)
    W2p = permute(W2, keep(wM, prime(s2), s2, wR)...)
    Rp = R === nothing ? nothing : permute(R, c, wR, prime(c))
    phip = permute(phi, keep(a, s1, s2, c)...)
    dimof(i) = i === nothing ? 1 : dim(i)
    return (Lp, W1p, W2p, Rp, phip, dimof(a), dimof(c), dim(s1), dimof(wL), dim(wM), dimof(wR))
end


# KrylovKit.eigsolve on a two-site ProjMPO (what ITensors' dmrg calls each
# bond): one itg_davidson_heff2 call (ProjMPO product as the fused H_eff
# chain, Davidson with the diagonal preconditioner); host tensors go to
# KrylovKit's generic method.
function KrylovKit.eigsolve(PH::ProjMPO, phi::Union{ITensor{3},ITensor{4}}, howmany::Int, which::Symbol;
                            krylovdim::Int=3, maxiter::Int=1, tol::Real=1e-14, kwargs...)
    if !(_iscu(phi) && PH.nsite == 2)
        return invoke(KrylovKit.eigsolve, Tuple{Any,Any,Int,Symbol}, PH, phi, howmany, which;
                      krylovdim=krylovdim, maxiter=maxiter, tol=tol, kwargs...)
    end
    Lp, W1p, W2p, Rp, phip, chiL, chiR, d, wL, wM, wR = _heff2_operands(PH, phi)
    one_ = CuVector{Float64}([1.0])   # edge environments: a 1 x 1 x 1 tensor holding 1
    Ld = Lp === nothing ? one_ : _devdata(Lp)
    Rd = Rp === nothing ? one_ : _devdata(Rp)
    W1d = _devdata(W1p); W2d = _devdata(W2p)
    x = copy(_devdata(phip))
    e = Ref{Cdouble}(); nmv = Ref{Cint}()
    st = GC.@preserve one_ Ld Rd W1d W2d x ccall((:itg_davidson_heff2, libitg), Cint,
               (Ptr{Cvoid}, Int64, Int64, Int64, Int64, Int64, Int64, CuPtr{Float64},
                CuPtr{Float64}, CuPtr{Float64}, CuPtr{Float64}, CuPtr{Float64}, Cint, Cint,
                Cdouble, Cint, Ref{Cdouble}, Ref{Cint}),
               handle(), chiL, chiR, d, wL, wM, wR, pointer(Ld), pointer(W1d), pointer(W2d), pointer(Rd),
               pointer(x), krylovdim, maxiter, tol, precision[], e, nmv)
    check(st, "itg_davidson_heff2")
    vec_ = ITensor(Dense(x), inds(phip))
    return [e[]], [vec_], (numops=Int(nmv[]), converged=1)
end

# replacebond! (ITensors' dmrg bond split): factorize phi across the bond with
# itg_factorize_trunc (the orthonormal factor built from rotations, the other
# one a matrix product) at the handle's precision; noise terms, swapped sites
# and host tensors go to ITensors' generic method.
function replacebond!(M::MPS, b::Int, phi::Union{ITensor{3},ITensor{4}}; kwargs...)
    if !_iscu(phi) || get(kwargs, :eigen_perturbation, nothing) !== nothing || get(kwargs, :swapsites, false) ||
       get(kwargs, :which_decomp, nothing) ∉ (nothing, "svd")
        return invoke(replacebond!, Tuple{MPS,Int,ITensor}, M, b, phi; kwargs...)
    end
    ortho::String = get(kwargs, :ortho, "left")
    Linds = commoninds(phi, M[b])
    Rinds = uniqueinds(phi, M[b])
    phip = permute(phi, Linds..., Rinds...)
    m = prod(dim.(Linds)); n = prod(dim.(Rinds))
    Lb, S, Cb, dk, te = _factorize_trunc(_devdata(phip), m, n;
                                         ortho=ortho == "left" ? :left : :right,
                                         maxdim=get(kwargs, :maxdim, min(m, n)), mindim=get(kwargs, :mindim, 1),
                                         cutoff=Float64(get(kwargs, :cutoff, 0.0)),
                                         method=get(kwargs, :svd_method, 0))
    l = Index(dk; tags=tags(linkind(M, b)))
    if ortho == "left"
        M[b] = ITensor(Dense(Lb[1:m*dk]), IndexSet(Linds..., l))
        M[b+1] = ITensor(Dense(Cb[1:dk*n]), IndexSet(l, Rinds...))
        # orthogonality centre at b + 1
        ITensors.setleftlim!(M, b)
        ITensors.setrightlim!(M, b + 2)
    else
        M[b] = ITensor(Dense(Cb[1:m*dk]), IndexSet(Linds..., l))
        M[b+1] = ITensor(Dense(Lb[1:n*dk]), IndexSet(Rinds..., l))
        # orthogonality centre at b
        ITensors.setleftlim!(M, b - 1)
        ITensors.setrightlim!(M, b + 1)
    end
    return Spectrum(Array(S[1:dk]) .^ 2, te)
end

end # module
