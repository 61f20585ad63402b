# Julia glue: ITensorsGPU.jl's storage-level overloads routed to libitg.so.
#
# This file mirrors the methods the reference adds for CuDense/CuDiag storage
# (src/ITensorsGPU.jl:32-43 import list; src/tensor/cudense.jl,
# src/tensor/cudiag.jl, src/tensor/culinearalgebra.jl, src/tensor/cutruncate.jl)
# and replaces their cuTENSOR / cuBLAS / cuSOLVER bodies with `ccall`s into the
# C ABI declared in include/itg.h.  Tensor data stays in CUDA.jl `CuVector`s;
# only device pointers cross the boundary.
#
# It cannot be executed in the build environment (no Julia toolchain); it is
# kept in step with include/itg.h and the Python ctypes layer (itg/_lib.py),
# which the tests exercise.
module ITGBackend

using CUDA
using ITensors
using ITensors.NDTensors
import ITensors.NDTensors: contract!!, permutedims!!, truncate!
import LinearAlgebra

const libitg = joinpath(@__DIR__, "..", "libitg.so")

const ITG_OK = Cint(0)
const ITG_ERR_SHAPE = Cint(2)
const ITG_PREC_FP64 = Cint(0)
const ITG_PREC_SPLIT = Cint(1)

const _handle = Ref{Ptr{Cvoid}}(C_NULL)
const precision = Ref{Cint}(ITG_PREC_FP64)

function handle()
    if _handle[] == C_NULL
        h = Ref{Ptr{Cvoid}}(C_NULL)
        st = ccall((:itg_create, libitg), Cint, (Cint, Ref{Ptr{Cvoid}}), CUDA.device().handle, h)
        st == ITG_OK || error("itg_create failed ($st)")
        # share CUDA.jl's task-local stream so ordering with CUDA.jl kernels holds
        ccall((:itg_set_stream, libitg), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), h[], CUDA.stream().handle)
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

# mode labels as int32, dims as int64 (column-major NDTensors layout)
_dims(T) = Int64[dims(inds(T))...]
_labels(l) = Int32[l...]

# element types: ITG_F64 = 0, ITG_C64 = 1 (ComplexF64, interleaved like Julia's own layout)
const ITGElT = Union{Float64,ComplexF64}
_dt(::Type{Float64}) = Cint(0)
_dt(::Type{ComplexF64}) = Cint(1)
_vptr(T) = reinterpret(CuPtr{Cvoid}, pointer(data(store(T))))

# contract!! (src/tensor/cudense.jl:83-110): one call covers the scalar,
# outer-product and general cases, real, complex and mixed operands (R is
# ComplexF64 when either operand is).
function contract!!(R::CuDenseTensor{<:ITGElT,NR}, labelsR::NTuple{NR},
                    T1::CuDenseTensor{E1,N1}, labelsT1::NTuple{N1},
                    T2::CuDenseTensor{E2,N2}, labelsT2::NTuple{N2}) where {NR,N1,N2,E1<:ITGElT,E2<:ITGElT}
    st = ccall((:itg_contract_z, libitg), Cint,
               (Ptr{Cvoid}, Cint, Cint, Ptr{Cdouble},
                CuPtr{Cvoid}, Cint, Ptr{Int64}, Ptr{Int32},
                CuPtr{Cvoid}, Cint, Ptr{Int64}, Ptr{Int32},
                Ptr{Cdouble},
                CuPtr{Cvoid}, Cint, Ptr{Int64}, Ptr{Int32}, Cint),
               handle(), _dt(E1), _dt(E2), Cdouble[1.0, 0.0],
               _vptr(T1), N1, _dims(T1), _labels(labelsT1),
               _vptr(T2), N2, _dims(T2), _labels(labelsT2),
               Cdouble[0.0, 0.0],
               _vptr(R), NR, _dims(R), _labels(labelsR), precision[])
    check(st, "itg_contract_z")
    return R
end

# permute! (src/tensor/cudense.jl:447-500)
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

# Base.:+ on CuDense tensors (src/tensor/cudense.jl:333-361): B .= A(permuted) + B
function Base.:+(B::CuDenseTensor{ElT,N}, A::CuDenseTensor{ElT,N}) where {ElT<:ITGElT,N}
    ia = inds(A); ib = inds(B)
    la = Int32[findfirst(==(i), ib) for i in ia]
    lb = Int32[1:N...]
    st = ccall((:itg_axpby_permuted, libitg), Cint,
               (Ptr{Cvoid}, Cint, Cdouble, CuPtr{Cvoid}, Cint, Ptr{Int64}, Ptr{Int32},
                Cdouble, CuPtr{Cvoid}, Ptr{Int32}, CuPtr{Cvoid}),
               handle(), _dt(ElT), 1.0, _vptr(A), N, _dims(A), la, 1.0, _vptr(B), lb, _vptr(B))
    check(st, "itg_axpby_permuted")
    return B
end

# truncate! (src/tensor/cutruncate.jl:1-93); legacy_gpu = true keeps the
# reference GPU rule, the default is ITensors' CPU rule.
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

# svd of an order-2 CuDense tensor (src/tensor/culinearalgebra.jl:33-72).
# S is returned as Diag storage (the reference builds a dense dS x dS matrix).
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

function LinearAlgebra.qr(T::CuDenseTensor{ElT,2,IndsT}) where {ElT<:ITGElT,IndsT}
    m, n = dims(T); r = min(m, n)
    Q = CuVector{ElT}(undef, m * r); R = CuVector{ElT}(undef, r * n)
    st = ccall((ElT === ComplexF64 ? :itg_qr_z : :itg_qr, libitg), Cint,
               (Ptr{Cvoid}, Int64, Int64, CuPtr{Cvoid}, Int64, CuPtr{Cvoid}, CuPtr{Cvoid}),
               handle(), m, n, _vptr(T), m, reinterpret(CuPtr{Cvoid}, pointer(Q)),
               reinterpret(CuPtr{Cvoid}, pointer(R)))
    check(st, "itg_qr")
    q = eltype(IndsT)(r)
    return Tensor(Dense(Q), IndsT((ind(T, 1), q))), Tensor(Dense(R), IndsT((q, ind(T, 2))))
end

function LinearAlgebra.eigen(T::Hermitian{ElT,<:CuDenseTensor{ElT,2,IndsT}}; maxdim::Int=size(T, 1),
                             mindim::Int=size(T, 1), cutoff::Float64=0.0, kwargs...) where {ElT<:ITGElT,IndsT}
    A = parent(T); n = dims(A)[1]
    D = CuVector{Float64}(undef, n); U = CuVector{ElT}(undef, n * n)
    k = Ref{Int64}(); te = Ref{Cdouble}(); dc = Ref{Cdouble}()
    st = ccall((ElT === ComplexF64 ? :itg_eigh_trunc_z : :itg_eigh_trunc, libitg), Cint,
               (Ptr{Cvoid}, Int64, CuPtr{Cvoid}, Int64, Int64, Int64, Cdouble, Cint, Cint, Cint,
                CuPtr{Float64}, CuPtr{Cvoid}, Ref{Int64}, Ref{Cdouble}, Ref{Cdouble}),
               handle(), n, _vptr(A), n, maxdim, mindim, cutoff, 0, 1, 0, pointer(D),
               reinterpret(CuPtr{Cvoid}, pointer(U)), k, te, dc)
    check(st, "itg_eigh_trunc")
    dk = k[]; l = eltype(IndsT)(dk); r = eltype(IndsT)(dk)
    return Tensor(Diag(D[1:dk]), IndsT((l, r))), Tensor(Dense(U[1:n*dk]), IndsT((ind(A, 2), r))),
           Spectrum(Array(D[1:dk]), te[])
end

# factorize of an order-2 CuDense tensor (the two-site bond split of dmrg,
# ITensors' factorize with which_decomp = "svd"): ortho = "left" returns L with
# orthonormal columns and R = S V^T, ortho = "right" returns L = U S and R
# with orthonormal rows.  method: 0 auto, 1 FP64 Jacobi, 2 mixed.
const ITG_ORTHO_LEFT = Cint(0)
const ITG_ORTHO_RIGHT = Cint(1)
function factorize_svd(T::CuDenseTensor{Float64,2,IndsT}; ortho::String="left", maxdim::Int=minimum(dims(T)),
                       mindim::Int=1, cutoff::Float64=0.0, method::Int=0, kwargs...) where {IndsT}
    m, n = dims(T); r = min(m, n); big = max(m, n) * r
    Lb = CuVector{Float64}(undef, big); S = CuVector{Float64}(undef, r); Cb = CuVector{Float64}(undef, big)
    k = Ref{Int64}(); te = Ref{Cdouble}(); dc = Ref{Cdouble}()
    o = ortho == "left" ? ITG_ORTHO_LEFT : ITG_ORTHO_RIGHT
    st = ccall((:itg_factorize_trunc, libitg), Cint,
               (Ptr{Cvoid}, Int64, Int64, CuPtr{Float64}, Int64, Int64, Int64, Cdouble, Cint, Cint, Cint,
                Cint, Cint, Cint, CuPtr{Float64}, CuPtr{Float64}, CuPtr{Float64}, Ref{Int64}, Ref{Cdouble},
                Ref{Cdouble}),
               handle(), m, n, pointer(data(store(T))), m, maxdim, mindim, cutoff, 0, 1, 0, o, method,
               precision[], pointer(Lb), pointer(S), pointer(Cb), k, te, dc)
    check(st, "itg_factorize_trunc")
    dk = k[]; l = eltype(IndsT)(dk)
    if ortho == "left"
        Lt = Tensor(Dense(Lb[1:m*dk]), IndsT((ind(T, 1), l)))
        Rt = Tensor(Dense(Cb[1:dk*n]), IndsT((l, ind(T, 2))))
    else
        Lt = Tensor(Dense(Cb[1:m*dk]), IndsT((ind(T, 1), l)))
        Rt = Tensor(Dense(Lb[1:n*dk]), IndsT((ind(T, 2), l)))
    end
    return Lt, Rt, Spectrum(Array(S[1:dk]) .^ 2, te[])
end

# ProjMPO product + eigensolver for the two-site update: the dmrg sweep calls
# this with the device buffers of L, W1, W2, R and phi.
function davidson_heff2!(phi::CuVector{Float64}, L, W1, W2, R, chiL, chiR, d, wL, wM, wR;
                         krylovdim::Int=3, maxiter::Int=2, tol::Float64=1e-14)
    e = Ref{Cdouble}(); nmv = Ref{Cint}()
    st = ccall((:itg_davidson_heff2, libitg), Cint,
               (Ptr{Cvoid}, Int64, Int64, Int64, Int64, Int64, Int64, CuPtr{Float64},
                CuPtr{Float64}, CuPtr{Float64}, CuPtr{Float64}, CuPtr{Float64}, Cint, Cint,
                Cdouble, Cint, Ref{Cdouble}, Ref{Cint}),
               handle(), chiL, chiR, d, wL, wM, wR, pointer(L), pointer(W1), pointer(W2),
               pointer(R), pointer(phi), krylovdim, maxiter, tol, precision[], e, nmv)
    check(st, "itg_davidson_heff2")
    return e[], phi
end

end # module
