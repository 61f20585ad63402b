"""Davidson eigensolver for a Hermitian linear map of ITensors.

ITensors' `davidson(A, phi; maxiter, ...)` (external to the reference, used by
test/test_cuiterativesolvers.jl:13-28 with an `ITensorMap` wrapper) for real
and complex tensors: A is any callable ITensor -> ITensor.  The basis vectors,
matrix-vector products and every vector update stay on the device (contract,
scale, axpby, norm in libitg.so); the Rayleigh-Ritz problem of the subspace
(k x k, Hermitian) is solved by itg_eigh_trunc, a complex one through its real
2k x 2k representation [[Re, -Im], [Im, Re]] whose eigenvalues come in equal
pairs and whose eigenvectors [x; y] give the complex eigenvector x + i y.

The H_eff eigensolver of dmrg is the fused itg_davidson_heff2; this one serves
general maps.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import tensor as T
from .tensor import ITensor


class ITensorMap:
    """x -> noprime(A * x) for an operator ITensor A with index pairs (s, s')
    (the wrapper of test/test_cuiterativesolvers.jl:7-11)."""

    def __init__(self, A: ITensor):
        self.A = A

    def __call__(self, x: ITensor) -> ITensor:
        y = T.contract(self.A, x)
        return y.replaceinds(y.inds, [i.noprime() if i.plev > 0 else i for i in y.inds])


def _inner(a: ITensor, b: ITensor):
    """<a|b> = (dag(a) * b)[] with b permuted to a's index order."""
    return T.contract(T.dag(a), b).scalar()


def _lowest_eig(Hs: np.ndarray):
    """Lowest eigenpair of a small Hermitian matrix on the device (itg_eigh_trunc)."""
    k = Hs.shape[0]
    cplx = np.iscomplexobj(Hs) and np.abs(Hs.imag).max() > 0
    M = np.block([[Hs.real, -Hs.imag], [Hs.imag, Hs.real]]) if cplx else Hs.real
    n = M.shape[0]
    M = 0.5 * (M + M.T)
    import torch
    Md = torch.from_numpy(np.asfortranarray(M).ravel(order="F").copy()).to(T._dev())
    D = T.empty_dev(n)
    U = T.empty_dev(n * n)
    kk = C.c_int64()
    te = C.c_double()
    dc = C.c_double()
    T._h().call("itg_eigh_trunc", C.c_int64(n), T._ptr(Md), C.c_int64(n), C.c_int64(n), C.c_int64(n),
                C.c_double(0.0), 0, 1, 0, T._ptr(D), T._ptr(U), C.byref(kk), C.byref(te), C.byref(dc))
    m = int(kk.value)
    lam = float(D[m - 1].item())                       # descending order: the last kept is the lowest
    u = U[(m - 1) * n: m * n].cpu().numpy()
    if cplx:
        y = u[:k] + 1j * u[k:]
        return lam, y / np.linalg.norm(y)
    return lam, u / np.linalg.norm(u)


def _combine(coeffs, vecs) -> ITensor:
    """sum_i c_i v_i (real or complex coefficients)."""
    out = None
    for c, v in zip(coeffs, vecs):
        term = T._scale(v, complex(c) if np.iscomplexobj(c) else float(c))
        out = term if out is None else T._axpby(1.0, term, 1.0, out)
    return out


def davidson(A, x0: ITensor, *, maxiter: int = 10, tol: float = 1e-12, restart_dim: int = 30):
    """Lowest eigenpair (lambda, x) of the Hermitian map A, starting from x0.

    maxiter counts the vectors added to the subspace (the Krylov dimension of
    ITensors' davidson); the subspace restarts from the current Ritz vector
    when it reaches restart_dim.  Stops when |A x - lambda x| <= tol |lambda|.
    """
    x = T._scale(x0, 1.0 / T.norm(x0))
    V = [x]
    AV = [A(x)]
    lam = None
    for it in range(max(1, maxiter) + 1):
        k = len(V)
        Hs = np.empty((k, k), dtype=complex)
        for i in range(k):
            for j in range(i, k):
                hij = _inner(V[i], AV[j])
                Hs[i, j] = hij
                Hs[j, i] = np.conj(hij)
        lam, y = _lowest_eig(Hs)
        x = _combine(y, V)
        Ax = _combine(y, AV)
        r = T._axpby(-lam, x, 1.0, Ax)
        rn = T.norm(r)
        if rn <= tol * max(abs(lam), 1e-300) or it == maxiter:
            break
        if k >= restart_dim:
            V, AV = [x], [Ax]
        t = r
        for _ in range(2):                               # Gram-Schmidt twice against the basis
            for v in V:
                t = T._axpby(1.0, T._scale(v, -_inner(v, t)), 1.0, t)
        tn = T.norm(t)
        if tn <= 1e-14 * rn:
            break
        t = T._scale(t, 1.0 / tn)
        V.append(t)
        AV.append(A(t))
    return lam, x
