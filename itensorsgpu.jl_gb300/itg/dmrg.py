"""Two-site DMRG sweeps over libitg.so (the dmrg(H, psi, sweeps) entry point).

ITensors.jl's ``dmrg`` (ITensors 0.2, called at examples/dmrg.jl:25 and
test/dmrg.jl:27,75 of the reference) sweeps bonds b = 1..N-1 and back
(``sweepnext``), and for every bond: forms phi = psi[b] * psi[b+1], finds the
lowest eigenvector of the ProjMPO effective Hamiltonian, factorises it with a
truncated SVD (``replacebond!``/``factorize``) and updates the projected
environments.  This module does the same with every tensor operation in
libitg.so: Davidson with the H_eff chain (itg_davidson_heff2), the truncated
SVD with on-device truncation (itg_svd_trunc_ex), gather/scale Diag kernels for
S and gather-GEMM contractions for the environments, all at the run's
precision.  The host only orchestrates.
"""
from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass, field

import numpy as np

from . import tensor as T
from ._lib import ITG_F64, PREC_FP64, PREC_SPLIT, NotConverged, i32arr, i64arr
from .mps import MPO, MPS
from .tensor import Dense, ITensor, Index


class Sweeps:
    """Sweep schedule (ITensors' Sweeps with maxdim!/mindim!/cutoff!/noise!)."""

    def __init__(self, nsweep: int, maxdim=None, mindim=None, cutoff=None, noise=None):
        self.nsweep = int(nsweep)
        self._maxdim = list(maxdim) if maxdim is not None else [1]
        self._mindim = list(mindim) if mindim is not None else [1]
        self._cutoff = list(cutoff) if cutoff is not None else [0.0]
        self._noise = list(noise) if noise is not None else [0.0]

    @staticmethod
    def _at(v, i):
        return v[min(i, len(v) - 1)]

    def maxdim(self, i):
        return int(self._at(self._maxdim, i))

    def mindim(self, i):
        return int(self._at(self._mindim, i))

    def cutoff(self, i):
        return float(self._at(self._cutoff, i))

    def noise(self, i):
        return float(self._at(self._noise, i))


def maxdim_(sw: Sweeps, *v):
    sw._maxdim = list(v)


def mindim_(sw: Sweeps, *v):
    sw._mindim = list(v)


def cutoff_(sw: Sweeps, *v):
    sw._cutoff = list(v)


def noise_(sw: Sweeps, *v):
    sw._noise = list(v)


def sweepnext(N: int):
    """(b, half) pairs of one sweep: bonds 0..N-2 left to right, then back."""
    for b in range(N - 1):
        yield b, 1
    for b in range(N - 2, -1, -1):
        yield b, 2


@dataclass
class SweepRecord:
    energy: float
    maxlinkdim: int
    maxtruncerr: float
    seconds: float
    matvecs: int
    # seconds per phase (eigensolver, factorisation, environment update, the
    # rest); phases are separated by stream synchronisations only when
    # dmrg(..., phase_timing=True)
    phases: dict = field(default_factory=dict)
    # factorisations of the sweep: Jacobi sweeps in total, and how many mixed
    # SVDs failed their refinement check and were redone in FP64
    svd_sweeps: int = 0
    svd_fallbacks: int = 0


@dataclass
class DMRGResult:
    energy: float
    psi: MPS
    sweeps: list = field(default_factory=list)


# ---------------------------------------------------------- raw helpers
def _ptr(t):
    return C.c_void_p(t.data_ptr())


def _contract_raw(h, A, dA, mA, B, dB, mB, dC, mC, precision=PREC_FP64, out=None):
    n = int(np.prod(dC)) if len(dC) else 1
    if out is None:
        out = T.empty_dev(n)
    h.call("itg_contract", ITG_F64, C.c_double(1.0), _ptr(A), len(dA), i64arr(dA), i32arr(mA),
           _ptr(B), len(dB), i64arr(dB), i32arr(mB), C.c_double(0.0), _ptr(out), len(dC),
           i64arr(dC), i32arr(mC), int(precision))
    return out


def _diag_raw(h, d, dD, mD, Tt, dT, mT, dC, mC):
    n = int(np.prod(dC))
    out = T.empty_dev(n)
    h.call("itg_diag_contract", ITG_F64, C.c_double(1.0), _ptr(d), 0, len(dD), i64arr(dD), i32arr(mD),
           _ptr(Tt), len(dT), i64arr(dT), i32arr(mT), C.c_double(0.0), _ptr(out), len(dC),
           i64arr(dC), i32arr(mC))
    return out


def _permute_raw(h, A, dA, mA, mB):
    out = T.empty_dev(int(np.prod(dA)))
    h.call("itg_permute", ITG_F64, C.c_double(1.0), _ptr(A), len(dA), i64arr(dA), i32arr(mA),
           _ptr(out), i32arr(mB))
    return out


class _Chain:
    """Raw device view of an MPS / MPO for the sweep: arrays + shapes."""

    def __init__(self, psi: MPS, H: MPO):
        self.N = len(psi)
        self.A = []   # (chiL, d, chiR)
        self.Ad = []
        for t in psi.tensors:
            self.A.append(t.store.data.contiguous())
            self.Ad.append(t.dims)
        self.W = []
        self.Wd = []
        for t in H.tensors:
            self.W.append(t.store.data.contiguous())
            self.Wd.append(t.dims)  # (wl, d, d, wr)


def _env_left(h, Lt, Ld, A, Ad, W, Wd, prec):
    """L_new[b, x, b'] = sum L[a,w,a'] A[a,s,b] W[w,s',s,x] A[a',s',b']."""
    a, d, b = Ad
    wl, _, _, x = Wd
    # modes: a=1 w=2 ap=3 s=4 b=5 sp=6 x=7 bp=8
    t1 = _contract_raw(h, Lt, Ld, [1, 2, 3], A, Ad, [1, 4, 5], (wl, a, d, b), [2, 3, 4, 5], prec)
    t2 = _contract_raw(h, t1, (wl, a, d, b), [2, 3, 4, 5], W, Wd, [2, 6, 4, 7], (a, b, d, x),
                       [3, 5, 6, 7], prec)
    Ln = _contract_raw(h, t2, (a, b, d, x), [3, 5, 6, 7], A, Ad, [3, 6, 8], (b, x, b), [5, 7, 8], prec)
    return Ln, (b, x, b)


def _env_right(h, Rt, Rd, A, Ad, W, Wd, prec):
    """R_new[a, w, a'] = sum A[a,s,b] W[w,s',s,x] R[b,x,b'] A[a',s',b']."""
    a, d, b = Ad
    w, _, _, x = Wd
    # modes: a=1 s=2 b=3 x=4 bp=5 w=6 sp=7 ap=8
    t1 = _contract_raw(h, A, Ad, [1, 2, 3], Rt, Rd, [3, 4, 5], (a, d, x, b), [1, 2, 4, 5], prec)
    t2 = _contract_raw(h, t1, (a, d, x, b), [1, 2, 4, 5], W, Wd, [6, 7, 2, 4], (a, b, w, d),
                       [1, 5, 6, 7], prec)
    Rn = _contract_raw(h, t2, (a, b, w, d), [1, 5, 6, 7], A, Ad, [8, 7, 5], (a, w, a), [1, 6, 8], prec)
    return Rn, (a, w, a)


def _contract_acc(h, alpha, A, dA, mA, B, dB, mB, out, dC, mC, precision):
    """out = alpha * (A x B) + out."""
    h.call("itg_contract", ITG_F64, C.c_double(alpha), _ptr(A), len(dA), i64arr(dA), i32arr(mA),
           _ptr(B), len(dB), i64arr(dB), i32arr(mB), C.c_double(1.0), _ptr(out), len(dC),
           i64arr(dC), i32arr(mC), int(precision))


def _noise_split(h, phi, shape, Lt, Ld, W1, W1d, W2, W2d, Rt, Rd, ha, noise, maxdim, mindim, cutoff,
                 legacy, precision):
    """Bond split through the perturbed density matrix (the noise > 0 path).

    ITensors 0.2's dmrg with noise adds noise * (nt nt^T) to the reduced
    density matrix of phi, nt being phi with the environment and MPO tensor of
    the side being kept applied and the MPO link left open (its noiseterm),
    then keeps the leading eigenvectors of the sum (factorize with
    which_decomp = "eigen", eigen(::Hermitian), src/tensor/culinearalgebra.jl:74-108).
    Left-moving half (ha == 1): rho over (a d1), A_b = U, A_{b+1} = U^T phi.
    Right-moving half: rho over (d2 c), A_{b+1} = V^T, A_b = phi V.
    Returns (A_b, A_{b+1}, k, truncerr).
    """
    a, d1, d2, c = shape
    w, x = W1d[0], W1d[3]
    y = W2d[3]
    if ha == 1:
        m = a * d1
        rho = _contract_raw(h, phi, shape, [1, 2, 3, 4], phi, shape, [5, 6, 3, 4], (a, d1, a, d1),
                            [1, 2, 5, 6], precision)
        # t1[w, a', s, d2, c] = L[a, w, a'] phi[a, s, d2, c]
        t1 = _contract_raw(h, Lt, Ld, [1, 7, 5], phi, shape, [1, 2, 3, 4], (w, a, d1, d2, c), [7, 5, 2, 3, 4],
                           precision)
        # nt[a', t, x, d2, c] = t1[w, a', s, d2, c] W1[w, t, s, x]
        nt = _contract_raw(h, t1, (w, a, d1, d2, c), [7, 5, 2, 3, 4], W1, W1d, [7, 6, 2, 8], (a, d1, x, d2, c),
                           [5, 6, 8, 3, 4], precision)
        ntd = (a, d1, x, d2, c)
        _contract_acc(h, noise, nt, ntd, [5, 6, 8, 3, 4], nt, ntd, [9, 10, 8, 3, 4], rho, (a, d1, a, d1),
                      [5, 6, 9, 10], precision)
    else:
        m = d2 * c
        rho = _contract_raw(h, phi, shape, [1, 2, 3, 4], phi, shape, [1, 2, 5, 6], (d2, c, d2, c),
                            [3, 4, 5, 6], precision)
        # t1[a, d1, s, x, c'] = phi[a, d1, s, c] R[c, x, c']
        t1 = _contract_raw(h, phi, shape, [1, 2, 3, 4], Rt, Rd, [4, 8, 6], (a, d1, d2, y, c), [1, 2, 3, 8, 6],
                           precision)
        # nt[t, c', a, d1, w] = t1[a, d1, s, x, c'] W2[w, t, s, x]
        wm = W2d[0]
        nt = _contract_raw(h, t1, (a, d1, d2, y, c), [1, 2, 3, 8, 6], W2, W2d, [7, 5, 3, 8],
                           (d2, c, a, d1, wm), [5, 6, 1, 2, 7], precision)
        ntd = (d2, c, a, d1, wm)
        _contract_acc(h, noise, nt, ntd, [5, 6, 1, 2, 7], nt, ntd, [9, 10, 1, 2, 7], rho, (d2, c, d2, c),
                      [5, 6, 9, 10], precision)
    D = T.empty_dev(m)
    U = T.empty_dev(m * m)
    k = C.c_int64()
    te = C.c_double()
    dc = C.c_double()
    h.call("itg_eigh_trunc", C.c_int64(m), _ptr(rho), C.c_int64(m), C.c_int64(maxdim), C.c_int64(mindim),
           C.c_double(cutoff), 0, 1, int(legacy), _ptr(D), _ptr(U), C.byref(k), C.byref(te), C.byref(dc))
    kk = int(k.value)
    Uk = U[: m * kk]
    if ha == 1:
        Ab = Uk.clone()
        Ab1 = _contract_raw(h, Uk, (a, d1, kk), [1, 2, 7], phi, shape, [1, 2, 3, 4], (kk, d2, c), [7, 3, 4],
                            precision)
    else:
        Ab1 = _permute_raw(h, Uk, (d2, c, kk), [1, 2, 3], [3, 1, 2])
        Ab = _contract_raw(h, phi, shape, [1, 2, 3, 4], Uk, (d2, c, kk), [3, 4, 7], (a, d1, kk), [1, 2, 7],
                           precision)
    return Ab, Ab1, kk, te.value


def _orthogonalize_left_end(h, ch: _Chain):
    """Right-orthogonalise sites N-1..1 by QR (orthogonalize!(psi, 1)) and normalise site 0."""
    for j in range(ch.N - 1, 0, -1):
        a, d, b = ch.Ad[j]
        # M = A_j as (a) x (d b); QR of M^T = Q R  ->  A_j = R^T Q^T
        Mt = _permute_raw(h, ch.A[j], (a, d, b), [1, 2, 3], [2, 3, 1])  # (d, b, a)
        m, n = d * b, a
        r = min(m, n)
        Q = T.empty_dev(m * r)
        R = T.empty_dev(r * n)
        h.call("itg_qr", C.c_int64(m), C.c_int64(n), _ptr(Mt), C.c_int64(m), _ptr(Q), _ptr(R))
        # A_j = Q^T as (r, d, b)
        ch.A[j] = _permute_raw(h, Q, (d, b, r), [2, 3, 1], [1, 2, 3])
        ch.Ad[j] = (r, d, b)
        # A_{j-1}[a', s, r] = sum_a A_{j-1}[a', s, a] R[r, a]
        pa, pd, _ = ch.Ad[j - 1]
        ch.A[j - 1] = _contract_raw(h, ch.A[j - 1], ch.Ad[j - 1], [1, 2, 3], R, (r, n), [4, 3],
                                    (pa, pd, r), [1, 2, 4])
        ch.Ad[j - 1] = (pa, pd, r)
    nrm = C.c_double()
    h.call("itg_nrm2", C.c_int64(ch.A[0].numel()), _ptr(ch.A[0]), C.byref(nrm))
    h.call("itg_scal", C.c_int64(ch.A[0].numel()), C.c_double(1.0 / nrm.value), _ptr(ch.A[0]))


def _dmrg_complex(H: MPO, psi0: MPS, sweeps: Sweeps, krylovdim: int, maxiter: int, eigsolve_tol: float,
                  precision: int, outputlevel: int):
    """Two-site DMRG on ComplexF64 tensors, at the ITensor level of the library.

    ITensors' algorithm step by step (the projected environments as ITensors,
    the ProjMPO product as four contractions L * phi * W1 * W2 * R, the
    eigensolver davidson on that map, the bond split by replacebond! through
    the complex SVD), every operation on the device through libitg.so's complex
    entry points (itg_contract_z, itg_svd_trunc_z, itg_qr_z).  Used when the MPO
    or the MPS has complex tensors; the real path is the fused one above.
    """
    from . import mpsops
    from .solvers import davidson
    N = len(psi0)
    psi = psi0.copy()
    for j in range(N):
        if not psi[j].is_complex:
            psi[j] = T.complex_(psi[j])
    W = [H[j] if H[j].is_complex else T.complex_(H[j]) for j in range(N)]
    mpsops.orthogonalize_(psi, 0)
    prec = int(precision)

    def ctr(a, b):
        return T.contract(a, b, precision=prec)

    def edge(ket_link, w_link):
        t = T.cuITensor(np.ones((1, 1, 1), dtype=np.complex128), ket_link, w_link, ket_link.prime())
        return t

    Lenv = [None] * (N + 1)
    Renv = [None] * (N + 1)
    Lenv[0] = edge(psi[0].inds[0], W[0].inds[0])
    Renv[N] = edge(psi[N - 1].inds[2], W[N - 1].inds[3])

    def ext_right(R, A, Wj):   # R_{j} from R_{j+1}: sites j..N-1
        return ctr(ctr(ctr(R, A), Wj), T.dag(T.prime(A)))

    def ext_left(L, A, Wj):
        return ctr(ctr(ctr(L, A), Wj), T.dag(T.prime(A)))

    for j in range(N - 1, 1, -1):
        Renv[j] = ext_right(Renv[j + 1], psi[j], W[j])
    energy = 0.0
    records = []
    for sw in range(sweeps.nsweep):
        t0 = time.perf_counter()
        maxdim, mindim, cutoff = sweeps.maxdim(sw), sweeps.mindim(sw), sweeps.cutoff(sw)
        maxerr = 0.0
        nmv = 0
        for b, ha in sweepnext(N):
            phi = ctr(psi[b], psi[b + 1])
            L, R, W1, W2 = Lenv[b], Renv[b + 2], W[b], W[b + 1]

            def heff(x):
                nonlocal nmv
                nmv += 1
                y = ctr(ctr(ctr(ctr(L, x), W1), W2), R)
                y = y.replaceinds(y.inds, [i.noprime() if i.plev > 0 else i for i in y.inds])
                return T.permute(y, *x.inds)

            energy, phi = davidson(heff, phi, maxiter=max(1, krylovdim * maxiter), tol=eigsolve_tol,
                                   restart_dim=max(2, krylovdim + 1))
            energy = float(np.real(energy))
            spec = mpsops.replacebond_(psi, b, phi, ortho="left" if ha == 1 else "right", maxdim=maxdim,
                                       mindim=mindim, cutoff=cutoff)
            maxerr = max(maxerr, float(spec.truncerr))
            if ha == 1:
                Lenv[b + 1] = ext_left(L, psi[b], W1)
            else:
                Renv[b + 1] = ext_right(R, psi[b + 1], W2)
        T._h().call("itg_synchronize")
        rec = SweepRecord(energy, psi.maxlinkdim(), maxerr, time.perf_counter() - t0, nmv)
        records.append(rec)
        if outputlevel > 0:
            print(f"After sweep {sw + 1} energy={energy:.14f} maxlinkdim={rec.maxlinkdim} "
                  f"maxerr={rec.maxtruncerr:.2e} time={rec.seconds:.3f}", flush=True)
    return energy, psi, records


def dmrg(H: MPO, psi0: MPS, sweeps: Sweeps, *, krylovdim: int = 3, maxiter: int = 2,
         eigsolve_tol: float = 1e-14, precision: str | int = "fp64", legacy_gpu_truncate: bool = False,
         svd_method: int = 0, preconditioner=None, bond_hook=None, phase_timing: bool = False,
         outputlevel: int = 0, return_result: bool = False):
    """Ground state by two-site DMRG.  Returns (energy, psi) like ITensors' dmrg.

    krylovdim / maxiter: Davidson subspace size before a restart and number of
    restarts per bond.  precision "split" runs the chi^3 contractions of the
    eigensolver and the matrix products of the large-matrix SVD on the tensor
    cores (FP64 operands split into exact bf16 digit products).  svd_method:
    0 auto (Jacobi up to 192 columns, mixed FP32-Jacobi + refinement above),
    1 FP64 Jacobi, 2 mixed.

    preconditioner: None (the diagonal one) or an itg.learned.LearnedPreconditioner
    (itg_davidson_heff2_learned; falls back to the diagonal one when it stalls).
    bond_hook(ctx): called before every eigensolve with a dict of the bond's
    device tensors and dimensions (used to collect training data).

    A sweep with noise(sweeps, sw) > 0 splits each bond through the perturbed
    density matrix (ITensors' noise term) and itg_eigh_trunc instead of the SVD.
    """
    if isinstance(precision, str):
        precision = {"fp64": PREC_FP64, "split": PREC_SPLIT}[precision.lower()]
    h = T._h()
    N = len(psi0)
    if len(H) != N:
        raise T.DimensionMismatch(2, "dmrg: MPO and MPS lengths differ")
    if N < 2:
        raise ValueError("dmrg needs at least two sites")
    psi0 = T.cu(psi0)
    H = T.cu(H)
    if any(t.is_complex for t in list(psi0.tensors) + list(H.tensors)):
        if preconditioner is not None or bond_hook is not None or any(sweeps.noise(s) > 0 for s in range(sweeps.nsweep)):
            raise ValueError("dmrg on complex tensors: no learned preconditioner, bond hook or noise term")
        energy, psi, records = _dmrg_complex(H, psi0, sweeps, krylovdim, maxiter, eigsolve_tol, precision,
                                             outputlevel)
        if return_result:
            return DMRGResult(energy, psi, records)
        return energy, psi
    ch = _Chain(psi0.copy(), H)
    _orthogonalize_left_end(h, ch)
    one = T.empty_dev(1).fill_(1.0)
    Lenv = [None] * (N + 1)
    Renv = [None] * (N + 1)
    Lenv[0] = (one, (1, 1, 1))
    Renv[N] = (one, (1, 1, 1))
    for j in range(N - 1, 1, -1):
        Renv[j] = _env_right(h, Renv[j + 1][0], Renv[j + 1][1], ch.A[j], ch.Ad[j], ch.W[j], ch.Wd[j],
                             precision)
    energy = 0.0
    records = []
    schmidt = [None] * (N + 1)  # latest singular values on link j (between sites j-1 and j)
    fallbacks_total = 0
    for sw in range(sweeps.nsweep):
        t0 = time.perf_counter()
        maxdim, mindim, cutoff = sweeps.maxdim(sw), sweeps.mindim(sw), sweeps.cutoff(sw)
        maxerr = 0.0
        nmv_tot = 0
        svd_sw = 0
        fb0 = C.c_int64()
        h.call("itg_svd_info", None, None, C.byref(fb0))
        ph = dict(eig=0.0, svd=0.0, env=0.0)

        def tick(key, t):
            if phase_timing:
                h.call("itg_synchronize")
                now = time.perf_counter()
                ph[key] += now - t
                return now
            return t

        for b, ha in sweepnext(N):
            tp = tick("env", time.perf_counter()) if phase_timing else 0.0
            a, d1, _ = ch.Ad[b]
            _, d2, c = ch.Ad[b + 1]
            k_old = ch.Ad[b][2]
            # phi = A_b * A_{b+1}: (a, d1, d2, c)
            phi = _contract_raw(h, ch.A[b], (a, d1, k_old), [1, 2, 3], ch.A[b + 1], (k_old, d2, c),
                                [3, 4, 5], (a, d1, d2, c), [1, 2, 4, 5])
            Lt, Ld = Lenv[b]
            Rt, Rd = Renv[b + 2]
            W1, W1d = ch.W[b], ch.Wd[b]
            W2, W2d = ch.W[b + 1], ch.Wd[b + 1]
            lamL = schmidt[b] if (schmidt[b] is not None and len(schmidt[b]) == a) else None
            lamR = schmidt[b + 2] if (schmidt[b + 2] is not None and len(schmidt[b + 2]) == c) else None
            if bond_hook is not None:
                bond_hook(dict(b=b, half=ha, sweep=sw, chiL=a, chiR=c, d=d1, wL=W1d[0], wM=W1d[3], wR=W2d[3],
                               L=Lt, W1=W1, W2=W2, R=Rt, phi=phi, lamL=lamL, lamR=lamR))
            e = C.c_double()
            nmv = C.c_int()
            if preconditioner is None:
                h.call("itg_davidson_heff2", C.c_int64(a), C.c_int64(c), C.c_int64(d1), C.c_int64(W1d[0]),
                       C.c_int64(W1d[3]), C.c_int64(W2d[3]), _ptr(Lt), _ptr(W1), _ptr(W2), _ptr(Rt),
                       _ptr(phi), int(krylovdim), int(maxiter), C.c_double(eigsolve_tol), int(precision),
                       C.byref(e), C.byref(nmv))
            else:
                fb = C.c_int()
                h.call("itg_davidson_heff2_learned", C.c_int64(a), C.c_int64(c), C.c_int64(d1),
                       C.c_int64(W1d[0]), C.c_int64(W1d[3]), C.c_int64(W2d[3]), _ptr(Lt), _ptr(W1), _ptr(W2),
                       _ptr(Rt), _ptr(phi), int(krylovdim), int(maxiter), C.c_double(eigsolve_tol),
                       int(precision), preconditioner.ptr,
                       _ptr(lamL) if lamL is not None else None, _ptr(lamR) if lamR is not None else None,
                       C.byref(e), C.byref(nmv), C.byref(fb))
                fallbacks_total += fb.value
            energy = e.value
            nmv_tot += nmv.value
            tp = tick("eig", tp)
            nz = sweeps.noise(sw)
            if nz > 0:
                Ab, Ab1, kk, te_v = _noise_split(h, phi, (a, d1, d2, c), Lt, Ld, W1, W1d, W2, W2d, Rt, Rd, ha,
                                                 nz, maxdim, mindim, cutoff, legacy_gpu_truncate, precision)
                tp = tick("svd", tp)
                maxerr = max(maxerr, te_v)
                schmidt[b + 1] = None
                ch.A[b], ch.Ad[b] = Ab, (a, d1, kk)
                ch.A[b + 1], ch.Ad[b + 1] = Ab1, (kk, d2, c)
                if ha == 1:
                    Lenv[b + 1] = _env_left(h, Lt, Ld, ch.A[b], ch.Ad[b], W1, W1d, precision)
                else:
                    Renv[b + 1] = _env_right(h, Rt, Rd, ch.A[b + 1], ch.Ad[b + 1], W2, W2d, precision)
                tick("env", tp)
                continue
            # bond split of phi as (a d1) x (d2 c): one orthonormal factor
            # (left-moving half: A_b; right-moving: A_{b+1}), the other one
            # carries S (itg_factorize_trunc)
            m, n = a * d1, d2 * c
            r = min(m, n)
            Lb = T.empty_dev(max(m, n) * r)
            S = T.empty_dev(r)
            Cb = T.empty_dev(max(m, n) * r)
            k = C.c_int64()
            te = C.c_double()
            dc = C.c_double()
            try:
                h.call("itg_factorize_trunc", C.c_int64(m), C.c_int64(n), _ptr(phi), C.c_int64(m),
                       C.c_int64(maxdim), C.c_int64(mindim), C.c_double(cutoff), 0, 1,
                       int(legacy_gpu_truncate), 0 if ha == 1 else 1, int(svd_method), int(precision),
                       _ptr(Lb), _ptr(S), _ptr(Cb), C.byref(k), C.byref(te), C.byref(dc))
            except NotConverged:
                pass  # factors are still returned; the rotation limit is generous
            tp = tick("svd", tp)
            swc = C.c_int()
            h.call("itg_svd_info", C.byref(swc), None, None)
            svd_sw += swc.value
            kk = int(k.value)
            maxerr = max(maxerr, te.value)
            schmidt[b + 1] = S[:kk].clone()
            if ha == 1:
                # A_b = L[(a d1), k]; A_{b+1}[k, d2, c] = (S V^T)[k, (d2 c)]
                ch.A[b] = Lb[: m * kk].clone()
                ch.Ad[b] = (a, d1, kk)
                ch.A[b + 1] = Cb[: kk * n].clone()
                ch.Ad[b + 1] = (kk, d2, c)
                Lenv[b + 1] = _env_left(h, Lt, Ld, ch.A[b], ch.Ad[b], W1, W1d, precision)
            else:
                # A_b[a, d1, k] = (U S)[(a d1), k];  A_{b+1} = V^T, V = L[(d2 c), k]
                ch.A[b] = Cb[: m * kk].clone()
                ch.Ad[b] = (a, d1, kk)
                ch.A[b + 1] = _permute_raw(h, Lb[: n * kk], (d2, c, kk), [1, 2, 3], [3, 1, 2])
                ch.Ad[b + 1] = (kk, d2, c)
                Renv[b + 1] = _env_right(h, Rt, Rd, ch.A[b + 1], ch.Ad[b + 1], W2, W2d, precision)
            tick("env", tp)
        h.call("itg_synchronize")
        secs = time.perf_counter() - t0
        if phase_timing:
            ph["other"] = max(0.0, secs - ph["eig"] - ph["svd"] - ph["env"])
        fb1 = C.c_int64()
        h.call("itg_svd_info", None, None, C.byref(fb1))
        rec = SweepRecord(energy, max(x[2] for x in ch.Ad[:-1]), maxerr, secs, nmv_tot,
                          ph if phase_timing else {}, svd_sw, int(fb1.value - fb0.value))
        records.append(rec)
        if outputlevel > 0:
            print(f"After sweep {sw + 1} energy={energy:.14f} maxlinkdim={rec.maxlinkdim} "
                  f"maxerr={rec.maxtruncerr:.2e} time={rec.seconds:.3f}", flush=True)
    # package the result as an MPS with fresh link indices
    links = [Index(1, "Link,l=0")] + [Index(ch.Ad[j][2], f"Link,l={j + 1}") for j in range(N - 1)] + \
            [Index(1, f"Link,l={N}")]
    ts = [ITensor(Dense(ch.A[j]), (links[j], psi0.sites[j], links[j + 1])) for j in range(N)]
    psi = MPS(ts, psi0.sites, -1, 1)
    if return_result:
        res = DMRGResult(energy, psi, records)
        res.fallbacks = fallbacks_total
        return res
    return energy, psi


def inner(phi: MPS, psi: MPS) -> float:
    """<phi|psi> for real MPS with matching site indices (inner, ITensors)."""
    h = T._h()
    phi, psi = T.cu(phi), T.cu(psi)
    E = T.empty_dev(1).fill_(1.0)
    Ed = (1, 1)
    for j in range(len(psi)):
        a, d, b = phi[j].dims
        a2, d2, b2 = psi[j].dims
        # E[a, a2] -> t[a2, d, b] = sum_a E[a,a2] phi[a,d,b] -> E'[b, b2] = sum t[a2,d,b] psi[a2,d,b2]
        t = _contract_raw(h, E, Ed, [1, 2], phi[j].store.data, (a, d, b), [1, 3, 4], (a2, d, b), [2, 3, 4])
        E = _contract_raw(h, t, (a2, d, b), [2, 3, 4], psi[j].store.data, (a2, d2, b2), [2, 3, 5],
                          (b, b2), [4, 5])
        Ed = (b, b2)
    return float(E[0].item())


def expect_energy(H: MPO, psi: MPS) -> float:
    """<psi|H|psi> / <psi|psi> through left environments."""
    h = T._h()
    H, psi = T.cu(H), T.cu(psi)
    one = T.empty_dev(1).fill_(1.0)
    Lt, Ld = one, (1, 1, 1)
    for j in range(len(psi)):
        Lt, Ld = _env_left(h, Lt, Ld, psi[j].store.data.contiguous(), psi[j].dims,
                           H[j].store.data.contiguous(), H[j].dims, PREC_FP64)
    return float(Lt[0].item()) / inner(psi, psi)
