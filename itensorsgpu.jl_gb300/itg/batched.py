"""Many independent DMRG instances advanced in lockstep (one launch per step for all).

All instances are chains of the same length and MPO bond structure (e.g. an
ensemble of disordered XXZ chains with different couplings) but each has its
own bond dimensions and maxdim.  Every bond update runs for all instances at
once: phi formation and environment updates as grouped contractions
(itg_contract_grouped), the eigensolver as itg_davidson_heff2_batched (H_eff
chain as grouped launches, segmented vector kernels), and the factorisation as
itg_svd_trunc_batched (one CTA per instance).  Results equal looping
itg.dmrg over the instances (same algorithm; the SVD is always FP64 Jacobi here).
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np

from . import tensor as T
from ._lib import i32arr, i64arr
from .dmrg import _Chain, _diag_raw, _orthogonalize_left_end, _permute_raw, sweepnext
from .mps import MPO, MPS


def _ptrs(ts):
    return (C.c_void_p * len(ts))(*[C.c_void_p(t.data_ptr()) for t in ts])


def _grouped(h, A, dA, mA, B, dB, mB, dC, mC):
    """C_i = A_i * B_i for all i (same modes, per-instance dims); returns the C_i."""
    outs = [T.empty_dev(int(np.prod(d))) for d in dC]
    flat = lambda ds: [int(x) for d in ds for x in d]
    h.call("itg_contract_grouped", len(A), C.c_double(1.0), _ptrs(A), len(mA), i64arr(flat(dA)), i32arr(mA),
           _ptrs(B), len(mB), i64arr(flat(dB)), i32arr(mB), C.c_double(0.0), _ptrs(outs), len(mC),
           i64arr(flat(dC)), i32arr(mC))
    return outs


def _env_left_g(h, Ls, Lds, As, Ads, Ws, Wds):
    dims = [(a, d, b, wd[0], wd[3]) for (a, d, b), wd in zip(Ads, Wds)]
    t1 = _grouped(h, Ls, Lds, [1, 2, 3], As, Ads, [1, 4, 5], [(w, a, d, b) for a, d, b, w, x in dims], [2, 3, 4, 5])
    t2 = _grouped(h, t1, [(w, a, d, b) for a, d, b, w, x in dims], [2, 3, 4, 5], Ws, Wds, [2, 6, 4, 7],
                  [(a, b, d, x) for a, d, b, w, x in dims], [3, 5, 6, 7])
    Ln = _grouped(h, t2, [(a, b, d, x) for a, d, b, w, x in dims], [3, 5, 6, 7], As, Ads, [3, 6, 8],
                  [(b, x, b) for a, d, b, w, x in dims], [5, 7, 8])
    return Ln, [(b, x, b) for a, d, b, w, x in dims]


def _env_right_g(h, Rs, Rds, As, Ads, Ws, Wds):
    dims = [(a, d, b, wd[0], wd[3]) for (a, d, b), wd in zip(Ads, Wds)]
    t1 = _grouped(h, As, Ads, [1, 2, 3], Rs, Rds, [3, 4, 5], [(a, d, x, b) for a, d, b, w, x in dims], [1, 2, 4, 5])
    t2 = _grouped(h, t1, [(a, d, x, b) for a, d, b, w, x in dims], [1, 2, 4, 5], Ws, Wds, [6, 7, 2, 4],
                  [(a, b, w, d) for a, d, b, w, x in dims], [1, 5, 6, 7])
    Rn = _grouped(h, t2, [(a, b, w, d) for a, d, b, w, x in dims], [1, 5, 6, 7], As, Ads, [8, 7, 5],
                  [(a, w, a) for a, d, b, w, x in dims], [1, 6, 8])
    return Rn, [(a, w, a) for a, d, b, w, x in dims]


def dmrg_batched(Hs, psis, nsweep: int, maxdims, cutoff: float, *, mindim: int = 1, krylovdim: int = 3,
                 maxiter: int = 2, eigsolve_tol: float = 1e-14):
    """Two-site DMRG for many instances in lockstep.

    maxdims: per instance, an int or a per-sweep list (last value repeats).
    Returns (energies, psis, seconds_per_sweep).
    """
    h = T._h()
    cnt = len(Hs)
    if cnt != len(psis) or cnt == 0:
        raise ValueError("dmrg_batched: need matching, non-empty lists of MPOs and MPSs")
    N = len(psis[0])
    if any(len(p) != N for p in psis) or any(len(x) != N for x in Hs):
        raise T.DimensionMismatch(2, "dmrg_batched: all chains must have the same length")
    md = [m if isinstance(m, (list, tuple)) else [m] for m in maxdims]
    at = lambda v, s: v[min(s, len(v) - 1)]
    chains = []
    for H, psi in zip(Hs, psis):
        ch = _Chain(T.cu(psi).copy(), T.cu(H))
        _orthogonalize_left_end(h, ch)
        chains.append(ch)
    one = T.empty_dev(1).fill_(1.0)
    Lenv = [[None] * (N + 1) for _ in range(cnt)]
    Renv = [[None] * (N + 1) for _ in range(cnt)]
    for i in range(cnt):
        Lenv[i][0] = (one, (1, 1, 1))
        Renv[i][N] = (one, (1, 1, 1))
    for j in range(N - 1, 1, -1):
        Rn, Rd = _env_right_g(h, [Renv[i][j + 1][0] for i in range(cnt)], [Renv[i][j + 1][1] for i in range(cnt)],
                              [c.A[j] for c in chains], [c.Ad[j] for c in chains],
                              [c.W[j] for c in chains], [c.Wd[j] for c in chains])
        for i in range(cnt):
            Renv[i][j] = (Rn[i], Rd[i])
    energies = np.zeros(cnt)
    secs = []
    for sw in range(nsweep):
        t0 = time.perf_counter()
        for b, ha in sweepnext(N):
            Ab = [c.A[b] for c in chains]
            Abd = [c.Ad[b] for c in chains]
            A1 = [c.A[b + 1] for c in chains]
            A1d = [c.Ad[b + 1] for c in chains]
            phis = _grouped(h, Ab, Abd, [1, 2, 3], A1, A1d, [3, 4, 5],
                            [(x[0], x[1], y[1], y[2]) for x, y in zip(Abd, A1d)], [1, 2, 4, 5])
            chiL = [x[0] for x in Abd]
            chiR = [y[2] for y in A1d]
            d = Abd[0][1]
            W1d, W2d = chains[0].Wd[b], chains[0].Wd[b + 1]
            e = (C.c_double * cnt)()
            nmv = (C.c_int * cnt)()
            h.call("itg_davidson_heff2_batched", cnt, i64arr(chiL), i64arr(chiR), C.c_int64(d),
                   C.c_int64(W1d[0]), C.c_int64(W1d[3]), C.c_int64(W2d[3]),
                   _ptrs([Lenv[i][b][0] for i in range(cnt)]), _ptrs([c.W[b] for c in chains]),
                   _ptrs([c.W[b + 1] for c in chains]), _ptrs([Renv[i][b + 2][0] for i in range(cnt)]),
                   _ptrs(phis), int(krylovdim), int(maxiter), C.c_double(eigsolve_tol), e, nmv)
            energies[:] = np.frombuffer(e, dtype=np.float64)
            ms = [chiL[i] * d for i in range(cnt)]
            ns = [d * chiR[i] for i in range(cnt)]
            rs = [min(a, bb) for a, bb in zip(ms, ns)]
            Us = [T.empty_dev(m * r) for m, r in zip(ms, rs)]
            Ss = [T.empty_dev(r) for r in rs]
            Vs = [T.empty_dev(n * r) for n, r in zip(ns, rs)]
            ks = (C.c_int64 * cnt)()
            tes = (C.c_double * cnt)()
            h.call("itg_svd_trunc_batched", cnt, i64arr(ms), i64arr(ns), _ptrs(phis),
                   i64arr([at(md[i], sw) for i in range(cnt)]), C.c_int64(mindim), C.c_double(cutoff), 0, 1, 0,
                   _ptrs(Us), _ptrs(Ss), _ptrs(Vs), ks, tes)
            for i, c in enumerate(chains):
                kk = int(ks[i])
                a, d1, d2, cc = chiL[i], d, d, chiR[i]
                Uk, Vk, Sk = Us[i][: ms[i] * kk], Vs[i][: ns[i] * kk], Ss[i][:kk]
                if ha == 1:
                    c.A[b] = Uk.clone()
                    c.Ad[b] = (a, d1, kk)
                    c.A[b + 1] = _diag_raw(h, Sk, (kk, kk), [1, 2], Vk, (d2, cc, kk), [3, 4, 1], (kk, d2, cc),
                                           [2, 3, 4])
                    c.Ad[b + 1] = (kk, d2, cc)
                else:
                    c.A[b] = _diag_raw(h, Sk, (kk, kk), [1, 2], Uk, (a, d1, kk), [3, 4, 1], (a, d1, kk),
                                       [3, 4, 2])
                    c.Ad[b] = (a, d1, kk)
                    c.A[b + 1] = _permute_raw(h, Vk, (d2, cc, kk), [1, 2, 3], [3, 1, 2])
                    c.Ad[b + 1] = (kk, d2, cc)
            if ha == 1:
                Ln, Ld = _env_left_g(h, [Lenv[i][b][0] for i in range(cnt)], [Lenv[i][b][1] for i in range(cnt)],
                                     [c.A[b] for c in chains], [c.Ad[b] for c in chains],
                                     [c.W[b] for c in chains], [c.Wd[b] for c in chains])
                for i in range(cnt):
                    Lenv[i][b + 1] = (Ln[i], Ld[i])
            else:
                Rn, Rd = _env_right_g(h, [Renv[i][b + 2][0] for i in range(cnt)],
                                      [Renv[i][b + 2][1] for i in range(cnt)],
                                      [c.A[b + 1] for c in chains], [c.Ad[b + 1] for c in chains],
                                      [c.W[b + 1] for c in chains], [c.Wd[b + 1] for c in chains])
                for i in range(cnt):
                    Renv[i][b + 1] = (Rn[i], Rd[i])
        h.call("itg_synchronize")
        secs.append(time.perf_counter() - t0)
    out = []
    for c, psi in zip(chains, psis):
        links = [T.Index(1, "Link,l=0")] + [T.Index(c.Ad[j][2], f"Link,l={j + 1}") for j in range(N - 1)] + \
                [T.Index(1, f"Link,l={N}")]
        ts = [T.ITensor(T.Dense(c.A[j]), (links[j], psi.sites[j], links[j + 1])) for j in range(N)]
        out.append(MPS(ts, psi.sites, 0, 1))
    return energies.copy(), out, secs
