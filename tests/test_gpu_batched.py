"""Many independent DMRG instances in lockstep (grouped contraction, batched
Jacobi SVD, batched Davidson) against looping the single-instance path.

* grouped contraction: every problem equals its own itg_contract (same tile
  code: bit-identical);
* batched SVD: singular values and truncation against LAPACK per instance;
* batched Davidson: energies equal the single-instance solver per instance;
* dmrg_batched on disordered XXZ chains with uneven maxdim: energies equal
  looping itg.dmrg (and the oracle) to 1e-9.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import itg_oracle as O

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch
    return torch.from_numpy(O.flat(a).copy()).cuda()


def test_grouped_contraction_equals_single(gpu):
    import torch
    from itg import _lib
    h = _lib.handle(0)
    rng = np.random.default_rng(0)
    probs = [(7, 5, 9), (130, 33, 70), (1, 4, 300), (64, 128, 64)]
    As = [_dev(rng.standard_normal((m, k))) for m, k, n in probs]
    Bs = [_dev(rng.standard_normal((k, n))) for m, k, n in probs]
    Cs = [torch.empty(m * n, dtype=torch.float64, device="cuda") for m, k, n in probs]
    ptrs = lambda ts: (C.c_void_p * len(ts))(*[C.c_void_p(t.data_ptr()) for t in ts])
    dA = [x for m, k, n in probs for x in (m, k)]
    dB = [x for m, k, n in probs for x in (k, n)]
    dC = [x for m, k, n in probs for x in (m, n)]
    h.call("itg_contract_grouped", len(probs), C.c_double(1.0), ptrs(As), 2, _lib.i64arr(dA), _lib.i32arr([1, 2]),
           ptrs(Bs), 2, _lib.i64arr(dB), _lib.i32arr([2, 3]), C.c_double(0.0), ptrs(Cs), 2, _lib.i64arr(dC),
           _lib.i32arr([1, 3]))
    for (m, k, n), A, B, Cg in zip(probs, As, Bs, Cs):
        Cs1 = torch.empty_like(Cg)
        h.call("itg_contract", 0, C.c_double(1.0), C.c_void_p(A.data_ptr()), 2, _lib.i64arr([m, k]),
               _lib.i32arr([1, 2]), C.c_void_p(B.data_ptr()), 2, _lib.i64arr([k, n]), _lib.i32arr([2, 3]),
               C.c_double(0.0), C.c_void_p(Cs1.data_ptr()), 2, _lib.i64arr([m, n]), _lib.i32arr([1, 3]), 0)
        assert torch.equal(Cg, Cs1)
        ref = O.unflat(A.cpu().numpy(), (m, k)) @ O.unflat(B.cpu().numpy(), (k, n))
        assert np.linalg.norm(O.unflat(Cg.cpu().numpy(), (m, n)) - ref) <= 1e-12 * np.linalg.norm(ref)


def test_batched_svd_matches_lapack(gpu):
    import torch
    from itg import _lib
    h = _lib.handle(0)
    rng = np.random.default_rng(1)
    shapes = [(12, 12), (40, 20), (20, 40), (256, 256), (130, 90)]
    Ms = [rng.standard_normal(s) for s in shapes]
    As = [_dev(M) for M in Ms]
    rs = [min(s) for s in shapes]
    Us = [torch.empty(s[0] * r, dtype=torch.float64, device="cuda") for s, r in zip(shapes, rs)]
    Ss = [torch.empty(r, dtype=torch.float64, device="cuda") for r in rs]
    Vs = [torch.empty(s[1] * r, dtype=torch.float64, device="cuda") for s, r in zip(shapes, rs)]
    ptrs = lambda ts: (C.c_void_p * len(ts))(*[C.c_void_p(t.data_ptr()) for t in ts])
    k = (C.c_int64 * len(shapes))()
    te = (C.c_double * len(shapes))()
    maxd = [0, 10, 15, 100, 0]
    h.call("itg_svd_trunc_batched", len(shapes), _lib.i64arr([s[0] for s in shapes]),
           _lib.i64arr([s[1] for s in shapes]), ptrs(As), _lib.i64arr(maxd), C.c_int64(1), C.c_double(1e-12),
           0, 1, 0, ptrs(Us), ptrs(Ss), ptrs(Vs), k, te)
    for i, (M, s) in enumerate(zip(Ms, shapes)):
        Uo, So, Vo, teo, _ = O.svd_trunc(M, maxdim=maxd[i], cutoff=1e-12)
        kk = k[i]
        assert kk == len(So)
        Sh = Ss[i].cpu().numpy()[:kk]
        assert np.abs(Sh - So).max() < 1e-13 * So[0]
        U = O.unflat(Us[i].cpu().numpy()[: s[0] * kk], (s[0], kk))
        V = O.unflat(Vs[i].cpu().numpy()[: s[1] * kk], (s[1], kk))
        assert np.abs((U * Sh) @ V.T - (Uo * So) @ Vo.T).max() < 1e-12 * So[0]
        assert te[i] == pytest.approx(teo, rel=1e-9, abs=1e-18)


def test_dmrg_batched_equals_looped_xxz(gpu):
    N, cnt = 12, 6
    rng = np.random.default_rng(2024)
    maxdims = [16, 32, 16, 24, 32, 20]
    Hs, psis, Js, Ds = [], [], [], []
    for i in range(cnt):
        sites = gpu.siteinds("S=1/2", N)
        J = rng.uniform(0.5, 1.5, N - 1)
        D = rng.uniform(0.5, 1.5, N - 1)
        Js.append(J)
        Ds.append(D)
        Hs.append(gpu.cuMPO(gpu.xxz_mpo(sites, J=J, Delta=D)))
        psis.append(gpu.randomCuMPS(sites, 8, seed=300 + i))
    E, out, secs = gpu.dmrg_batched(Hs, psis, 4, maxdims, 1e-10)
    for i in range(cnt):
        sw = gpu.Sweeps(4, maxdim=[maxdims[i]], cutoff=[1e-10])
        e1, _ = gpu.dmrg(Hs[i], psis[i], sw, svd_method=1)
        assert abs(E[i] - e1) < 1e-9, (i, E[i], e1)
        eo, _ = O.dmrg(O.heisenberg_mpo(N, J=Js[i], Delta=Ds[i]), O.random_mps([2] * N, 8, 300 + i),
                       [maxdims[i]], [1e-10], 4)
        assert abs(E[i] - eo) < 1e-9, (i, E[i], eo)
