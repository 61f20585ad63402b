"""Truncation, SVD, eigen and QR on the GPU against the oracle.

* truncate: the reference golden vectors (test/test_cutruncate.jl:9-17) through
  itg_truncate with legacy_gpu = 1, and random spectra bit-exact against both
  oracle rules (integer keep count exact, sums identical);
* svd: A = U S V^T and orthogonality at 1e-14 (test/test_cuitensor.jl:105-112),
  singular values against LAPACK at 1e-13 relative to sigma_max;
* qr: reconstruction and orthogonality at 1e-14 (test/test_cuitensor.jl:125-130);
* eigen: descending eigenvalues against LAPACK, truncation.
"""
import ctypes as C
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import itg_oracle as O

pytestmark = pytest.mark.gpu
GOLD = json.loads((Path(__file__).parent / "golden" / "reference_known_answers.json").read_text())


def _truncate_gpu(P, legacy, **kw):
    import torch
    from itg import _lib
    from itg.tensor import _ptr
    h = _lib.handle(0)
    Pd = torch.tensor(np.asarray(P, dtype=np.float64), device="cuda")
    n = C.c_int64()
    te = C.c_double()
    dc = C.c_double()
    h.call("itg_truncate", _ptr(Pd), C.c_int64(len(P)), C.c_int64(int(kw.get("maxdim", 0))),
           C.c_int64(int(kw.get("mindim", 1))), C.c_double(kw.get("cutoff", 0.0)),
           int(kw.get("absoluteCutoff", False)), int(kw.get("doRelCutoff", True)), int(legacy),
           C.byref(n), C.byref(te), C.byref(dc))
    return n.value, te.value, dc.value


@pytest.mark.parametrize("case", GOLD["truncate"], ids=lambda c: c["source"])
def test_truncate_reference_golden_on_gpu(gpu, case):
    kw = case["kwargs"]
    n, te, dc = _truncate_gpu(case["P"], True, cutoff=kw.get("cutoff", 0.0),
                              absoluteCutoff=kw.get("absoluteCutoff", False))
    P = np.asarray(case["P"])
    kept = [0.0] if P.max() == 0 else list(P[:n])
    assert kept == case["kept"]
    assert te == pytest.approx(case["truncerr"], rel=1.5e-8, abs=1e-300)
    assert dc == pytest.approx(case["docut"], rel=1.5e-8, abs=1e-300)


@pytest.mark.parametrize("legacy", [False, True])
def test_truncate_random_spectra_bit_exact(gpu, legacy):
    rng = np.random.default_rng(11)
    f = O.truncate_legacy_gpu if legacy else O.truncate_cpu
    for t in range(60):
        n = int(rng.integers(1, 300))
        P = np.sort(rng.exponential(size=n) * 10.0 ** rng.uniform(-12, 0, size=n))[::-1].copy()
        kw = dict(maxdim=int(rng.integers(0, n + 3)), mindim=int(rng.integers(1, 4)),
                  cutoff=float(10.0 ** rng.uniform(-14, -1)), absoluteCutoff=bool(rng.integers(0, 2)),
                  doRelCutoff=bool(rng.integers(0, 2)))
        got = _truncate_gpu(P, legacy, **kw)
        ref = f(P, **kw)
        assert got[0] == ref[0], (t, kw)
        assert got[1] == ref[1] and got[2] == ref[2], (t, kw, got, ref)


@pytest.mark.parametrize("m,n", [(7, 5), (5, 7), (64, 64), (300, 180), (180, 300), (520, 400)])
def test_svd_reconstruction_and_orthogonality(gpu, m, n):
    I = gpu.Index
    i, j = I(m), I(n)
    A = gpu.randomCuITensor(i, j, seed=m * 1000 + n)
    U, S, V, spec = gpu.svd(A, i)
    u = U.inds[-1]
    Ah = A.array()
    Uh, Sh, Vh = U.array(i, u), S.store.data.cpu().numpy(), V.array(j, V.inds[-1])
    assert np.allclose(Uh @ np.diag(Sh) @ Vh.T, Ah, rtol=0, atol=1e-13 * np.abs(Ah).max() * max(m, n))
    r = min(m, n)
    assert np.abs(Uh.T @ Uh - np.eye(r)).max() < 1e-13
    assert np.abs(Vh.T @ Vh - np.eye(r)).max() < 1e-13
    sref = np.linalg.svd(Ah, compute_uv=False)
    assert np.abs(Sh - sref).max() < 1e-13 * sref[0]
    assert np.all(np.diff(Sh) <= 0)
    # ITensor-level identity A = U * S * V
    R = U * S * V
    assert np.abs(R.array(i, j) - Ah).max() < 1e-12 * np.abs(Ah).max()


def test_svd_reference_case_isapprox(gpu):
    """test/test_cuitensor.jl:105-112: A(i,j,k,l) with dims 2,3,4,5, svd(A, (j,l));
    U U' ~ delta and V V' ~ delta at rtol 1e-14 (Julia isapprox, Frobenius norm)."""
    I = gpu.Index
    i, j, k, l = I(2), I(3), I(4), I(5)
    A = gpu.randomCuITensor(i, j, k, l, seed=77)
    U, S, V, spec = gpu.svd(A, j, l)
    R = U * S * V
    assert np.linalg.norm(R.array(i, j, k, l) - A.array()) <= 1.5e-8 * np.linalg.norm(A.array())
    for F, ind in ((U, U.inds[-1]), (V, V.inds[-1])):
        rest = [x for x in F.inds if x != ind]
        M = F.array(*rest, ind).reshape(-1, ind.dim, order="F")
        G = M.T @ M
        d = np.eye(ind.dim)
        assert np.linalg.norm(G - d) <= 1e-14 * max(np.linalg.norm(G), np.linalg.norm(d))


def test_svd_truncation_matches_oracle(gpu):
    rng = np.random.default_rng(5)
    m = n = 256
    Q1, _ = np.linalg.qr(rng.standard_normal((m, m)))
    Q2, _ = np.linalg.qr(rng.standard_normal((n, n)))
    s = np.exp(-np.arange(n) / 20.0)
    M = (Q1 * s) @ Q2.T
    I = gpu.Index
    i, j = I(m), I(n)
    A = gpu.cuITensor(M, i, j)
    for kw in (dict(cutoff=1e-10), dict(maxdim=50), dict(cutoff=1e-6, maxdim=200),
               dict(cutoff=1e-4, absoluteCutoff=True)):
        U, S, V, spec = gpu.svd(A, i, **kw)
        Uo, So, Vo, te, _ = O.svd_trunc(M, **kw)
        assert len(S.store.data) == len(So), kw
        assert np.abs(S.store.data.cpu().numpy() - So).max() < 1e-13
        assert spec.truncerr == pytest.approx(te, rel=1e-9, abs=1e-16)


@pytest.mark.parametrize("n,prec", [(300, 0), (258, 1), (512, 1), (1024, 1)])
def test_svd_mixed_haar_exp_spectrum(gpu, n, prec):
    """The Jacobi-SVD microbench matrix: A = U diag(exp(-k/20)) V^T with Haar U, V;
    mixed path (FP32 Jacobi + refinement, products at FP64 or split precision).
    n = 258 (not a multiple of 4) runs the element-wise FP32 block step, the
    other sizes the float4 one."""
    from itg import _lib
    import torch
    rng = np.random.default_rng(n)
    Q1, R1 = np.linalg.qr(rng.standard_normal((n, n)))
    Q1 *= np.sign(np.diag(R1))
    Q2, R2 = np.linalg.qr(rng.standard_normal((n, n)))
    Q2 *= np.sign(np.diag(R2))
    s = np.exp(-np.arange(n) / 20.0)
    M = (Q1 * s) @ Q2.T
    h = _lib.handle(0)
    p = lambda t: C.c_void_p(t.data_ptr())
    A = torch.from_numpy(O.flat(M).copy()).cuda()
    U = torch.empty(n * n, dtype=torch.float64, device="cuda")
    S = torch.empty(n, dtype=torch.float64, device="cuda")
    V = torch.empty_like(U)
    k, te, dc = C.c_int64(), C.c_double(), C.c_double()
    h.call("itg_svd_trunc_ex", C.c_int64(n), C.c_int64(n), p(A), C.c_int64(n), C.c_int64(0), C.c_int64(1),
           C.c_double(1e-12), 0, 1, 0, p(U), p(S), p(V), C.byref(k), C.byref(te), C.byref(dc), 2, prec)
    kk = k.value
    Uo, So, Vo, teo, _ = O.svd_trunc(M, cutoff=1e-12)
    # the mixed path's contract: P = S^2 to ~1e-13 P_max absolute (so the kept
    # count can differ by one at the cutoff); singular values and both factors
    # accurate above ~1e-4 sigma_max; with QR preconditioning (n > 192) the
    # left factor Q V_J is orthonormal for every kept column
    assert abs(kk - len(So)) <= 1
    kk = min(kk, len(So))
    Sh = S.cpu().numpy()[:kk]
    So = So[:kk]
    assert np.abs(Sh ** 2 - So ** 2).max() < 3e-13 * So[0] ** 2
    big = So > 1e-4 * So[0]
    assert np.abs(Sh[big] - So[big]).max() < 1e-12 * So[0]
    Uh = O.unflat(U.cpu().numpy()[: n * kk], (n, kk))
    Vh = O.unflat(V.cpu().numpy()[: n * kk], (n, kk))
    assert np.abs(Uh.T @ Uh - np.eye(kk)).max() < 1e-12
    Ub, Vb = Uh[:, big], Vh[:, big]
    assert np.abs(Vb.T @ Vb - np.eye(Vb.shape[1])).max() < 1e-12
    # vectors: error ~1e-13 P_max / (P gap), so the product is checked where
    # P gaps exceed ~1e-5 P_max
    top = So > 1e-2 * So[0]
    Ut, Vt = Uh[:, top], Vh[:, top]
    # (split products carry itg_split_error_bound(n) ~ 1e-11 n relative error)
    ptol = 1e-10 if prec == 0 else 1e-8
    assert np.abs((Ut * Sh[top]) @ Vt.T - (Uo[:, top] * So[top]) @ Vo[:, top].T).max() < ptol * So[0]
    # truncerr sums the discarded P values, each to ~1e-13 P_max
    assert abs(te.value - teo) < 1e-13 * (n - kk + 1) * So[0] ** 2


def test_qr(gpu):
    I = gpu.Index
    i, j, k, l = I(2), I(3), I(4), I(5)
    A = gpu.randomCuITensor(i, j, k, l, seed=21)
    Q, R = gpu.qr(A, i, l)
    q = Q.inds[-1]
    assert np.abs((Q * R).array(i, j, k, l) - A.array()).max() < 1e-13
    Qm = Q.array(i, l, q).reshape(10, -1, order="F")
    assert np.abs(Qm.T @ Qm - np.eye(Qm.shape[1])).max() < 1e-14
    # tall and wide matrices
    for (m, n) in ((200, 50), (40, 90)):
        a, b = I(m), I(n)
        M = gpu.randomCuITensor(a, b, seed=m + n)
        Q, R = gpu.qr(M, a)
        assert np.abs((Q * R).array(a, b) - M.array()).max() < 1e-12
        Qh = Q.array(a, Q.inds[-1])
        assert np.abs(Qh.T @ Qh - np.eye(Qh.shape[1])).max() < 1e-13


def test_eigen_hermitian(gpu):
    I = gpu.Index
    n = 150
    i = I(n)
    ip = i.prime()
    rng = np.random.default_rng(8)
    X = rng.standard_normal((n, n))
    M = X @ X.T / n
    A = gpu.cuITensor(M, i, ip)
    D, U, spec = gpu.eigen(A, [i], [ip])
    w = D.store.data.cpu().numpy()
    wref = np.linalg.eigvalsh(M)[::-1]
    assert np.abs(w - wref).max() < 1e-12 * wref[0]
    Uh = U.array(ip, U.inds[-1])
    assert np.abs(Uh.T @ Uh - np.eye(n)).max() < 1e-12
    assert np.abs(Uh @ np.diag(w) @ Uh.T - M).max() < 1e-12 * wref[0]
    # truncated, indefinite matrix
    S = X + X.T
    D, U, spec = gpu.eigen(gpu.cuITensor(S, i, ip), [i], [ip], maxdim=20)
    wref = np.linalg.eigvalsh(S)[::-1]
    assert np.abs(D.store.data.cpu().numpy() - wref[:20]).max() < 1e-11 * np.abs(wref).max()


@pytest.mark.parametrize("method", [1, 2])
def test_svd_qr_preconditioning_and_jacobi_modes(gpu, method):
    """The QR-preconditioned Jacobi (default) and the plain one, block-cyclic
    (default), element pairs per step, or all sweeps in one cooperative
    launch, give the same
    factorisation (singular values to 1e-13 sigma_max for the FP64 method;
    the mixed method to its P accuracy), and preconditioning cuts the sweeps
    on a graded spectrum."""
    from itg import _lib
    import torch
    n, m = 300, 340
    rng = np.random.default_rng(77)
    Q1, _ = np.linalg.qr(rng.standard_normal((m, n)))
    Q2, _ = np.linalg.qr(rng.standard_normal((n, n)))
    s = np.exp(-np.arange(n) / 20.0)
    M = (Q1 * s) @ Q2.T
    h = _lib.handle(0)
    p = lambda t: C.c_void_p(t.data_ptr())
    A = torch.from_numpy(O.flat(M).copy()).cuda()
    res = {}
    try:
        for pre, mode in ((1, 0), (0, 0), (1, 1), (1, 2)):
            h.call("itg_set_svd_options", pre, mode)
            U = torch.empty(m * n, dtype=torch.float64, device="cuda")
            S = torch.empty(n, dtype=torch.float64, device="cuda")
            V = torch.empty(n * n, dtype=torch.float64, device="cuda")
            k, te, dc = C.c_int64(), C.c_double(), C.c_double()
            h.call("itg_svd_trunc_ex", C.c_int64(m), C.c_int64(n), p(A), C.c_int64(m), C.c_int64(0), C.c_int64(1),
                   C.c_double(1e-12), 0, 1, 0, p(U), p(S), p(V), C.byref(k), C.byref(te), C.byref(dc), method, 0)
            sw = C.c_int()
            h.call("itg_svd_info", C.byref(sw), None, None)
            kk = k.value
            res[(pre, mode)] = (kk, S.cpu().numpy()[:kk], O.unflat(U.cpu().numpy()[: m * kk], (m, kk)),
                                O.unflat(V.cpu().numpy()[: n * kk], (n, kk)), sw.value)
    finally:
        h.call("itg_set_svd_options", 1, 0)
    kk0 = res[(1, 0)][0]
    for key, (kk, Sh, Uh, Vh, sw) in res.items():
        if method == 1:
            assert kk == kk0, key
        else:
            assert abs(kk - kk0) <= 1, key
        kk = min(kk, kk0)
        Sh, Uh, Vh = Sh[:kk], Uh[:, :kk], Vh[:, :kk]
        big = s[:kk] > 1e-4
        tol = 3e-13 if method == 1 else 1e-12
        assert np.abs(Sh[big] - s[:kk][big]).max() < tol, key
        if method == 1 or key[0] == 1:
            # FP64 Jacobi: both factors; mixed with preconditioning: U = Q V_J
            assert np.abs(Uh.T @ Uh - np.eye(kk)).max() < 1e-12, key
        else:
            # mixed without preconditioning: V is the refined eigenvector set
            assert np.abs(Vh.T @ Vh - np.eye(kk)).max() < 1e-12, key
        if method == 1:
            assert np.abs(Vh.T @ Vh - np.eye(kk)).max() < 1e-12, key
            assert np.abs((Uh * Sh) @ Vh.T - M).max() < 2e-6, key
        else:
            Ub, Vb = Uh[:, big], Vh[:, big]
            assert np.abs(Ub.T @ Ub - np.eye(Ub.shape[1])).max() < 1e-12, key
            assert np.abs(Vb.T @ Vb - np.eye(Vb.shape[1])).max() < 1e-12, key
    # fewer sweeps with the preconditioner
    assert res[(1, 0)][4] < res[(0, 0)][4], (res[(1, 0)][4], res[(0, 0)][4])


@pytest.mark.parametrize("m,n", [(300, 300), (400, 260), (260, 400), (90, 70)])
@pytest.mark.parametrize("method,prec", [(1, 0), (2, 0), (2, 1)])
@pytest.mark.parametrize("ortho", [0, 1])
def test_factorize_trunc(gpu, m, n, method, prec, ortho):
    """itg_factorize_trunc: the orthonormal factor is orthonormal to 1e-13 for
    every kept column (also for singular values far below sqrt(eps) sigma_max),
    the product reproduces the oracle's truncated SVD, and k / S / truncerr
    follow the ITensors truncation of the oracle's spectrum.  With split
    products (prec 1) the Newton-Schulz steps measure X^T X through 48-bit
    operand digits, so the orthonormality holds to 2e-13 there."""
    from itg import _lib
    import torch
    rng = np.random.default_rng(m * 7 + n + method + 10 * prec + 100 * ortho)
    r = min(m, n)
    Q1, _ = np.linalg.qr(rng.standard_normal((m, r)))
    Q2, _ = np.linalg.qr(rng.standard_normal((n, r)))
    s = np.exp(-np.arange(r) / 12.0)  # down to ~1e-11 at r = 300
    M = (Q1 * s) @ Q2.T
    h = _lib.handle(0)
    p = lambda t: C.c_void_p(t.data_ptr())
    A = torch.from_numpy(O.flat(M).copy()).cuda()
    big = max(m, n) * r
    L = torch.empty(big, dtype=torch.float64, device="cuda")
    S = torch.empty(r, dtype=torch.float64, device="cuda")
    Cm = torch.empty(big, dtype=torch.float64, device="cuda")
    k, te, dc = C.c_int64(), C.c_double(), C.c_double()
    # FP64 Jacobi: keep sigma down to ~1e-9 sigma_max; mixed: down to ~1e-6
    # (its singular vectors are resolved above ~1e-7 sigma_max)
    cutoff = 1e-18 if method == 1 else 1e-12
    h.call("itg_factorize_trunc", C.c_int64(m), C.c_int64(n), p(A), C.c_int64(m), C.c_int64(0), C.c_int64(1),
           C.c_double(cutoff), 0, 1, 0, ortho, method, prec, p(L), p(S), p(Cm), C.byref(k), C.byref(te),
           C.byref(dc))
    kk = k.value
    Uo, So, Vo, teo, _ = O.svd_trunc(M, cutoff=cutoff)
    Uf, Sf, Vft = np.linalg.svd(M, full_matrices=False)
    if method == 1:
        # FP64 Jacobi: P to ~n eps P_max, so the kept set is the oracle's
        assert kk == len(So)
        p_tol = 2e-13
    else:
        # mixed: P to ~1e-13 P_max absolute; a value that close to the cutoff
        # may land on the other side
        assert abs(kk - len(So)) <= 1
        p_tol = 3e-13
    kc = min(kk, len(So))
    Sh = S.cpu().numpy()[:kk]
    assert np.abs(Sh[:kc] ** 2 - So[:kc] ** 2).max() < p_tol * So[0] ** 2
    if ortho == 0:
        Lh = O.unflat(L.cpu().numpy()[: m * kk], (m, kk))
        Ch = O.unflat(Cm.cpu().numpy()[: kk * n], (kk, n))
        prod = Lh @ Ch
    else:
        Lh = O.unflat(L.cpu().numpy()[: n * kk], (n, kk))
        Ch = O.unflat(Cm.cpu().numpy()[: m * kk], (m, kk))
        prod = Ch @ Lh.T
    assert np.abs(Lh.T @ Lh - np.eye(kk)).max() < (1e-13 if prec == 0 else 2e-13)
    ref = (Uf[:, :kk] * Sf[:kk]) @ Vft[:kk]
    if method == 1:
        assert np.abs(prod - ref).max() < 1e-12 * So[0]
        assert abs(te.value - teo) < 1e-13 * So[0] ** 2
    else:
        # singular vectors below ~1e-4 sigma_max are resolved only to
        # ~1e-13 P_max / (gap in P): the product differs from the truncated SVD
        # by a small multiple of the smallest kept singular value
        assert np.abs(prod - ref).max() < 10 * Sf[kk - 1]
        assert abs(te.value - float(np.sum(Sf[kk:] ** 2))) < 1e-13 * (r - kk + 1) * So[0] ** 2


@pytest.mark.parametrize("pre", [1, 0])
@pytest.mark.parametrize("shape", [(40, 30), (6, 20), (50, 300)])
def test_jacobi_rank_deficient_converges(gpu, pre, shape):
    """Exactly rank-deficient inputs (the bond matrices of a direct sum of two
    MPS or MPO): the FP64 Jacobi must settle (noise-level columns are not
    rotated) and the rotation factor must stay orthonormal."""
    from itg import _lib
    import torch
    h = _lib.handle(0)
    m, n = shape
    rng = np.random.default_rng(m * n + pre)
    X = rng.standard_normal((m, 3)) @ rng.standard_normal((3, n))          # rank 3
    X[:, : n // 2] = np.round(X[:, : n // 2])                              # integer block, still low rank
    X = np.concatenate([X[:, : n // 2], X[:, : n - n // 2]], axis=1)       # duplicated columns
    p = lambda t: C.c_void_p(t.data_ptr())
    A = torch.from_numpy(np.asfortranarray(X).ravel(order="F").copy()).cuda()
    r = min(m, n)
    L = torch.empty(max(m, n) * r, dtype=torch.float64, device="cuda")
    S = torch.empty(r, dtype=torch.float64, device="cuda")
    Cm = torch.empty(max(m, n) * r, dtype=torch.float64, device="cuda")
    k = C.c_int64()
    h.call("itg_set_svd_options", pre, 0)
    try:
        for ortho in (0, 1):
            h.call("itg_factorize_trunc", C.c_int64(m), C.c_int64(n), p(A), C.c_int64(m), C.c_int64(r), C.c_int64(1),
                   C.c_double(0.0), 0, 1, 0, ortho, 1, 0, p(L), p(S), p(Cm), C.byref(k), None, None)
            kk = k.value
            if ortho == 0:
                Lh = L[: m * kk].cpu().numpy().reshape(kk, m).T
                Ch = Cm[: kk * n].cpu().numpy().reshape(n, kk).T
                rec = Lh @ Ch
            else:
                Lh = L[: n * kk].cpu().numpy().reshape(kk, n).T
                Ch = Cm[: m * kk].cpu().numpy().reshape(kk, m).T
                rec = Ch @ Lh.T
            assert np.abs(Lh.T @ Lh - np.eye(kk)).max() < 1e-13
            assert np.abs(rec - X).max() < 1e-12 * np.abs(X).max()
    finally:
        h.call("itg_set_svd_options", 1, 0)


def test_svd_phase_profiler_covers_the_factorisation(gpu):
    """The event profiler's SVD phases (ITG_KERNEL_SVD_QR / _JACOBI / _REFINE =
    4 / 5 / 6) each record time for a mixed bond split large enough for the
    QR-preconditioned blocked path, their sum stays within the call's wall time,
    and recording them does not change the factors."""
    import time
    from itg import _lib
    import torch
    n = 512
    rng = np.random.default_rng(11)
    Q1, _ = np.linalg.qr(rng.standard_normal((n, n)))
    Q2, _ = np.linalg.qr(rng.standard_normal((n, n)))
    M = (Q1 * np.exp(-np.arange(n) / 40.0)) @ Q2.T
    h = _lib.handle(0)
    p = lambda t: C.c_void_p(t.data_ptr())
    A = torch.from_numpy(O.flat(M).copy()).cuda()

    def split():
        L = torch.empty(n * n, dtype=torch.float64, device="cuda")
        S = torch.empty(n, dtype=torch.float64, device="cuda")
        Cm = torch.empty(n * n, dtype=torch.float64, device="cuda")
        k = C.c_int64()
        h.call("itg_factorize_trunc", C.c_int64(n), C.c_int64(n), p(A), C.c_int64(n), C.c_int64(n // 2),
               C.c_int64(1), C.c_double(0.0), 0, 1, 0, 0, 2, 1, p(L), p(S), p(Cm), C.byref(k), None, None)
        return L[: n * k.value].clone(), S[: k.value].clone()

    L0, S0 = split()
    torch.cuda.synchronize()
    h.call("itg_profile", 1)
    t0 = time.perf_counter()
    L1, S1 = split()
    torch.cuda.synchronize()
    wall_ms = (time.perf_counter() - t0) * 1e3
    phases = []
    for kind in (4, 5, 6):
        ms, nl = C.c_double(), C.c_int64()
        h.call("itg_profile_read", kind, C.byref(ms), C.byref(nl))
        assert nl.value >= 1 and ms.value > 0.0, kind
        phases.append(ms.value)
    h.call("itg_profile", 0)
    assert sum(phases) <= wall_ms * 1.05 + 0.5, (phases, wall_ms)
    assert torch.equal(L0, L1) and torch.equal(S0, S1)
