"""ComplexF64 storage (ITG_C64) against NumPy complex128, following the
reference's complex test loops (test/test_cucontract.jl:9,
test/test_cudense.jl:9, test/test_cuitensor.jl:10, test/test_cudiag.jl:9,54).

Contraction is checked through itg_contract (complex x complex with real
scalars), itg_contract_z (mixed operands, complex scalars, split precision)
and the ITensor mirror; permutation and sums are exact.
"""
import ctypes as C
import itertools

import numpy as np
import pytest

from oracle import itg_oracle as O

pytestmark = pytest.mark.gpu


def crand(rng, shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


def rel(a, b):
    return np.linalg.norm(np.ravel(a - b)) / max(np.linalg.norm(np.ravel(b)), 1e-300)


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a).ravel(order="F"))).cuda()


def _host(t, shape):
    return t.cpu().numpy().reshape(shape, order="F")


CASES = [
    # (labels A, labels B, labels C)
    ("ij", "jk", "ik"),
    ("ijk", "kjl", "li"),
    ("abcd", "dxcy", "xbya"),
    ("ij", "ij", ""),
    ("i", "j", "ij"),
]


@pytest.mark.parametrize("la,lb,lc", CASES)
@pytest.mark.parametrize("kinds", [("c", "c"), ("c", "r"), ("r", "c")])
def test_contract_z_matches_einsum(gpu, la, lb, lc, kinds):
    import torch
    from itg import _lib
    h = _lib.handle(0)
    rng = np.random.default_rng(hash((la, lb, kinds)) % 2**32)
    dims = {x: int(d) for x, d in zip("ijklabcdxy", rng.integers(2, 9, 10))}
    shpA, shpB, shpC = [tuple(dims[x] for x in l) for l in (la, lb, lc)]
    A = crand(rng, shpA) if kinds[0] == "c" else rng.standard_normal(shpA)
    B = crand(rng, shpB) if kinds[1] == "c" else rng.standard_normal(shpB)
    ref = O.contract(A, list(la), B, list(lb), list(lc))
    code = {x: k + 1 for k, x in enumerate(sorted(set(la + lb + lc)))}
    out = torch.zeros(max(int(np.prod(shpC)), 1), dtype=torch.complex128, device="cuda")
    one, zero = (C.c_double * 2)(1.0, 0.0), (C.c_double * 2)(0.0, 0.0)
    p = lambda t: C.c_void_p(t.data_ptr())
    dtA = _lib.ITG_C64 if kinds[0] == "c" else _lib.ITG_F64
    dtB = _lib.ITG_C64 if kinds[1] == "c" else _lib.ITG_F64
    Ad, Bd = _dev(A), _dev(B)
    h.call("itg_contract_z", dtA, dtB, one, p(Ad), len(la), _lib.i64arr(shpA), _lib.i32arr([code[x] for x in la]),
           p(Bd), len(lb), _lib.i64arr(shpB), _lib.i32arr([code[x] for x in lb]), zero, p(out), len(lc),
           _lib.i64arr(shpC), _lib.i32arr([code[x] for x in lc]), 0)
    got = _host(out, shpC) if lc else out.cpu().numpy()[0]
    assert rel(got, ref) < 1e-13


def test_contract_dtype_c64_scalars_and_split(gpu):
    """itg_contract with ITG_C64 (real alpha, beta accumulate), itg_contract_z
    with complex alpha / beta, and the split-precision engine on complex data."""
    import torch
    from itg import _lib
    h = _lib.handle(0)
    rng = np.random.default_rng(5)
    A, B, C0 = crand(rng, (40, 30)), crand(rng, (30, 50)), crand(rng, (40, 50))
    p = lambda t: C.c_void_p(t.data_ptr())
    Ad, Bd = _dev(A), _dev(B)
    args = lambda: (p(Ad), 2, _lib.i64arr([40, 30]), _lib.i32arr([1, 2]), p(Bd), 2, _lib.i64arr([30, 50]),
                    _lib.i32arr([2, 3]))
    Cd = _dev(C0)
    h.call("itg_contract", _lib.ITG_C64, C.c_double(2.0), *args(), C.c_double(-0.5), p(Cd), 2,
           _lib.i64arr([40, 50]), _lib.i32arr([1, 3]), 0)
    assert rel(_host(Cd, (40, 50)), 2.0 * A @ B - 0.5 * C0) < 1e-13
    al, be = 0.3 - 1.2j, 0.7 + 0.4j
    Cd = _dev(C0)
    h.call("itg_contract_z", _lib.ITG_C64, _lib.ITG_C64, (C.c_double * 2)(al.real, al.imag), *args(),
           (C.c_double * 2)(be.real, be.imag), p(Cd), 2, _lib.i64arr([40, 50]), _lib.i32arr([1, 3]), 0)
    assert rel(_host(Cd, (40, 50)), al * A @ B + be * C0) < 1e-13
    Cd = torch.zeros(40 * 50, dtype=torch.complex128, device="cuda")
    h.call("itg_contract", _lib.ITG_C64, C.c_double(1.0), *args(), C.c_double(0.0), p(Cd), 2,
           _lib.i64arr([40, 50]), _lib.i32arr([1, 3]), 1)
    assert rel(_host(Cd, (40, 50)), A @ B) < 1e-12


def test_complex_itensor_ops(gpu):
    I = gpu.Index
    i, j, k, l = I(2, "i"), I(3, "j"), I(4, "k"), I(5, "l")
    rng = np.random.default_rng(11)
    # constructors
    Z = gpu.cuITensor(complex, i, j, k)
    assert Z.is_complex and np.all(Z.array() == 0)
    O1 = gpu.cuITensor(1.0 + 0.0j, i, j, k)
    assert np.all(O1.array() == np.ones((2, 3, 4), dtype=complex))
    A = gpu.randomCuITensor(complex, i, j, k, seed=3)
    assert A.is_complex
    a = A.array()
    # permute (exact)
    P = gpu.permute(A, k, j, i)
    assert np.array_equal(P.array(), np.transpose(a, (2, 1, 0)))
    # sums, also real + complex
    B = gpu.randomCuITensor(complex, k, i, j, seed=4)
    R = gpu.randomCuITensor(j, i, k, seed=5)
    assert np.array_equal((A + B).array(), a + np.transpose(B.array(), (1, 2, 0)))
    assert np.array_equal((A - R).array(), a - np.transpose(R.array(), (1, 0, 2)))
    # scalar multiples, norm, dag
    assert rel((A * (2 - 1j)).array(), (2 - 1j) * a) < 1e-15
    x = rng.standard_normal((2, 3))
    Rx = gpu.cuITensor(x, i, j) * 1j                     # real tensor, complex scalar
    assert Rx.is_complex and np.array_equal(Rx.array(), 1j * x)
    nrm = gpu.norm(A)
    assert nrm == pytest.approx(np.linalg.norm(a), rel=1e-14)
    s = (gpu.dag(A) * A).scalar()
    assert s.imag == pytest.approx(0.0, abs=1e-13) and np.sqrt(s.real) == pytest.approx(nrm, rel=1e-14)
    assert np.array_equal(gpu.dag(A).array(), np.conj(a))
    # complex(A)
    Rr = gpu.randomCuITensor(i, j, seed=6)
    assert np.array_equal(gpu.complex(Rr).array(), Rr.array().astype(complex))
    # contraction through ITensor *, mixed
    Ck = gpu.randomCuITensor(complex, k, l, seed=7)
    assert rel((A * Ck).array(), np.einsum("ijk,kl->ijl", a, Ck.array())) < 1e-14
    Rk = gpu.randomCuITensor(l, k, seed=8)
    assert rel((A * Rk).array(), np.einsum("ijk,lk->ijl", a, Rk.array())) < 1e-14
    L, R, spec = gpu.factorize(A, i, j, ortho="left")
    assert rel((L * R).array(i, j, k), a) < 1e-13
    L, R, spec = gpu.factorize(A, i, j, ortho="right", maxdim=2)
    assert R.inds[-1].dim == 2


@pytest.mark.parametrize("split", [("j", "l"), ("i", "l"), ("i", "j", "k")])
def test_complex_svd_and_qr(gpu, split):
    """test/test_cuitensor.jl:100-130 for ComplexF64: A = U S dag(V) with
    isometric U, V; A = Q R with isometric Q."""
    I = gpu.Index
    ix = {"i": I(2, "i"), "j": I(3, "j"), "k": I(4, "k"), "l": I(5, "l")}
    i, j, k, l = ix["i"], ix["j"], ix["k"], ix["l"]
    A = gpu.randomCuITensor(complex, i, j, k, l, seed=21)
    a = A.array()
    left = [ix[x] for x in split]
    right = [x for x in (i, j, k, l) if x not in left]
    U, S, V, spec = gpu.svd(A, *left)
    u, v = U.inds[-1], V.inds[-1]
    assert rel((U * S * gpu.dag(V)).array(i, j, k, l), a) < 1e-13
    Um = U.array(*left, u).reshape(-1, u.dim, order="F")
    Vm = V.array(*right, v).reshape(-1, v.dim, order="F")
    assert np.abs(Um.conj().T @ Um - np.eye(u.dim)).max() < 1e-13
    assert np.abs(Vm.conj().T @ Vm - np.eye(v.dim)).max() < 1e-13
    sv = np.linalg.svd(a.transpose([list((i, j, k, l)).index(x) for x in left + right])
                       .reshape(Um.shape[0], -1, order="F"), compute_uv=False)
    assert np.abs(np.sort(gpu.dense(S).array().diagonal())[::-1] - sv[: u.dim]).max() < 1e-13 * sv[0]
    Q, R = gpu.qr(A, *left)
    q = Q.inds[-1]
    assert rel((Q * R).array(i, j, k, l), a) < 1e-13
    Qm = Q.array(*left, q).reshape(-1, q.dim, order="F")
    assert np.abs(Qm.conj().T @ Qm - np.eye(q.dim)).max() < 1e-13


def test_complex_permute_14_indices(gpu):
    inds = [gpu.Index(2) for _ in range(14)]
    A = gpu.randomCuITensor(complex, *inds, seed=12)
    a = A.array()
    rng = np.random.default_rng(2)
    for _ in range(5):
        perm = rng.permutation(14)
        P = gpu.permute(A, *[inds[p] for p in perm])
        assert np.array_equal(P.array(), np.transpose(a, perm))


@pytest.mark.parametrize("t1,t2", list(itertools.product([float, complex], repeat=2)))
def test_diag_contractions_mixed_types(gpu, t1, t2):
    """test/test_cudiag.jl:54-103: Matrix*Diag, Diag*Diag, UniformDiag*Diag and
    UniformDiag*Matrix for every combination of real and complex element types."""
    I = gpu.Index
    i, j = I(2, "i"), I(3, "j")
    rng = np.random.default_rng(31)
    Aij = gpu.randomCuITensor(t1, i, j, seed=40)
    Dv = rng.random(2) + (1j * rng.random(2) if t2 is complex else 0)
    Ev = rng.random(2) + (1j * rng.random(2) if t2 is complex else 0)
    D = gpu.diagITensor(Dv, i, i.prime())
    E = gpu.diagITensor(Ev, i, i.prime(2))
    a = Aij.array()
    # Matrix * Diag -> Matrix (indices j, i')
    C1 = Aij * D
    assert rel(C1.array(j, i.prime()), a.T @ np.diag(Dv)) < 1e-14
    # Diag * Diag -> Diag
    C2 = E * D
    assert rel(gpu.dense(C2).array(i.prime(2), i.prime()), np.diag(Ev) @ np.diag(Dv)) < 1e-14
    # UniformDiag * Diag
    two = gpu.diagITensor([2.0 + (0j if t2 is complex else 0)], i, i.prime(2), uniform=True)
    C3 = two * D
    assert rel(gpu.dense(C3).array(i.prime(2), i.prime()), 2.0 * np.diag(Dv)) < 1e-14
    # UniformDiag * Matrix
    C4 = gpu.diagITensor([2.0 + (0j if t2 is complex else 0)], i, i.prime(), uniform=True) * Aij
    assert rel(C4.array(i.prime(), j), 2.0 * a) < 1e-14


@pytest.mark.parametrize("cplx_start", [False, True])
def test_davidson_itensor_map(gpu, cplx_start):
    """test/test_cuiterativesolvers.jl: davidson on the Hermitian map
    v -> noprime(A * v) with A = B * dag(B) (complex), from a real or complex
    start; plus a real symmetric map."""
    i = gpu.Index(10, "i")
    rng = np.random.default_rng(3)
    B = crand(rng, (10, 10))
    Hm = B @ B.conj().T
    A = gpu.cuITensor(Hm, i, i.prime())
    M = gpu.ITensorMap(A)
    v0 = gpu.randomCuITensor(complex, i, seed=5) if cplx_start else gpu.randomCuITensor(i, seed=5)
    lam, v = gpu.davidson(M, v0, maxiter=10)
    assert rel(M(v).array(), lam * v.array()) < 1e-10
    assert lam == pytest.approx(np.linalg.eigvalsh(Hm.T)[0], rel=1e-10)
    S = rng.standard_normal((12, 12))
    S = S + S.T
    j = gpu.Index(12, "j")
    lam, v = gpu.davidson(gpu.ITensorMap(gpu.cuITensor(S, j, j.prime())), gpu.randomCuITensor(j, seed=6), maxiter=12)
    assert lam == pytest.approx(np.linalg.eigvalsh(S)[0], rel=1e-10)
    assert not v.is_complex


def test_complex_hermitian_eigen(gpu):
    """eigen on a ComplexF64 Hermitian matrix (culinearalgebra.jl:84-85): M U = U D,
    U unitary, eigenvalues as LAPACK's; truncation keeps the largest."""
    n = 24
    rng = np.random.default_rng(9)
    B = crand(rng, (n, n))
    Hm = B + B.conj().T
    i = gpu.Index(n, "i")
    A = gpu.cuITensor(Hm, i, i.prime())
    D, U, spec = gpu.eigen(A, [i], [i.prime()])
    r = U.inds[-1]
    Um = U.array(i.prime(), r)
    d = gpu.dense(D).array().diagonal()
    assert np.abs(Um.conj().T @ Um - np.eye(n)).max() < 1e-13
    assert rel(Hm @ Um, Um * d[None, :]) < 1e-13
    assert np.abs(d - np.linalg.eigvalsh(Hm)[::-1]).max() < 1e-12 * np.abs(d).max()
    D5, U5, _ = gpu.eigen(A, [i], [i.prime()], maxdim=5)
    assert U5.inds[-1].dim == 5
    assert np.abs(gpu.dense(D5).array().diagonal() - d[:5]).max() < 1e-12 * np.abs(d).max()


def test_complex_mps_operations(gpu):
    """MPS/MPO operations on complex site tensors: gauge moves, overlaps with
    conjugated bras, MPO products, sums and truncation against dense vectors."""
    N = 6
    sites = [gpu.Index(2, "Site") for _ in range(N)]
    rng = np.random.default_rng(4)

    def cmps(seed, chi):
        links = [gpu.Index(1)] + [gpu.Index(chi, "Link") for _ in range(N - 1)] + [gpu.Index(1)]
        ts = [gpu.randomCuITensor(complex, links[j], sites[j], links[j + 1], seed=seed + j) for j in range(N)]
        return gpu.MPS(ts, sites, -1, N)

    def vec(psi):
        return O.mps_vector([t.array() for t in gpu.cpu(psi).tensors])

    phi, psi = cmps(10, 3), cmps(20, 4)
    vphi, vpsi = vec(phi), vec(psi)
    assert gpu.inner(phi, psi) == pytest.approx(np.vdot(vphi, vpsi), rel=1e-12)
    gpu.orthogonalize_(psi, 2)
    assert rel(vec(psi), vpsi) < 1e-12
    gpu.orthogonalize_(psi, 0, maxdim=4)
    assert rel(vec(psi), vpsi) < 1e-12
    K = gpu.randomCuMPO(sites, seed=40)
    Kc = gpu.MPO([t * (1 + 0.5j) for t in K.tensors], sites)
    Km = O.mpo_matrix([t.array() for t in gpu.cpu(Kc).tensors])
    assert gpu.inner(phi, Kc, psi) == pytest.approx(vphi.conj() @ Km @ vpsi, rel=1e-12)
    out = gpu.contract(Kc, psi)
    assert rel(vec(out), Km @ vpsi) < 1e-12
    s = gpu.add(phi, psi)
    assert rel(vec(s), vphi + vpsi) < 1e-12
    gpu.truncate_(s, maxdim=7)
    assert s.maxlinkdim() <= 7 and rel(vec(s), vphi + vpsi) < 1e-12
