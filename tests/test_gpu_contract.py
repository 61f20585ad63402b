"""Contraction parity (GPU vs oracle), mirroring test/test_cucontract.jl.

Tolerance: relative Frobenius error <= 1e-12 for the FP64 path (the
parity bar of this path; the reference's own tests use rtol = sqrt(eps) ~ 1.5e-8).
"""
import itertools
import random

import numpy as np
import pytest

from oracle import itg_oracle as O

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def relerr(x, y):
    nd = np.linalg.norm(np.asarray(y).ravel())
    return np.linalg.norm((np.asarray(x) - np.asarray(y)).ravel()) / (nd if nd > 0 else 1.0)


def _oracle_contract(A, B, Cinds):
    """Oracle result of ITensor A*B in the index order Cinds."""
    la = [id(i) for i in ()]  # placeholder to keep names short
    labA = [(i.id, i.plev) for i in A.inds]
    labB = [(i.id, i.plev) for i in B.inds]
    labC = [(i.id, i.plev) for i in Cinds]
    return O.contract(A.array(), labA, B.array(), labB, labC)


@pytest.fixture(scope="module")
def idx(gpu):
    I = gpu.Index
    return {n: I(d, n) for n, d in zip("ijkla", (2, 3, 4, 5, 6))}


def test_scalar_and_vector_cases(gpu, idx):
    i, j = idx["i"], idx["j"]
    s = gpu.cuITensor(np.array(3.0).reshape(()))
    Ai = gpu.randomCuITensor(i, seed=1)
    Aj = gpu.randomCuITensor(j, seed=2)
    Ai2 = gpu.randomCuITensor(i, seed=3)
    # scalar * tensor (contract!! N1==0 branch, cudense.jl:89-94)
    C = s * Ai
    assert relerr(C.array(i), 3.0 * Ai.array()) < RTOL
    C = Ai * s
    assert relerr(C.array(i), 3.0 * Ai.array()) < RTOL
    # inner product -> order-0
    C = Ai * Ai2
    assert C.order() == 0
    assert abs(C.scalar() - float(Ai.array() @ Ai2.array())) < 1e-13
    # outer product (N1+N2==NR branch)
    C = Ai * Aj
    assert relerr(C.array(i, j), np.outer(Ai.array(), Aj.array())) < RTOL


def test_matrix_cases_all_transposes(gpu, idx):
    i, j, k = idx["i"], idx["j"], idx["k"]
    Aij = gpu.randomCuITensor(i, j, seed=4)
    Ajk = gpu.randomCuITensor(j, k, seed=5)
    for a_inds in ((i, j), (j, i)):
        for b_inds in ((j, k), (k, j)):
            A = gpu.permute(Aij, *a_inds)
            B = gpu.permute(Ajk, *b_inds)
            C = A * B
            ref = _oracle_contract(A, B, C.inds)
            assert relerr(C.array(), ref) < RTOL
    # matrix * vector
    Aj = gpu.randomCuITensor(j, seed=6)
    C = Aij * Aj
    assert relerr(C.array(i), Aij.array(i, j) @ Aj.array()) < RTOL


def test_3tensor_all_permutations(gpu, idx):
    i, j, k, l = idx["i"], idx["j"], idx["k"], idx["l"]
    Aijk = gpu.randomCuITensor(i, j, k, seed=7)
    Ajkl = gpu.randomCuITensor(j, k, l, seed=8)
    for pa in itertools.permutations([i, j, k]):
        for pb in itertools.permutations([j, k, l]):
            A = gpu.permute(Aijk, *pa)
            B = gpu.permute(Ajkl, *pb)
            C = B * A
            assert relerr(C.array(), _oracle_contract(B, A, C.inds)) < RTOL


def test_4tensor_times_3tensor_all_permutations(gpu, idx):
    i, j, k, l, a = idx["i"], idx["j"], idx["k"], idx["l"], idx["a"]
    Aijkl = gpu.randomCuITensor(i, j, k, l, seed=9)
    Akla = gpu.randomCuITensor(k, l, a, seed=10)
    Ajkl = gpu.randomCuITensor(j, k, l, seed=11)
    for p4 in itertools.permutations([i, j, k, l]):
        A4 = gpu.permute(Aijkl, *p4)
        for p3 in itertools.permutations([k, l, a]):
            B = gpu.permute(Akla, *p3)
            C = B * A4
            assert relerr(C.array(), _oracle_contract(B, A4, C.inds)) < RTOL
        for p3 in itertools.permutations([j, k, l]):
            B = gpu.permute(Ajkl, *p3)
            C = B * A4  # -> 1-tensor
            assert relerr(C.array(), _oracle_contract(B, A4, C.inds)) < RTOL


def test_supersized_14_index(gpu):
    I = gpu.Index
    a_only = [I(2) for _ in range(7)]
    b_only = [I(2) for _ in range(7)]
    shared = [I(2) for _ in range(7)]
    A = gpu.randomCuITensor(*(a_only + shared), seed=12)
    B = gpu.randomCuITensor(*(b_only + shared), seed=13)
    C = A * B
    assert relerr(C.array(), _oracle_contract(A, B, C.inds)) < RTOL
    rng = random.Random(5)
    for _ in range(3):
        ia = a_only + shared
        ib = b_only + shared
        rng.shuffle(ia)
        rng.shuffle(ib)
        Ap = gpu.permute(A, *ia)
        Bp = gpu.permute(B, *ib)
        C = Ap * Bp
        assert relerr(C.array(), _oracle_contract(Ap, Bp, C.inds)) < RTOL


def test_random_rank3_to_6_contractions(gpu):
    """Seeded random pairwise contractions (rank 3-6, random permutations)."""
    rng = np.random.default_rng(2024)
    I = gpu.Index
    for trial in range(40):
        nc = int(rng.integers(1, 3))
        na = int(rng.integers(1, 4))
        nb = int(rng.integers(1, 4))
        dims = lambda n: [int(x) for x in rng.integers(2, 9, size=n)]
        c_ids = [I(d) for d in dims(nc)]
        a_ids = [I(d) for d in dims(na)]
        b_ids = [I(d) for d in dims(nb)]
        ia = list(rng.permutation(len(c_ids + a_ids)))
        ib = list(rng.permutation(len(c_ids + b_ids)))
        A = gpu.randomCuITensor(*[(c_ids + a_ids)[q] for q in ia], seed=100 + trial)
        B = gpu.randomCuITensor(*[(c_ids + b_ids)[q] for q in ib], seed=200 + trial)
        C = A * B
        assert relerr(C.array(), _oracle_contract(A, B, C.inds)) < RTOL, trial


def test_large_gemm_shaped_contraction(gpu):
    """H_eff-like shape: L(chi,5,chi) * psi(chi,2,2,chi) at chi = 96 (several tiles, ragged edges)."""
    I = gpu.Index
    chi = 96
    a, w, ap, s1, s2, b = I(chi), I(5), I(chi), I(2), I(2), I(chi)
    L = gpu.randomCuITensor(a, w, ap, seed=31)
    psi = gpu.randomCuITensor(a, s1, s2, b, seed=32)
    C = L * psi
    assert relerr(C.array(), _oracle_contract(L, psi, C.inds)) < RTOL


def test_beta_accumulate_and_errors(gpu):
    import ctypes as C_
    from itg import _lib
    from itg.tensor import _ptr
    h = _lib.handle(0)
    I = gpu.Index
    i, j, k = I(7), I(9), I(11)
    A = gpu.randomCuITensor(i, j, seed=41)
    B = gpu.randomCuITensor(j, k, seed=42)
    C0 = gpu.randomCuITensor(i, k, seed=43)
    Cd = C0.store.data.clone()
    h.call("itg_contract", 0, C_.c_double(2.0), _ptr(A.store.data), 2, _lib.i64arr([7, 9]),
           _lib.i32arr([1, 2]), _ptr(B.store.data), 2, _lib.i64arr([9, 11]), _lib.i32arr([2, 3]),
           C_.c_double(-0.5), _ptr(Cd), 2, _lib.i64arr([7, 11]), _lib.i32arr([1, 3]), 0)
    ref = 2.0 * A.array() @ B.array() - 0.5 * C0.array()
    assert relerr(Cd.cpu().numpy().reshape(7, 11, order="F"), ref) < RTOL
    # dimension mismatch -> DimensionMismatch (the reference's exception)
    with pytest.raises(gpu.DimensionMismatch):
        h.call("itg_contract", 0, C_.c_double(1.0), _ptr(A.store.data), 2, _lib.i64arr([7, 9]),
               _lib.i32arr([1, 2]), _ptr(B.store.data), 2, _lib.i64arr([8, 11]), _lib.i32arr([2, 3]),
               C_.c_double(0.0), _ptr(Cd), 2, _lib.i64arr([7, 11]), _lib.i32arr([1, 3]), 0)
