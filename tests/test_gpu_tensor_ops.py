"""Permutation, permuted add, Diag contractions, level-1 kernels, RNG (GPU vs oracle).

Exact (bit-identical) where the reference tests use == : permute
(test/test_cuitensor.jl:29-54) and permuted + (test/test_cuitensor.jl:89-99,
test/test_cudense.jl:16-42).
"""
import ctypes as C
import itertools
import random

import numpy as np
import pytest

from oracle import itg_oracle as O

pytestmark = pytest.mark.gpu


def relerr(x, y):
    nd = np.linalg.norm(np.asarray(y).ravel())
    return np.linalg.norm((np.asarray(x) - np.asarray(y)).ravel()) / (nd if nd > 0 else 1.0)


def test_permute_exact_all_orders(gpu):
    I = gpu.Index
    i, j, k, l = I(2), I(3), I(33), I(17)
    A = gpu.randomCuITensor(i, j, k, l, seed=1)
    Ah = A.array()
    for p in itertools.permutations([i, j, k, l]):
        P = gpu.permute(A, *p)
        ref = O.permute(Ah, [i, j, k, l], list(p))
        assert np.array_equal(P.array(), ref)


def test_permute_large_tensor_14_indices_exact(gpu):
    I = gpu.Index
    inds = [I(2) for _ in range(14)]
    A = gpu.randomCuITensor(*inds, seed=2)
    Ah = A.array()
    rng = random.Random(0)
    for _ in range(20):
        p = inds[:]
        rng.shuffle(p)
        assert np.array_equal(gpu.permute(A, *p).array(), O.permute(Ah, inds, p))


def test_permute_wide_transpose(gpu):
    I = gpu.Index
    a, b = I(1000), I(777)
    A = gpu.randomCuITensor(a, b, seed=3)
    assert np.array_equal(gpu.permute(A, b, a).array(), A.array().T)


def test_add_sub_permuted_exact(gpu):
    I = gpu.Index
    i, j, k = I(2), I(3), I(4)
    dA = gpu.randomCuITensor(i, j, k, seed=4)
    dB = gpu.randomCuITensor(k, i, j, seed=5)
    A, B = dA.array(i, j, k), dB.array(i, j, k)
    assert np.array_equal((dA + dB).array(i, j, k), A + B)
    assert np.array_equal((dA - dB).array(i, j, k), A - B)
    assert np.array_equal((dB + dA).array(i, j, k), B + A)
    with pytest.raises(gpu.DimensionMismatch):
        _ = dA + gpu.randomCuITensor(i, j, seed=6)


def test_scalar_mul_div_norm(gpu):
    I = gpu.Index
    A = gpu.randomCuITensor(I(5), I(6), seed=7)
    Ah = A.array()
    assert np.array_equal((2.5 * A).array(), 2.5 * Ah)
    assert relerr((A / 4.0).array(), Ah / 4.0) < 1e-15
    assert abs(gpu.norm(A) - np.linalg.norm(Ah)) < 1e-13 * np.linalg.norm(Ah)


def test_random_normal_matches_oracle_stream(gpu):
    I = gpu.Index
    A = gpu.randomCuITensor(I(1001), seed=99)
    ref = O.philox_normal(1001, 99, 0)
    assert np.allclose(A.array(), ref, rtol=1e-13, atol=1e-14)


def test_diag_times_dense_all_orders(gpu):
    I = gpu.Index
    i, j, k = I(6), I(6), I(5)
    d = np.arange(1.0, 7.0)
    D = gpu.diagITensor(d, i, j)
    T = gpu.randomCuITensor(j, k, seed=8)
    for p in itertools.permutations([j, k]):
        Tp = gpu.permute(T, *p)
        for order in (lambda: D * Tp, lambda: Tp * D):
            C = order()
            ref = O.diag_dense(d, (6, 6), ["i", "j"], False, Tp.array(),
                               ["j" if x == j else "k" for x in Tp.inds],
                               ["i" if x == i else ("j" if x == j else "k") for x in C.inds])
            assert relerr(C.array(), ref) < 1e-15
    # full contraction of the diagonal with a matrix on both indices (trace-like)
    M = gpu.randomCuITensor(i, j, seed=9)
    C = D * M
    assert abs(C.scalar() - float(np.sum(d * np.diag(M.array())))) < 1e-12


def test_uniform_diag_respects_permutation(gpu):
    """UniformDiag x dense with a permuted order (the case cudiag.jl:105-112 gets wrong,
    test/test_cudiag.jl:49,95 are @test_broken)."""
    I = gpu.Index
    i, j, k = I(4), I(4), I(3)
    T = gpu.randomCuITensor(k, j, seed=10)
    D = gpu.delta(i, j, value=2.0)
    C = D * T
    ref = 2.0 * O.permute(T.array(), ["k", "j"], ["k", "j"])
    assert relerr(C.array(k, i), ref) < 1e-15


def test_diag_times_diag_and_dense(gpu):
    I = gpu.Index
    i, j, k = I(5), I(5), I(5)
    a = np.arange(1.0, 6.0)
    b = np.linspace(-1, 1, 5)
    A = gpu.diagITensor(a, i, j)
    B = gpu.diagITensor(b, j, k)
    C = A * B
    assert C.isdiag()
    assert relerr(C.store.data.cpu().numpy(), a * b) < 1e-15
    full = gpu.dense(C).array(i, k)
    assert relerr(full, np.diag(a * b)) < 1e-15
    U = gpu.delta(i, j, value=3.0)
    C2 = U * B
    assert relerr(C2.store.data.cpu().numpy(), 3.0 * b) < 1e-15


def test_dot_nrm2_axpy_deterministic(gpu):
    from itg import _lib
    from itg.tensor import _ptr
    import torch
    h = _lib.handle(0)
    n = 1_000_003
    x = torch.from_numpy(O.philox_normal(n, 5)).cuda()
    y = torch.from_numpy(O.philox_normal(n, 6)).cuda()
    r1, r2 = C.c_double(), C.c_double()
    h.call("itg_dot", C.c_int64(n), _ptr(x), _ptr(y), C.byref(r1))
    h.call("itg_dot", C.c_int64(n), _ptr(x), _ptr(y), C.byref(r2))
    assert r1.value == r2.value
    ref = float(np.dot(x.cpu().numpy(), y.cpu().numpy()))
    assert abs(r1.value - ref) < 1e-10 * np.sqrt(n)
    h.call("itg_nrm2", C.c_int64(n), _ptr(x), C.byref(r1))
    assert abs(r1.value - np.linalg.norm(x.cpu().numpy())) < 1e-12 * r1.value
    yy = y.clone()
    h.call("itg_axpy", C.c_int64(n), C.c_double(0.5), _ptr(x), _ptr(yy))
    assert relerr(yy.cpu().numpy(), y.cpu().numpy() + 0.5 * x.cpu().numpy()) < 1e-15


def test_cu_cpu_roundtrip(gpu):
    I = gpu.Index
    i, j = I(3), I(4)
    arr = np.arange(12.0).reshape(3, 4)
    A = gpu.ITensor_host(arr, i, j)
    dA = gpu.cu(A)
    assert dA.is_cuda
    back = gpu.cpu(dA)
    assert not back.is_cuda and np.array_equal(back.array(), arr)
    assert np.array_equal(gpu.cuITensor(arr, i, j).array(j, i), arr.T)
