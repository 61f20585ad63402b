"""Parity at the benchmark workloads' own sizes, through the C ABI.

* Two-site H_eff matvec (itg_heff2_apply) at chi in {256, 512, 1024, 2048},
  L, R (chi, 5, chi), psi (chi, 2, 2, chi), W1, W2 (5, 2, 2, 5), entries
  N(0, 1): FP64 and split precision against the oracle's FP64 matvec
  (oracle.heff_apply, the four-contraction ProjMPO product) within 1e-12
  relative Frobenius.  The reference anchor is the pattern of
  test/test_cucontract.jl:170-196 (GPU contraction vs the CPU result).
* The seeded random pairwise contractions of the contraction benchmark
  (ranks 3-6, random index orders, dims 2..2048, M, N, K ~ 2^10..2^12): FP64
  and split against the oracle's compensated checker (oracle.contract_exact:
  error-free integer slices, exact BLAS products, compensated recombination),
  which is accurate to about one rounding of each output even at the largest
  contraction depth, within 1e-12 relative Frobenius; the split path also
  within its stated bound (itg_split_error_bound).
"""
import ctypes as C

import numpy as np
import pytest

from oracle import itg_oracle as O

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def relerr(x, y):
    return np.linalg.norm((np.asarray(x) - np.asarray(y)).ravel()) / np.linalg.norm(np.asarray(y).ravel())


def _dev(a):
    import torch
    return torch.from_numpy(O.flat(a).copy()).cuda()


@pytest.fixture(scope="module", params=[256, 512, 1024, 2048])
def heff_case(request):
    chi, d, w = request.param, 2, 5
    rng = np.random.default_rng(1234 + 1 + chi)
    L = rng.standard_normal((chi, w, chi))
    R = rng.standard_normal((chi, w, chi))
    W1 = rng.standard_normal((w, d, d, w))
    W2 = rng.standard_normal((w, d, d, w))
    psi = rng.standard_normal((chi, d, d, chi))
    ref = O.heff_apply(L, W1, W2, R, psi)
    return chi, d, w, (L, W1, W2, R, psi), ref


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "split"])
def test_heff_apply_at_benchmark_chi_matches_oracle(gpu, heff_case, precision):
    import torch
    from itg import _lib
    chi, d, w, ins, ref = heff_case
    h = _lib.handle(0)
    ptr = lambda t: C.c_void_p(t.data_ptr())
    Ld, W1d, W2d, Rd, pd = map(_dev, ins)
    out = torch.full_like(pd, float("nan"))
    h.call("itg_heff2_apply", C.c_int64(chi), C.c_int64(chi), C.c_int64(d), C.c_int64(w), C.c_int64(w),
           C.c_int64(w), ptr(Ld), ptr(W1d), ptr(W2d), ptr(Rd), ptr(pd), ptr(out), precision)
    got = O.unflat(out.cpu().numpy(), ins[4].shape)
    err = relerr(got, ref)
    assert err <= RTOL, (chi, precision, err)


def _contract_cases():
    import bench
    return bench._contract_cases(8, 1234 + 2)


@pytest.mark.parametrize("ci", range(8))
def test_benchmark_random_contractions_match_compensated_oracle(gpu, ci):
    import torch
    from itg import _lib
    mA, mB, mC, dims, mnk = _contract_cases()[ci]
    dA, dB, dC = ([dims[m] for m in ms] for ms in (mA, mB, mC))
    rng = np.random.default_rng(50 + ci)
    A = rng.standard_normal(dA)
    B = rng.standard_normal(dB)
    ref = O.contract_exact(A, mA, B, mB, mC)
    K = int(np.prod([dims[m] for m in mA if m not in mC]))
    h = _lib.handle(0)
    p = lambda t: C.c_void_p(t.data_ptr())
    Ad, Bd = _dev(A), _dev(B)
    nrm = np.linalg.norm(ref.ravel())
    for prec in (0, 1):
        Cd = torch.full((int(np.prod(dC)),), float("nan"), dtype=torch.float64, device="cuda")
        h.call("itg_contract", 0, C.c_double(1.0), p(Ad), len(mA), _lib.i64arr(dA), _lib.i32arr(mA),
               p(Bd), len(mB), _lib.i64arr(dB), _lib.i32arr(mB), C.c_double(0.0), p(Cd), len(mC),
               _lib.i64arr(dC), _lib.i32arr(mC), prec)
        got = O.unflat(Cd.cpu().numpy(), dC)
        err = relerr(got, ref)
        assert err <= RTOL, (ci, prec, K, err)
        if prec == 1:
            bound = h.lib.itg_split_error_bound(K) * np.linalg.norm(A.ravel()) * np.linalg.norm(B.ravel())
            assert np.linalg.norm((got - ref).ravel()) <= bound, (ci, K)
        del Cd
    assert nrm > 0
