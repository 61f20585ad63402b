"""Split-precision contraction path (ITG_PREC_SPLIT) against the oracle.

* integer inputs (|x| <= 63) are represented exactly by the leading digit, so
  the tcgen05 pipeline must reproduce the FP64 result bit for bit: this checks
  the TMA tiles, the MMA descriptors, the exact TMEM partial sums, the int64
  drains and the integer FP64 conversion;
* Gaussian inputs: relative Frobenius error below the stated bound
  itg_split_error_bound(K) * |A|_F |B|_F / |C|_F, and in practice below 1e-12;
* ragged shapes (M, N, K not multiples of the tiles), both operand layouts, the
  N <= 128 tile, K long enough for many exact groups and all levels, and for a
  level whose int32 group sums must be flushed part-way (more than 127 groups);
* the H_eff chain with ITG_PREC_SPLIT, and a DMRG run whose energy matches the
  FP64 run within 1e-9.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import itg_oracle as O

pytestmark = pytest.mark.gpu


def _contract(gpu, A, dA, mA, B, dB, mB, dC, mC, prec):
    import torch
    from itg import _lib
    h = _lib.handle(0)
    out = torch.empty(int(np.prod(dC)), dtype=torch.float64, device="cuda")
    p = lambda t: C.c_void_p(t.data_ptr())
    h.call("itg_contract", 0, C.c_double(1.0), p(A), len(dA), _lib.i64arr(dA), _lib.i32arr(mA), p(B),
           len(dB), _lib.i64arr(dB), _lib.i32arr(mB), C.c_double(0.0), p(out), len(dC), _lib.i64arr(dC),
           _lib.i32arr(mC), prec)
    return out


def _dev(a):
    import torch
    return torch.from_numpy(O.flat(a).copy()).cuda()


CASES = [
    # (dims A, modes A, dims B, modes B, modes C): GEMM-like with K-major / M-major operands
    ((64, 32), (1, 2), (32, 48), (2, 3), (1, 3)),                # M-major A, K-major B
    ((32, 200), (2, 1), (32, 130), (2, 3), (1, 3)),              # K-major A, ragged M, N > 128
    ((300, 7, 5), (1, 2, 3), (7, 5, 257), (2, 3, 4), (4, 1)),    # C transposed, ragged
    ((1000, 40), (2, 1), (1000, 90), (2, 3), (1, 3)),            # long K: many groups, N <= 128
    ((96, 5, 96), (1, 2, 3), (96, 2, 2, 96), (1, 4, 5, 6), (3, 6, 2, 4, 5)),  # H_eff step 1
    ((60000, 130), (2, 1), (60000, 260), (2, 3), (1, 3)),        # K = 60000: a level of > 127 groups
]


@pytest.mark.parametrize("case", CASES, ids=[str(i) for i in range(len(CASES))])
def test_split_integer_inputs_exact(gpu, case):
    dA, mA, dB, mB, mC = case
    rng = np.random.default_rng(len(dA) * 7 + dA[0])
    A = rng.integers(-63, 64, size=dA).astype(np.float64)
    B = rng.integers(-63, 64, size=dB).astype(np.float64)
    lab = dict(zip(mA, dA))
    lab.update(zip(mB, dB))
    dC = tuple(lab[m] for m in mC)
    ref = O.contract(A, list(mA), B, list(mB), list(mC))
    got = _contract(gpu, _dev(A), dA, mA, _dev(B), dB, mB, dC, mC, 1).cpu().numpy()
    assert np.array_equal(O.unflat(got, dC), ref)


@pytest.mark.parametrize("case", CASES, ids=[str(i) for i in range(len(CASES))])
def test_split_gaussian_within_bound(gpu, case):
    from itg import _lib
    lib = _lib.load_library()
    dA, mA, dB, mB, mC = case
    rng = np.random.default_rng(17 + dA[0])
    A = rng.standard_normal(dA)
    B = rng.standard_normal(dB)
    lab = dict(zip(mA, dA))
    lab.update(zip(mB, dB))
    dC = tuple(lab[m] for m in mC)
    K = int(np.prod([lab[m] for m in mA if m in mB]))
    ref = O.contract(A, list(mA), B, list(mB), list(mC))
    got = O.unflat(_contract(gpu, _dev(A), dA, mA, _dev(B), dB, mB, dC, mC, 1).cpu().numpy(), dC)
    err = np.linalg.norm(got - ref)
    bound = lib.itg_split_error_bound(K) * np.linalg.norm(A) * np.linalg.norm(B)
    assert err <= bound
    assert err / np.linalg.norm(ref) < 1e-12


def test_split_wide_dynamic_range(gpu):
    """Rows/columns with very different scales: per-row/column exponents."""
    rng = np.random.default_rng(3)
    A = rng.standard_normal((200, 150)) * np.exp2(rng.integers(-40, 40, size=(200, 1)))
    B = rng.standard_normal((150, 170)) * np.exp2(rng.integers(-40, 40, size=(1, 170)))
    ref = A @ B
    got = O.unflat(_contract(gpu, _dev(A), (200, 150), (1, 2), _dev(B), (150, 170), (2, 3), (200, 170),
                             (1, 3), 1).cpu().numpy(), (200, 170))
    # element-wise relative to the row/column scales
    scale = np.abs(A).max(1, keepdims=True) * np.abs(B).max(0, keepdims=True) * 150
    assert np.max(np.abs(got - ref) / scale) < 1e-13


def test_split_heff_matches_oracle(gpu):
    from itg import _lib
    import torch
    chi, d, w = 128, 2, 5
    rng = np.random.default_rng(5)
    L = rng.standard_normal((chi, w, chi))
    R = rng.standard_normal((chi, w, chi))
    W1 = rng.standard_normal((w, d, d, w))
    W2 = rng.standard_normal((w, d, d, w))
    psi = rng.standard_normal((chi, d, d, chi))
    h = _lib.handle(0)
    p = lambda t: C.c_void_p(t.data_ptr())
    Ld, W1d, W2d, Rd, pd = map(_dev, (L, W1, W2, R, psi))
    out = torch.empty_like(pd)
    h.call("itg_heff2_apply", C.c_int64(chi), C.c_int64(chi), C.c_int64(d), C.c_int64(w), C.c_int64(w),
           C.c_int64(w), p(Ld), p(W1d), p(W2d), p(Rd), p(pd), p(out), 1)
    ref = O.heff_apply(L, W1, W2, R, psi)
    got = O.unflat(out.cpu().numpy(), psi.shape)
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-12


@pytest.mark.parametrize("chiL,chiR,d,w", [(7, 9, 2, 5), (40, 33, 2, 4), (130, 130, 2, 5), (50, 70, 2, 3),
                                            (33, 17, 3, 4)])
def test_split_heff_middle_step_shapes(gpu, chiL, chiR, d, w):
    """The split matvec's middle step runs on the tensor cores for nc = w d^2 and
    nj = d^2 w up to 32 (one or two K = 16 steps, 16- or 32-column TMEM level
    accumulators, a ragged last row block) and on FP64 FMA above (d = 3, w = 4:
    nc = 36); both within 1e-12 of the oracle."""
    from itg import _lib
    import torch
    rng = np.random.default_rng(chiL * 7 + chiR)
    L = rng.standard_normal((chiL, w, chiL))
    R = rng.standard_normal((chiR, w, chiR))
    W1 = rng.standard_normal((w, d, d, w))
    W2 = rng.standard_normal((w, d, d, w))
    psi = rng.standard_normal((chiL, d, d, chiR))
    h = _lib.handle(0)
    p = lambda t: C.c_void_p(t.data_ptr())
    Ld, W1d, W2d, Rd, pd = map(_dev, (L, W1, W2, R, psi))
    out = torch.full_like(pd, float("nan"))
    h.call("itg_heff2_apply", C.c_int64(chiL), C.c_int64(chiR), C.c_int64(d), C.c_int64(w), C.c_int64(w),
           C.c_int64(w), p(Ld), p(W1d), p(W2d), p(Rd), p(pd), p(out), 1)
    ref = O.heff_apply(L, W1, W2, R, psi)
    got = O.unflat(out.cpu().numpy(), psi.shape)
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-12


def test_split_dmrg_energy_matches_fp64(gpu):
    N = 16
    sites = gpu.siteinds("S=1/2", N)
    H = gpu.cuMPO(gpu.heisenberg_mpo(sites))
    psi0 = gpu.randomCuMPS(sites, 10, seed=1234)
    sw = gpu.Sweeps(4, maxdim=[10, 20, 50, 64], cutoff=[1e-12])
    e64, _ = gpu.dmrg(H, psi0, sw, precision="fp64")
    esp, _ = gpu.dmrg(H, psi0, sw, precision="split")
    assert abs(esp - e64) < 1e-9


def test_chosen_form_keeps_mps_orthonormal(gpu):
    """Split products + mixed SVD (bond splits through FP32 Jacobi, FP64
    refinement and Newton-Schulz): every site right of the centre stays
    right-orthonormal to 1e-13 after the sweeps.  Bond dimensions reach 256, so
    the splits go through the blocked FP32 Jacobi on 512-column matrices; the
    sweep builds its environments assuming this orthonormality, and a loss of
    delta would show up as a relative energy error of about N * delta."""
    N = 24
    sites = gpu.siteinds("S=1/2", N)
    H = gpu.cuMPO(gpu.heisenberg_mpo(sites))
    sw = gpu.Sweeps(3, maxdim=[64, 256], cutoff=[0.0])
    res = gpu.dmrg(H, gpu.randomCuMPS(sites, 16, seed=5), sw, precision="split", svd_method=2,
                   return_result=True)
    psi = res.psi
    assert psi.maxlinkdim() == 256
    worst = 0.0
    for j in range(1, N):
        t = psi[j]
        l = t.inds[0]
        P = (t * t.replaceinds([l], [l.prime()])).array(l, l.prime())
        worst = max(worst, np.abs(P - np.eye(l.dim)).max())
    assert worst < 1e-13, worst
    assert abs(gpu.expect_energy(H, psi) - res.energy) < 1e-11
