"""Two-site DMRG path on the GPU against the oracle and known answers.

* H_eff matvec (itg_heff2_apply) vs the oracle at 1e-12 relative Frobenius;
* Davidson (itg_davidson_heff2) vs the oracle's restatement of the same solver;
* dmrg() on the Heisenberg N=20 workload (maxdim [10,20,50,100,100],
  cutoff 1e-10, Davidson maxiter 2): energy vs the oracle's DMRG and vs exact
  diagonalisation;
* the reference's own DMRG known answers (test/dmrg.jl): critical TFIM N=32
  closed form within 1e-2 relative, S=1 Heisenberg N=10 energy < -12, with
  noise 0 and with the reference's noise 1e-10 (density-matrix bond split);
* the noise path against the oracle's restatement and exact diagonalisation;
* MPS utilities: product states, inner, expectation energy.
"""
import ctypes as C
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import itg_oracle as O

pytestmark = pytest.mark.gpu
GOLD = json.loads((Path(__file__).parent / "golden" / "reference_known_answers.json").read_text())


def relerr(x, y):
    return np.linalg.norm((np.asarray(x) - np.asarray(y)).ravel()) / np.linalg.norm(np.asarray(y).ravel())


def _dev(a):
    import torch
    return torch.from_numpy(O.flat(a).copy()).cuda()


def _heff_inputs(chi, chiR=None, d=2, w=5, seed=0):
    chiR = chiR or chi
    rng = np.random.default_rng(seed)
    L = rng.standard_normal((chi, w, chi))
    R = rng.standard_normal((chiR, w, chiR))
    W1 = rng.standard_normal((w, d, d, w))
    W2 = rng.standard_normal((w, d, d, w))
    psi = rng.standard_normal((chi, d, d, chiR))
    return L, W1, W2, R, psi


@pytest.mark.parametrize("chi,chiR,d,w", [(1, 2, 2, 5), (7, 9, 2, 5), (40, 33, 3, 4), (130, 130, 2, 5)])
def test_heff_apply_matches_oracle(gpu, chi, chiR, d, w):
    from itg import _lib
    L, W1, W2, R, psi = _heff_inputs(chi, chiR, d, w, seed=chi)
    out = _dev(np.zeros_like(psi))
    h = _lib.handle(0)
    ptr = lambda t: C.c_void_p(t.data_ptr())
    Ld, W1d, W2d, Rd, pd = map(_dev, (L, W1, W2, R, psi))
    h.call("itg_heff2_apply", C.c_int64(chi), C.c_int64(chiR), C.c_int64(d), C.c_int64(w),
           C.c_int64(w), C.c_int64(w), ptr(Ld), ptr(W1d), ptr(W2d), ptr(Rd), ptr(pd), ptr(out), 0)
    ref = O.heff_apply(L, W1, W2, R, psi)
    got = O.unflat(out.cpu().numpy(), psi.shape)
    assert relerr(got, ref) < 1e-12


def test_heff_diag_matches_oracle(gpu):
    from itg import _lib
    for chi, chiR, d, w in ((5, 7, 2, 5), (24, 24, 2, 5), (33, 17, 3, 4)):
        L, W1, W2, R, psi = _heff_inputs(chi, chiR, d, w, seed=9 + chi)
        h = _lib.handle(0)
        ptr = lambda t: C.c_void_p(t.data_ptr())
        Ld, W1d, W2d, Rd, pd = map(_dev, (L, W1, W2, R, psi))
        dg = _dev(np.zeros_like(psi))
        h.call("itg_heff2_diag", C.c_int64(chi), C.c_int64(chiR), C.c_int64(d), C.c_int64(w),
               C.c_int64(w), C.c_int64(w), ptr(Ld), ptr(W1d), ptr(W2d), ptr(Rd), ptr(dg))
        ref = O.flat(O.heff_diag(L, W1, W2, R))
        assert relerr(dg.cpu().numpy(), ref) < 1e-13


def _sym_heff(chi, d, w, seed):
    L, W1, W2, R, psi = _heff_inputs(chi, d=d, w=w, seed=seed)
    L = L + L.transpose(2, 1, 0)
    R = R + R.transpose(2, 1, 0)
    W1 = W1 + W1.transpose(0, 2, 1, 3)
    W2 = W2 + W2.transpose(0, 2, 1, 3)
    return L, W1, W2, R, psi


def _gpu_davidson(chi, d, w, L, W1, W2, R, psi, kd, mi, tol):
    from itg import _lib
    h = _lib.handle(0)
    ptr = lambda t: C.c_void_p(t.data_ptr())
    Ld, W1d, W2d, Rd, pd = map(_dev, (L, W1, W2, R, psi))
    e = C.c_double()
    nmv = C.c_int()
    h.call("itg_davidson_heff2", C.c_int64(chi), C.c_int64(chi), C.c_int64(d), C.c_int64(w),
           C.c_int64(w), C.c_int64(w), ptr(Ld), ptr(W1d), ptr(W2d), ptr(Rd), ptr(pd), kd, mi,
           C.c_double(tol), 0, C.byref(e), C.byref(nmv))
    return e.value, pd.cpu().numpy(), nmv.value


def test_davidson_converges_to_lowest_eigenvalue(gpu):
    """Converged runs reach the exact lowest eigenvalue of the (dense) operator.

    The operator is a random symmetric H_eff; its Rayleigh quotients start in
    the interior of diag(H), where a diagonally preconditioned Davidson is
    sensitive to rounding (1e-16 perturbations change a 5-matvec energy at
    1e-7), so only converged results are compared here."""
    chi, d, w = 12, 2, 5
    L, W1, W2, R, psi = _sym_heff(chi, d, w, seed=3)
    n = chi * d * d * chi
    H = np.stack([O.flat(O.heff_apply(L, W1, W2, R, O.unflat(np.eye(n)[:, i], psi.shape)))
                  for i in range(n)], axis=1)
    e0 = np.linalg.eigvalsh(0.5 * (H + H.T))[0]
    e, x, nmv = _gpu_davidson(chi, d, w, L, W1, W2, R, psi, 10, 200, 1e-9)
    assert abs(e - e0) < 1e-10 * abs(e0)
    assert np.linalg.norm(H @ x - e * x) < 1e-8 * abs(e0)


def test_davidson_matches_oracle_trajectory(gpu):
    """Well-conditioned start (the ground state plus 1e-3 noise): the GPU solver
    and the oracle's restatement follow the same iterates (same matvec count,
    energies within 1e-12 relative)."""
    chi, d, w = 12, 2, 5
    L, W1, W2, R, psi = _sym_heff(chi, d, w, seed=4)
    n = chi * d * d * chi
    H = np.stack([O.flat(O.heff_apply(L, W1, W2, R, O.unflat(np.eye(n)[:, i], psi.shape)))
                  for i in range(n)], axis=1)
    wv, V = np.linalg.eigh(0.5 * (H + H.T))
    rng = np.random.default_rng(0)
    start = O.unflat(V[:, 0] + 1e-3 * rng.standard_normal(n), psi.shape)
    mv = lambda v: H @ v
    dg = O.flat(O.heff_diag(L, W1, W2, R))
    for kd, mi in ((3, 2), (5, 3)):
        th_o, x_o, nmv_o = O.davidson(mv, O.flat(start), dg, kd, mi, 1e-14)
        e, x, nmv = _gpu_davidson(chi, d, w, L, W1, W2, R, start, kd, mi, 1e-14)
        assert nmv == nmv_o
        assert abs(e - th_o) < 1e-12 * abs(th_o)
        assert min(np.linalg.norm(x - x_o), np.linalg.norm(x + x_o)) < 1e-8


def test_davidson_graph_replay_identical(gpu):
    """itg_set_graphs(1): the captured H_eff chain replays the same kernels in
    the same order, so results are bit-identical to direct launches."""
    from itg import _lib
    chi, d, w = 20, 2, 5
    L, W1, W2, R, psi = _sym_heff(chi, d, w, seed=5)
    h = _lib.handle(0)
    res = []
    for g in (0, 1):
        h.call("itg_set_graphs", g)
        try:
            res.append(_gpu_davidson(chi, d, w, L, W1, W2, R, psi, 4, 3, 1e-14))
        finally:
            h.call("itg_set_graphs", 0)
    (e0, x0, n0), (e1, x1, n1) = res
    assert n0 == n1 and e0 == e1 and np.array_equal(x0, x1)


def _run_dmrg_pair(gpu, N, d, mpo_gpu, mpo_oracle, linkdim, seed, maxdims, cutoffs, nsweep, **kw):
    sites = gpu.siteinds("S=1/2" if d == 2 else "S=1", N)
    H = gpu.cuMPO(mpo_gpu(sites))
    psi0 = gpu.randomCuMPS(sites, linkdim, seed=seed)
    sw = gpu.Sweeps(nsweep, maxdim=maxdims, cutoff=cutoffs, mindim=kw.pop("mindim", [1]))
    res = gpu.dmrg(H, psi0, sw, return_result=True, **kw)
    e_o, _, hist = O.dmrg(mpo_oracle(N), O.random_mps([d] * N, linkdim, seed), maxdims, cutoffs, nsweep,
                          return_sweeps=True)
    return res, e_o, hist


def test_dmrg_heisenberg_n20_matches_oracle_and_ed(gpu):
    """The plain-method Heisenberg N=20 workload end to end."""
    N = 20
    res, e_o, hist = _run_dmrg_pair(gpu, N, 2, gpu.heisenberg_mpo, lambda n: O.heisenberg_mpo(n), 10,
                                    1234 + 0, [10, 20, 50, 100, 100], [1e-10], 5)
    e_ed = GOLD["ed"]["heisenberg_N20"]
    assert abs(res.energy - e_o) < 1e-10, (res.energy, e_o, res.energy - e_o)
    assert abs(res.energy - e_ed) < 1e-7
    assert res.psi.maxlinkdim() <= 100
    # per-sweep energies track the oracle
    for rec, (eo, _, _) in zip(res.sweeps, hist):
        assert abs(rec.energy - eo) < 1e-6


@pytest.mark.parametrize("form", ["chosen", "plain"])
def test_dmrg_heisenberg_n100_matches_oracle_fixture(gpu, form):
    """The N = 100 Heisenberg workload (random MPS of link dimension 16, Philox
    seed 1236; 10 sweeps with maxdim 16 -> 1024, cutoff 1e-12) in the chosen form
    (split-precision contractions, mixed SVD) and the plain form (FP64
    contractions, FP64 Jacobi SVD): final energy within 1e-10 of the oracle's
    FP64 run of the same workload (tests/golden/config3_oracle.json, made by
    tests/golden/make_config3_energy.py)."""
    fix = json.loads((Path(__file__).parent / "golden" / "config3_oracle.json").read_text())
    N = fix["N"]
    sites = gpu.siteinds("S=1/2", N)
    H = gpu.cuMPO(gpu.heisenberg_mpo(sites))
    psi0 = gpu.randomCuMPS(sites, fix["linkdim"], seed=fix["seed"])
    sw = gpu.Sweeps(fix["nsweep"], maxdim=fix["maxdims"], cutoff=[fix["cutoff"]])
    prec, svd = ("split", 2) if form == "chosen" else ("fp64", 1)
    res = gpu.dmrg(H, psi0, sw, precision=prec, svd_method=svd, return_result=True)
    assert abs(res.energy - fix["energy"]) < 1e-10, (form, res.energy, fix["energy"])
    # the sweeps follow the oracle's convergence once maxdim stops binding
    for rec, eo in list(zip(res.sweeps, fix["sweep_energies"]))[5:]:
        assert abs(rec.energy - eo) < 1e-9, (rec.energy, eo)


def _rotated_heisenberg(gpu, sites, seed):
    """U H U^dagger for the S=1/2 Heisenberg MPO and random single-site unitaries
    u_j: complex Hermitian site operators, the spectrum of H unchanged."""
    from itg.mps import MPO
    rng = np.random.default_rng(seed)
    H = gpu.heisenberg_mpo(sites)
    out = []
    for j, t in enumerate(H.tensors):
        z = rng.standard_normal((2, 2)) + 1j * rng.standard_normal((2, 2))
        u, _ = np.linalg.qr(z)
        W = t.array()                                   # (wl, s', s, wr)
        Wr = np.einsum("ap,wpqx,bq->wabx", u, W, u.conj())
        out.append(gpu.ITensor_host(Wr, *t.inds))
    return MPO(out, sites)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("split", 1e-9)])
def test_dmrg_complex_rotated_heisenberg_matches_ed(gpu, precision, tol):
    """A complex DMRG sweep (ComplexF64 MPO and MPS: ITensors' algorithm on the
    library's complex contraction, SVD and QR entry points): the Heisenberg
    chain N = 12 rotated by random single-site unitaries has complex matrix
    elements and the spectrum of the real chain, so the ground energy must be
    the exact-diagonalisation value."""
    N = 12
    sites = gpu.siteinds("S=1/2", N)
    H = gpu.cuMPO(_rotated_heisenberg(gpu, sites, seed=21))
    assert all(t.is_complex for t in H.tensors)
    psi0 = gpu.randomCuMPS(sites, 4, seed=8)
    sw = gpu.Sweeps(8, maxdim=[8, 16, 32, 64], cutoff=[1e-14])
    res = gpu.dmrg(H, psi0, sw, krylovdim=4, maxiter=3, eigsolve_tol=1e-13, precision=precision,
                   return_result=True)
    e_ed = GOLD["ed"]["heisenberg_N12"]
    assert abs(res.energy - e_ed) < tol, (res.energy, e_ed)
    assert all(t.is_complex for t in res.psi.tensors)
    # the state is an eigenvector: <psi|H|psi> = E with <psi|psi> = 1
    e_exp = gpu.inner(res.psi, H, res.psi)
    assert abs(complex(e_exp) - res.energy) < 10 * tol


def test_dmrg_heisenberg_n12_exact(gpu):
    """No truncation needed at N=12: the energy must reach ED at 1e-10."""
    N = 12
    res, e_o, _ = _run_dmrg_pair(gpu, N, 2, gpu.heisenberg_mpo, lambda n: O.heisenberg_mpo(n), 10, 77,
                                 [10, 20, 50, 100], [1e-14], 6)
    assert abs(res.energy - GOLD["ed"]["heisenberg_N12"]) < 1e-10
    assert abs(res.energy - e_o) < 1e-10


def test_dmrg_tfim_closed_form(gpu):
    g = GOLD["dmrg"]["tfim"]
    N = g["N"]
    sites = gpu.siteinds("S=1/2", N)
    H = gpu.cuMPO(gpu.tfim_mpo(sites, h=g["h"], J=g["J"]))
    psi0 = gpu.randomCuMPS(sites, 1, seed=g["seed"])
    sw = gpu.Sweeps(g["nsweep"], maxdim=g["maxdim"], cutoff=[g["cutoff"]])
    energy, psi = gpu.dmrg(H, psi0, sw)
    exact = O.tfim_closed_form(N)
    assert abs((energy - exact) / exact) < g["rel_tol"]
    assert abs(energy - exact) < 1e-6
    e_o, _ = O.dmrg(O.tfim_mpo(N, h=g["h"], J=g["J"]), O.random_mps([2] * N, 1, g["seed"]), g["maxdim"],
                    [g["cutoff"]], g["nsweep"])
    assert abs(energy - e_o) < 1e-9
    assert abs(gpu.expect_energy(H, psi) - energy) < 1e-9


def test_dmrg_spin1_bound(gpu):
    g = GOLD["dmrg"]["spin1_heisenberg"]
    sites = gpu.siteinds("S=1", g["N"])
    H = gpu.cuMPO(gpu.heisenberg_mpo(sites))
    psi0 = gpu.randomCuMPS(sites, 1, seed=11)
    sw = gpu.Sweeps(g["nsweep"], maxdim=g["maxdim"], mindim=g["mindim"], cutoff=[g["cutoff"]])
    energy, psi = gpu.dmrg(H, psi0, sw)
    assert energy < g["energy_below"]


def test_dmrg_noise_matches_oracle_and_ed(gpu):
    """noise > 0: bonds split through the perturbed density matrix and
    itg_eigh_trunc; the oracle restates ITensors' noise term in NumPy."""
    N = 10
    sites = gpu.siteinds("S=1/2", N)
    H = gpu.cuMPO(gpu.heisenberg_mpo(sites))
    noises = [1e-5, 1e-7, 1e-9, 0.0]
    sw = gpu.Sweeps(5, maxdim=[10, 20, 40, 64], cutoff=[1e-12], noise=noises)
    res = gpu.dmrg(H, gpu.randomCuMPS(sites, 4, seed=7), sw, return_result=True)
    e_o, _ = O.dmrg(O.heisenberg_mpo(N), O.random_mps([2] * N, 4, 7), [10, 20, 40, 64], [1e-12], 5,
                    noises=noises)
    assert abs(res.energy - e_o) < 1e-9
    assert abs(res.energy - O.heisenberg_ed_sz0(N)) < 1e-9
    assert abs(gpu.expect_energy(H, res.psi) - res.energy) < 1e-9


def test_dmrg_reference_cases_with_noise(gpu):
    """test/dmrg.jl as written: both known answers with noise!(sweeps, 1E-10)."""
    g = GOLD["dmrg"]["spin1_heisenberg"]
    sites = gpu.siteinds("S=1", g["N"])
    H = gpu.cuMPO(gpu.heisenberg_mpo(sites))
    sw = gpu.Sweeps(g["nsweep"], maxdim=g["maxdim"], mindim=g["mindim"], cutoff=[g["cutoff"]], noise=[1e-10])
    energy, _ = gpu.dmrg(H, gpu.randomCuMPS(sites, 1, seed=11), sw)
    assert energy < g["energy_below"]
    g = GOLD["dmrg"]["tfim"]
    sites = gpu.siteinds("S=1/2", g["N"])
    H = gpu.cuMPO(gpu.tfim_mpo(sites, h=g["h"], J=g["J"]))
    sw = gpu.Sweeps(g["nsweep"], maxdim=g["maxdim"], cutoff=[g["cutoff"]], noise=[1e-10])
    energy, _ = gpu.dmrg(H, gpu.randomCuMPS(sites, 1, seed=g["seed"]), sw)
    exact = O.tfim_closed_form(g["N"])
    assert abs((energy - exact) / exact) < g["rel_tol"]


def test_product_state_and_inner(gpu):
    N = 6
    sites = gpu.siteinds("S=1/2", N)
    up = gpu.productCuMPS(sites, ["Up"] * N)
    neel = gpu.productCuMPS(sites, ["Up", "Dn"] * (N // 2))
    assert gpu.inner(up, up) == pytest.approx(1.0)
    assert gpu.inner(up, neel) == pytest.approx(0.0)
    H = gpu.cuMPO(gpu.heisenberg_mpo(sites))
    # <up|H|up> = (N-1)/4 ; <neel|H|neel> = -(N-1)/4
    assert gpu.expect_energy(H, up) == pytest.approx((N - 1) / 4, abs=1e-14)
    assert gpu.expect_energy(H, neel) == pytest.approx(-(N - 1) / 4, abs=1e-14)
    psi = gpu.cpu(gpu.randomCuMPS(sites, 4, seed=3))
    assert not psi.is_cuda and gpu.cuMPS(psi).is_cuda
