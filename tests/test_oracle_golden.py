"""Pin the CPU oracle against the reference's own known answers (no GPU).

* truncate! golden vectors: test/test_cutruncate.jl:9-17
* TFIM closed form: test/dmrg.jl:58-81
* S=1 Heisenberg bound: test/dmrg.jl:5-29
* exact diagonalisation of the Heisenberg chain (independent known answer)
"""
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import itg_oracle as O

GOLD = json.loads((Path(__file__).parent / "golden" / "reference_known_answers.json").read_text())


@pytest.mark.parametrize("case", GOLD["truncate"], ids=lambda c: c["source"])
def test_truncate_legacy_matches_reference_golden(case):
    kw = case["kwargs"]
    n, te, dc = O.truncate_legacy_gpu(case["P"], cutoff=kw.get("cutoff", 0.0),
                                      absoluteCutoff=kw.get("absoluteCutoff", False))
    P = np.asarray(case["P"])
    kept = [0.0] if P.max() == 0 else list(P[:n])
    assert kept == case["kept"]
    assert te == pytest.approx(case["truncerr"], rel=1.5e-8, abs=1e-300)
    assert dc == pytest.approx(case["docut"], rel=1.5e-8, abs=1e-300)


def test_truncate_legacy_vs_cumulative_differ_as_documented():
    # P = exp(-2k/3), cutoff 1e-10: the reference GPU rule keeps len - cut_ind
    # states, the ITensors CPU rule keeps the cumulative-tail count.
    P = np.exp(-2 * np.arange(40) / 3)
    n_legacy, _, _ = O.truncate_legacy_gpu(P, cutoff=1e-10)
    n_cpu, _, _ = O.truncate_cpu(P, cutoff=1e-10)
    assert n_legacy == 6
    assert n_cpu == 35


def test_truncate_cpu_rules():
    P = np.array([0.5, 0.3, 0.1, 0.06, 0.04])
    # cumulative weight 0.04 + 0.06 = 0.1 <= 0.1*sum
    n, te, dc = O.truncate_cpu(P, cutoff=0.1)
    assert n == 3 and te == pytest.approx(0.1)
    n, te, _ = O.truncate_cpu(P, maxdim=2)
    assert n == 2 and te == pytest.approx(0.2)
    n, te, _ = O.truncate_cpu(P, cutoff=0.05, absoluteCutoff=True)
    assert n == 4 and te == pytest.approx(0.04)
    n, te, _ = O.truncate_cpu(P, cutoff=1.0, mindim=2)
    assert n == 2
    n, te, dc = O.truncate_cpu([2.0])
    assert (n, te, dc) == (1, 0.0, 1.0)


def test_philox_stream_is_fixed():
    x = O.philox_normal(8, seed=1234, offset=0)
    y = O.philox_normal(9, seed=1234, offset=0)
    assert np.array_equal(x, y[:8])
    z = O.philox_normal(8, seed=1234, offset=1)
    assert not np.allclose(x, z)
    big = O.philox_normal(200000, seed=7)
    assert abs(big.mean()) < 0.01 and abs(big.std() - 1) < 0.01


@pytest.mark.parametrize("N", [6, 8])
def test_oracle_mpo_matches_ed(N):
    Ws = O.heisenberg_mpo(N)
    H = O.mpo_matrix(Ws)
    e0 = np.linalg.eigvalsh(H)[0]
    assert e0 == pytest.approx(GOLD["ed"].get(f"heisenberg_N{N}", O.heisenberg_ed_sz0(N)), abs=1e-10)
    assert max(w.shape[3] for w in Ws[:-1]) == 5


def test_oracle_heff_matches_dense_matrix():
    rng = np.random.default_rng(0)
    chi, d, w = 3, 2, 5
    L = rng.standard_normal((chi, w, chi))
    R = rng.standard_normal((chi, w, chi))
    W1 = rng.standard_normal((w, d, d, w))
    W2 = rng.standard_normal((w, d, d, w))
    psi = rng.standard_normal((chi, d, d, chi))
    H = np.einsum("awc,wtsx,xvuy,byd->ctvdasub", L, W1, W2, R).reshape(chi * d * d * chi, -1, order="F")
    # F-order flattening on both sides: rows (c,t,v,d), cols (a,s,u,b)
    Hm = np.einsum("awc,wtsx,xvuy,byd->ctvdasub", L, W1, W2, R)
    out = O.heff_apply(L, W1, W2, R, psi)
    ref = np.einsum("ctvdasub,asub->ctvd", Hm, psi)
    assert np.allclose(out, ref, rtol=1e-12, atol=1e-12)
    dg = O.heff_diag(L, W1, W2, R)
    assert np.allclose(dg, np.einsum("ctvdctvd->ctvd", Hm))
    del H


def test_oracle_davidson_finds_lowest():
    rng = np.random.default_rng(1)
    n = 60
    A = rng.standard_normal((n, n))
    A = A + A.T
    w = np.linalg.eigvalsh(A)
    theta, x, nmv = O.davidson(lambda v: A @ v, rng.standard_normal(n), np.diag(A).copy(),
                               krylovdim=20, maxiter=40, tol=1e-10)
    assert theta == pytest.approx(w[0], abs=1e-8)
    assert np.linalg.norm(A @ x - theta * x) < 1e-8


@pytest.mark.slow
def test_oracle_dmrg_heisenberg_n12_vs_ed():
    N = 12
    Ws = O.heisenberg_mpo(N)
    A = O.random_mps([2] * N, 10, seed=1234)
    e, _ = O.dmrg(Ws, A, [10, 20, 50, 100], [1e-14], 6)
    assert e == pytest.approx(GOLD["ed"]["heisenberg_N12"], abs=1e-10)


@pytest.mark.slow
def test_oracle_dmrg_tfim_closed_form():
    g = GOLD["dmrg"]["tfim"]
    N = g["N"]
    Ws = O.tfim_mpo(N, h=g["h"], J=g["J"])
    A = O.random_mps([2] * N, 1, seed=g["seed"])
    e, _ = O.dmrg(Ws, A, g["maxdim"], [g["cutoff"]], g["nsweep"])
    exact = O.tfim_closed_form(N)
    assert abs((e - exact) / exact) < g["rel_tol"]
    assert abs(e - exact) < 1e-6  # much tighter than the reference's 1e-2


@pytest.mark.slow
def test_oracle_dmrg_spin1_bound():
    g = GOLD["dmrg"]["spin1_heisenberg"]
    N = g["N"]
    Ws = O.heisenberg_mpo(N, d=3)
    A = O.random_mps([3] * N, 1, seed=11)
    e, _ = O.dmrg(Ws, A, g["maxdim"], [g["cutoff"]], g["nsweep"])
    assert e < g["energy_below"]


@pytest.mark.slow
def test_oracle_dmrg_noise_path_vs_ed():
    """The density-matrix (noise > 0) bond split reaches the same ground state,
    and the spin-1 known answer holds with the reference's noise 1e-10."""
    N = 10
    e, _ = O.dmrg(O.heisenberg_mpo(N), O.random_mps([2] * N, 4, 7), [10, 20, 40, 64], [1e-12], 5,
                  noises=[1e-5, 1e-7, 1e-9, 0.0])
    assert e == pytest.approx(O.heisenberg_ed_sz0(N), abs=1e-9)
    g = GOLD["dmrg"]["spin1_heisenberg"]
    e, _ = O.dmrg(O.heisenberg_mpo(g["N"], d=3), O.random_mps([3] * g["N"], 1, seed=11), g["maxdim"],
                  [g["cutoff"]], g["nsweep"], noises=[1e-10])
    assert e < g["energy_below"]
