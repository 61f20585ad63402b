"""Host-side MPO construction and sweep schedule (no GPU): the MPOs the DMRG
path runs on equal the Hamiltonians built directly from spin operators."""
import numpy as np
import pytest
from conftest import mpo_dense_matrix


def _ops(d):
    s = (d - 1) / 2
    m = np.arange(s, -s - 1, -1)
    sz = np.diag(m)
    sp = np.zeros((d, d))
    for i in range(1, d):
        sp[i - 1, i] = np.sqrt(s * (s + 1) - m[i] * (m[i] + 1))
    sx = (sp + sp.T) / 2
    sy_im = (sp - sp.T) / 2  # Sy = -i (S+ - S-)/2; Sy Sy is real: -(S+ - S-)^2 / 4
    return sx, sy_im, sz


def _site_op(op, i, N, d):
    out = np.ones((1, 1))
    for j in range(N):
        out = np.kron(out, op if j == i else np.eye(d))
    return out


def _bond(a, b, i, j, N, d):
    return _site_op(a, i, N, d) @ _site_op(b, j, N, d)


def _heis_like(N, d, J, D):
    sx, syi, sz = _ops(d)
    H = np.zeros((d ** N, d ** N))
    for i in range(N - 1):
        # Sx Sx + Sy Sy = Sx Sx - (syi x syi) (syi = i Sy up to sign)
        H += J[i] * (_bond(sx, sx, i, i + 1, N, d) - _bond(syi, syi, i, i + 1, N, d)
                     + D[i] * _bond(sz, sz, i, i + 1, N, d))
    return H


def _dense(H):
    # site 0 is the slowest index of the dense matrix, as in the Kronecker products
    import itg
    return mpo_dense_matrix(H)


@pytest.mark.parametrize("d", [2, 3])
def test_heisenberg_mpo_matches_operator_sum(d):
    import itg
    N = 5
    sites = itg.siteinds("S=1/2" if d == 2 else "S=1", N)
    M = _dense(itg.heisenberg_mpo(sites))
    ref = _heis_like(N, d, np.ones(N - 1), np.ones(N - 1))
    assert np.allclose(M, ref, atol=1e-12)


def test_xxz_per_bond_couplings():
    import itg
    N = 6
    rng = np.random.default_rng(3)
    J, D = rng.uniform(0.5, 1.5, N - 1), rng.uniform(0.5, 1.5, N - 1)
    sites = itg.siteinds("S=1/2", N)
    M = _dense(itg.xxz_mpo(sites, J=J, Delta=D))
    ref = _heis_like(N, 2, J, D)
    assert np.allclose(M, ref, atol=1e-12)


def test_j1j2_and_tfim_mpos():
    import itg
    N = 6
    sites = itg.siteinds("S=1/2", N)
    sx, syi, sz = _ops(2)
    J2 = 0.37
    ref = _heis_like(N, 2, np.ones(N - 1), np.ones(N - 1))
    for i in range(N - 2):
        ref += J2 * (_bond(sx, sx, i, i + 2, N, 2) - _bond(syi, syi, i, i + 2, N, 2) + _bond(sz, sz, i, i + 2, N, 2))
    M = _dense(itg.j1j2_mpo(sites, J1=1.0, J2=J2))
    assert np.allclose(M, ref, atol=1e-12)
    h = 0.5
    ref = np.zeros((2 ** N, 2 ** N))
    for i in range(N - 1):
        ref -= _bond(sz, sz, i, i + 1, N, 2)
    for i in range(N):
        ref -= h * _site_op(sx, i, N, 2)
    M = _dense(itg.tfim_mpo(sites, h=h, J=1.0))
    assert np.allclose(M, ref, atol=1e-12)


def test_sweepnext_order():
    import itg
    N = 5
    seq = list(itg.sweepnext(N))
    assert seq == [(b, 1) for b in range(N - 1)] + [(b, 2) for b in range(N - 2, -1, -1)]


def test_sweeps_schedule_repeats_last_value():
    import itg
    sw = itg.Sweeps(5, maxdim=[10, 20], cutoff=[1e-8, 1e-10], mindim=[1])
    assert [sw.maxdim(i) for i in range(5)] == [10, 20, 20, 20, 20]
    assert [sw.cutoff(i) for i in range(5)] == [1e-8, 1e-10, 1e-10, 1e-10, 1e-10]
