"""C-ABI library and host-logic tests that need no GPU.

* libitg.so builds for sm_103a, loads, and exports every symbol include/itg.h
  declares; the ctypes signature table covers exactly those symbols.
* Host-side logic: MPO builders against the oracle's independent MPOs and ED,
  Sweeps schedule, sweepnext order, product-state construction, errors that
  need no device (ITensor host containers, missing GPU surfaces loudly).
"""
import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

from oracle import itg_oracle as O
from conftest import mpo_dense_matrix

REPO = Path(__file__).resolve().parent.parent
HEADER = REPO / "include" / "itg.h"


def header_symbols():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"ITG_API\s+(?:const\s+char\s*\*|int|double)\s+(itg_\w+)\s*\(", text)))


def test_header_declares_symbols():
    syms = header_symbols()
    assert "itg_contract" in syms and "itg_svd_trunc" in syms and len(syms) >= 30


def test_library_exports_every_header_symbol(itg_lib):
    missing = [s for s in header_symbols() if not hasattr(itg_lib, s)]
    assert not missing, missing


def test_ctypes_table_matches_header():
    from itg import _lib
    assert sorted(_lib.SIGNATURES) == header_symbols()


def test_status_strings_and_version(itg_lib):
    itg_lib.itg_status_string.restype = ctypes.c_char_p
    assert itg_lib.itg_status_string(2) == b"ITG_ERR_SHAPE"
    assert itg_lib.itg_version() >= 10000


def test_split_error_bound_is_host_only(itg_lib):
    f = itg_lib.itg_split_error_bound
    f.restype = ctypes.c_double
    f.argtypes = [ctypes.c_int64]
    b = f(1024)
    assert 0.0 <= b < 1e-10


def test_create_without_gpu_fails_cleanly(itg_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    h = ctypes.c_void_p()
    st = itg_lib.itg_create(0, ctypes.byref(h))
    assert st != 0 and not h.value


@pytest.mark.parametrize("N,d", [(6, 2), (5, 3)])
def test_product_heisenberg_mpo_matches_oracle(N, d):
    import itg
    sites = itg.siteinds("S=1/2" if d == 2 else "S=1", N)
    H = itg.heisenberg_mpo(sites)
    M = mpo_dense_matrix(H)
    Mo = O.mpo_matrix(O.heisenberg_mpo(N, d=d))
    assert np.allclose(M, Mo, atol=1e-14)
    assert max(t.dims[3] for t in H.tensors[:-1]) == 5


def test_product_tfim_and_j1j2_mpos_match_oracle():
    import itg
    sites = itg.siteinds("S=1/2", 6)
    assert np.allclose(mpo_dense_matrix(itg.tfim_mpo(sites, h=0.5)),
                       O.mpo_matrix(O.tfim_mpo(6, h=0.5)), atol=1e-14)
    Hj = itg.j1j2_mpo(sites, J1=1.0, J2=0.3)
    assert np.allclose(mpo_dense_matrix(Hj), O.mpo_matrix(O.heisenberg_mpo(6, J2=0.3)), atol=1e-14)
    assert max(t.dims[3] for t in Hj.tensors[:-1]) == 8


def test_xxz_per_bond_couplings():
    import itg
    rng = np.random.default_rng(3)
    J = rng.uniform(0.5, 1.5, 5)
    D = rng.uniform(0.5, 1.5, 5)
    sites = itg.siteinds("S=1/2", 6)
    M = mpo_dense_matrix(itg.xxz_mpo(sites, J=J, Delta=D))
    assert np.allclose(M, O.mpo_matrix(O.heisenberg_mpo(6, J=J, Delta=D)), atol=1e-14)


def test_sweeps_schedule_and_order():
    import itg
    sw = itg.Sweeps(5, maxdim=[10, 20, 50, 100, 100], cutoff=[1e-10])
    assert [sw.maxdim(i) for i in range(5)] == [10, 20, 50, 100, 100]
    assert sw.cutoff(4) == 1e-10 and sw.mindim(0) == 1
    itg.maxdim_(sw, 10, 20)
    assert sw.maxdim(3) == 20
    assert list(itg.sweepnext(4)) == [(0, 1), (1, 1), (2, 1), (2, 2), (1, 2), (0, 2)]


def test_product_state_host():
    import itg
    sites = itg.siteinds("S=1/2", 4)
    psi = itg.productMPS_host(sites, ["Up", "Dn", "Up", "Dn"])
    assert psi[1].array()[0, 1, 0] == 1.0 and psi[1].array().sum() == 1.0
    psi3 = itg.productMPS_host(itg.siteinds("S=1", 3), lambda j: j)
    assert psi3[2].array()[0, 2, 0] == 1.0


def test_host_itensor_needs_cu():
    import itg
    i, j = itg.Index(2), itg.Index(3)
    A = itg.ITensor_host(np.ones((2, 3)), i, j)
    with pytest.raises(TypeError):
        _ = A * A
    with pytest.raises(itg.DimensionMismatch):
        itg.ITensor_host(np.ones((3, 2)), i, j)
