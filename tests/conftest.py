"""Shared test setup: import paths, the `gpu` marker, device fixtures."""
import os
import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parent.parent
PKG = REPO / "itensorsgpu.jl_gb300"
for p in (str(REPO), str(PKG)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU and the built libitg.so")
    config.addinivalue_line("markers", "slow: long-running CPU oracle case")


def _cuda_ok():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def itg_lib():
    """Built libitg.so (compiled on demand); fails loudly if the build fails."""
    from itg import build
    build.build()
    from itg import _lib
    return _lib.load_library()


@pytest.fixture(scope="session")
def gpu(itg_lib):
    if not _cuda_ok():
        pytest.fail("GPU test collected on a machine without CUDA (run with -m 'not gpu')")
    import itg
    return itg


def mpo_dense_matrix(H):
    """Full matrix of a small host MPO (site 0 the slowest index), through the
    oracle's contraction of its W tensors."""
    import itg
    from oracle import itg_oracle as O
    return O.mpo_matrix([t.array() for t in itg.cpu(H).tensors])
