"""Failure detection on the GPU without a GPU fault.

Every device-side wait of the library is bounded by the handle's wait limit
(itg_set_wait_limit_ns).  Here a short limit is set and the wait self-tests
run the library's own waiting code on a wait that can never be satisfied (a
grid barrier counting one participant that never arrives; an mbarrier nobody
arrives on).  Each must come back with ITG_ERR_TIMEOUT after about the limit,
and the same handle must then run ordinary FP64 and split-precision
contractions correctly: the context stays usable.  The reference's only
failure handling on this path is the skip-and-warn around its cuTENSOR calls
(src/tensor/cudense.jl:321-323).
"""
import ctypes as C
import time

import numpy as np
import pytest

from oracle import itg_oracle as O

pytestmark = pytest.mark.gpu

LIMIT_NS = 50_000_000  # 50 ms


@pytest.mark.parametrize("which", [0, 1], ids=["grid_barrier", "mbarrier"])
def test_bounded_wait_runs_out_and_handle_stays_usable(gpu, which):
    import torch
    from itg import _lib
    h = _lib.Handle(0)
    try:
        h.call("itg_set_wait_limit_ns", C.c_uint64(LIMIT_NS))
        t0 = time.perf_counter()
        with pytest.raises(_lib.ITGError) as ei:
            h.call("itg_wait_selftest", which)
        dt = time.perf_counter() - t0
        assert ei.value.status == _lib.ITG_ERR_TIMEOUT, str(ei.value)
        assert "ran out" in str(ei.value)
        assert LIMIT_NS * 1e-9 * 0.9 <= dt < 10.0, dt
        h.call("itg_set_wait_limit_ns", C.c_uint64(4_000_000_000))
        # the same handle still computes: FP64 and split contractions vs the oracle
        rng = np.random.default_rng(11 + which)
        A = rng.standard_normal((300, 200))
        B = rng.standard_normal((200, 260))
        ref = A @ B
        p = lambda t: C.c_void_p(t.data_ptr())
        Ad = torch.from_numpy(O.flat(A).copy()).cuda()
        Bd = torch.from_numpy(O.flat(B).copy()).cuda()
        for prec in (0, 1):
            Cd = torch.full((300 * 260,), float("nan"), dtype=torch.float64, device="cuda")
            h.call("itg_contract", 0, C.c_double(1.0), p(Ad), 2, _lib.i64arr([300, 200]), _lib.i32arr([1, 2]),
                   p(Bd), 2, _lib.i64arr([200, 260]), _lib.i32arr([2, 3]), C.c_double(0.0), p(Cd), 2,
                   _lib.i64arr([300, 260]), _lib.i32arr([1, 3]), prec)
            h.call("itg_synchronize")
            got = O.unflat(Cd.cpu().numpy(), (300, 260))
            assert np.linalg.norm(got - ref) <= 1e-12 * np.linalg.norm(ref), prec
    finally:
        h.close()


def test_wait_limit_rejects_out_of_range(gpu):
    from itg import _lib
    h = _lib.handle(0)
    for bad in (0, 999, 61_000_000_000):
        with pytest.raises(_lib.ITGError) as ei:
            h.call("itg_set_wait_limit_ns", C.c_uint64(bad))
        assert ei.value.status == _lib.ITG_ERR_INVALID
    with pytest.raises(_lib.ITGError):
        h.call("itg_wait_selftest", 7)
