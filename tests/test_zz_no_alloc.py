"""itg_heff2_apply_noalloc: the H_eff matvec for callers that cannot let the
library allocate device memory (their memory comes from their own fixed pool,
or they cannot accept the synchronisation a cudaMalloc may cause).

Checks, through the C ABI, that two calls in a row give the same result as the
allocating entry point itg_heff2_apply (relative Frobenius difference <= 1e-12,
the FP64 contraction tolerance of the other tests), that a stale result from
the shared scratch array cannot leak into the next call, that a first call on a
fresh handle with autotuning on leaves every library workspace of the handle
unallocated, and that a problem larger than the fixed scratch array (also one
whose sizes would overflow 64-bit products) is refused with a clear error.
This file is collected last so that a failure here does not hide any other
test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def _inputs(chiL, chiR, d, w, seed):
    import torch
    g = torch.Generator(device="cpu").manual_seed(seed)
    mk = lambda *s: torch.randn(int(np.prod(s)), generator=g, dtype=torch.float64).cuda()
    return (mk(chiL, w, chiL), mk(w, d, d, w), mk(w, d, d, w), mk(chiR, w, chiR), mk(chiL, d, d, chiR))


def _apply(h, name, dims, tensors, out):
    chiL, chiR, d, w = dims
    p = lambda t: C.c_void_p(t.data_ptr())
    L, W1, W2, R, psi = tensors
    args = [C.c_int64(chiL), C.c_int64(chiR), C.c_int64(d), C.c_int64(w), C.c_int64(w), C.c_int64(w),
            p(L), p(W1), p(W2), p(R), p(psi), p(out)]
    if name == "itg_heff2_apply":
        args.append(0)
    h.call(name, *args)


@pytest.mark.parametrize("dims", [(16, 16, 2, 5), (96, 80, 2, 5), (33, 47, 3, 4)])
def test_noalloc_matches_allocating_entry_point_twice(gpu, dims):
    import torch
    from itg import _lib
    h = _lib.handle(0)
    chiL, chiR, d, w = dims
    for call, seed in enumerate((101, 202)):  # two calls in a row, different inputs
        ins = _inputs(chiL, chiR, d, w, seed + chiL)
        ref = torch.empty(chiL * d * d * chiR, dtype=torch.float64, device="cuda")
        got = torch.full_like(ref, float("nan"))
        _apply(h, "itg_heff2_apply", dims, ins, ref)
        _apply(h, "itg_heff2_apply_noalloc", dims, ins, got)
        torch.cuda.synchronize()
        err = (torch.linalg.norm(got - ref) / torch.linalg.norm(ref)).item()
        assert err <= RTOL, (call, err)


def test_noalloc_rejects_oversized_problem(gpu):
    import torch
    from itg import _lib
    h = _lib.handle(0)
    chi, d, w = 1024, 2, 5  # needs ~42 Mi doubles, the array holds 4 Mi
    small = torch.zeros(8, dtype=torch.float64, device="cuda")
    p = C.c_void_p(small.data_ptr())
    out = torch.zeros(8, dtype=torch.float64, device="cuda")
    with pytest.raises(_lib.ITGError) as ei:
        h.call("itg_heff2_apply_noalloc", C.c_int64(chi), C.c_int64(chi), C.c_int64(d), C.c_int64(w),
               C.c_int64(w), C.c_int64(w), p, p, p, p, p, C.c_void_p(out.data_ptr()))
    assert ei.value.status == _lib.ITG_ERR_UNSUPPORTED
    assert "no-allocation" in str(ei.value)


def _workspace(h):
    sc, sp, tu, pl = C.c_size_t(), C.c_size_t(), C.c_size_t(), C.c_int64()
    h.call("itg_workspace_info", C.byref(sc), C.byref(sp), C.byref(tu), C.byref(pl))
    return sc.value, sp.value, tu.value, pl.value


def test_noalloc_first_call_on_fresh_handle_allocates_nothing(gpu, monkeypatch):
    import torch
    from itg import _lib
    monkeypatch.setenv("ITG_AUTOTUNE", "1")
    dims = (64, 48, 2, 5)
    chiL, chiR, d, w = dims
    h = _lib.Handle(0)  # fresh handle: no workspace yet
    try:
        h.call("itg_set_autotune", 1)
        assert _workspace(h) == (0, 0, 0, 0)
        ins = _inputs(chiL, chiR, d, w, 7)
        got = torch.full((chiL * d * d * chiR,), float("nan"), dtype=torch.float64, device="cuda")
        _apply(h, "itg_heff2_apply_noalloc", dims, ins, got)
        torch.cuda.synchronize()
        assert _workspace(h) == (0, 0, 0, 0)
        # the allocating entry point on another handle gives the same numbers
        ref = torch.empty_like(got)
        _apply(_lib.handle(0), "itg_heff2_apply", dims, ins, ref)
        torch.cuda.synchronize()
        err = (torch.linalg.norm(got - ref) / torch.linalg.norm(ref)).item()
        assert err <= RTOL, err
    finally:
        h.close()


def test_noalloc_rejects_sizes_whose_products_overflow(gpu):
    import torch
    from itg import _lib
    h = _lib.handle(0)
    small = torch.zeros(8, dtype=torch.float64, device="cuda")
    p = C.c_void_p(small.data_ptr())
    out = torch.zeros(8, dtype=torch.float64, device="cuda")
    big = 1 << 40  # chiL * chiR * 20 wraps a signed 64-bit product
    for chiL, chiR, d in ((big, big, 2), (1, 1, 1 << 33), (big, 1, 2)):
        with pytest.raises(_lib.ITGError) as ei:
            h.call("itg_heff2_apply_noalloc", C.c_int64(chiL), C.c_int64(chiR), C.c_int64(d), C.c_int64(5),
                   C.c_int64(5), C.c_int64(5), p, p, p, p, p, C.c_void_p(out.data_ptr()))
        assert ei.value.status == _lib.ITG_ERR_UNSUPPORTED
        assert "no-allocation" in str(ei.value)
    assert torch.count_nonzero(out).item() == 0
