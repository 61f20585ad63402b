"""ctypes binding of libitg.so (the C ABI declared in include/itg.h).

This is the same binding a Julia ``ccall`` layer makes: plain device pointers,
int64 dimensions, int32 mode labels, int status codes.  A non-zero status is
raised as an exception that mirrors the reference's error behaviour:
ITG_ERR_SHAPE -> ``DimensionMismatch`` (the Julia exception the reference
throws, e.g. src/cuitensor.jl:55), anything else -> ``ITGError``.

There is no CPU fallback: if libitg.so is missing or no GPU is present, the
first call raises.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent.parent / "libitg.so"

ITG_OK, ITG_ERR_INVALID, ITG_ERR_SHAPE, ITG_ERR_ALLOC, ITG_ERR_CUDA = 0, 1, 2, 3, 4
ITG_ERR_TIMEOUT, ITG_ERR_NOTCONVERGED, ITG_ERR_UNSUPPORTED = 5, 6, 7
ITG_F64 = 0
ITG_C64 = 1
PREC_FP64, PREC_SPLIT = 0, 1
KERNEL_GEMM_F64, KERNEL_GEMM_SPLIT, KERNEL_SPLIT_PREP, KERNEL_HEFF_MID = 0, 1, 2, 3
SVD_AUTO, SVD_JACOBI, SVD_MIXED = 0, 1, 2


class ITGError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{msg} (status {status})")
        self.status = status


class DimensionMismatch(ITGError):
    """Raised where the reference raises Julia's DimensionMismatch."""


class NotConverged(ITGError):
    pass


_P = C.c_void_p
_I64P = C.POINTER(C.c_int64)
_I32P = C.POINTER(C.c_int32)
_DP = C.POINTER(C.c_double)

# name -> (restype, argtypes)
SIGNATURES = {
    "itg_create": (C.c_int, [C.c_int, C.POINTER(_P)]),
    "itg_destroy": (C.c_int, [_P]),
    "itg_set_stream": (C.c_int, [_P, _P]),
    "itg_get_stream": (C.c_int, [_P, C.POINTER(_P)]),
    "itg_synchronize": (C.c_int, [_P]),
    "itg_workspace_info": (C.c_int, [_P, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t), C.POINTER(C.c_size_t),
                                     _I64P]),
    "itg_set_graphs": (C.c_int, [_P, C.c_int]),
    "itg_last_error": (C.c_char_p, [_P]),
    "itg_status_string": (C.c_char_p, [C.c_int]),
    "itg_version": (C.c_int, []),
    "itg_profile": (C.c_int, [_P, C.c_int]),
    "itg_profile_read": (C.c_int, [_P, C.c_int, _DP, _I64P]),
    "itg_fp64_peak": (C.c_int, [_P, _DP]),
    "itg_malloc": (C.c_int, [_P, C.POINTER(_P), C.c_size_t]),
    "itg_free": (C.c_int, [_P, _P]),
    "itg_memcpy_h2d": (C.c_int, [_P, _P, _P, C.c_size_t]),
    "itg_memcpy_d2h": (C.c_int, [_P, _P, _P, C.c_size_t]),
    "itg_memcpy_d2d": (C.c_int, [_P, _P, _P, C.c_size_t]),
    "itg_memset_zero": (C.c_int, [_P, _P, C.c_size_t]),
    "itg_contract": (C.c_int, [_P, C.c_int, C.c_double,
                               _P, C.c_int, _I64P, _I32P,
                               _P, C.c_int, _I64P, _I32P,
                               C.c_double,
                               _P, C.c_int, _I64P, _I32P, C.c_int]),
    "itg_split_error_bound": (C.c_double, [C.c_int64]),
    "itg_set_wait_limit_ns": (C.c_int, [_P, C.c_uint64]),
    "itg_wait_selftest": (C.c_int, [_P, C.c_int]),
    "itg_split_partition": (C.c_int, [C.c_int64, C.c_int, C.c_int, _I32P, C.c_int, C.POINTER(C.c_int)]),
    "itg_contract_z": (C.c_int, [_P, C.c_int, C.c_int, _DP,
                                 _P, C.c_int, _I64P, _I32P,
                                 _P, C.c_int, _I64P, _I32P,
                                 _DP,
                                 _P, C.c_int, _I64P, _I32P, C.c_int]),
    "itg_conj": (C.c_int, [_P, C.c_int64, _P, _P]),
    "itg_svd_trunc_z": (C.c_int, [_P, C.c_int64, C.c_int64, _P, C.c_int64, C.c_int64, C.c_int64,
                                  C.c_double, C.c_int, C.c_int, C.c_int, _P, _P, _P, _I64P, _DP, _DP]),
    "itg_qr_z": (C.c_int, [_P, C.c_int64, C.c_int64, _P, C.c_int64, _P, _P]),
    "itg_eigh_trunc_z": (C.c_int, [_P, C.c_int64, _P, C.c_int64, C.c_int64, C.c_int64, C.c_double, C.c_int,
                                   C.c_int, C.c_int, _P, _P, _I64P, _DP, _DP]),
    "itg_real_to_complex": (C.c_int, [_P, C.c_int64, _P, _P]),
    "itg_zscal": (C.c_int, [_P, C.c_int64, _DP, _P]),
    "itg_permute": (C.c_int, [_P, C.c_int, C.c_double, _P, C.c_int, _I64P, _I32P, _P, _I32P]),
    "itg_axpby_permuted": (C.c_int, [_P, C.c_int, C.c_double, _P, C.c_int, _I64P, _I32P,
                                     C.c_double, _P, _I32P, _P]),
    "itg_diag_contract": (C.c_int, [_P, C.c_int, C.c_double, _P, C.c_int, C.c_int, _I64P, _I32P,
                                    _P, C.c_int, _I64P, _I32P, C.c_double,
                                    _P, C.c_int, _I64P, _I32P]),
    "itg_diag_diag": (C.c_int, [_P, C.c_int64, C.c_double, _P, C.c_int, _P, C.c_int, _P]),
    "itg_diag_to_dense": (C.c_int, [_P, _P, C.c_int, C.c_int, _I64P, _P]),
    "itg_scal": (C.c_int, [_P, C.c_int64, C.c_double, _P]),
    "itg_axpy": (C.c_int, [_P, C.c_int64, C.c_double, _P, _P]),
    "itg_axpby": (C.c_int, [_P, C.c_int64, C.c_double, _P, C.c_double, _P]),
    "itg_fill": (C.c_int, [_P, C.c_int64, C.c_double, _P]),
    "itg_dot": (C.c_int, [_P, C.c_int64, _P, _P, _DP]),
    "itg_nrm2": (C.c_int, [_P, C.c_int64, _P, _DP]),
    "itg_dot_dev": (C.c_int, [_P, C.c_int64, _P, _P, _P]),
    "itg_gemv_t": (C.c_int, [_P, C.c_int64, C.c_int64, _P, C.c_int64, _P, _P]),
    "itg_gemv_n": (C.c_int, [_P, C.c_int64, C.c_int64, _P, C.c_int64, _P, C.c_double, _P]),
    "itg_random_normal": (C.c_int, [_P, C.c_int64, C.c_uint64, C.c_uint64, _P]),
    "itg_truncate": (C.c_int, [_P, _P, C.c_int64, C.c_int64, C.c_int64, C.c_double,
                               C.c_int, C.c_int, C.c_int, _I64P, _DP, _DP]),
    "itg_svd_trunc": (C.c_int, [_P, C.c_int64, C.c_int64, _P, C.c_int64,
                                C.c_int64, C.c_int64, C.c_double, C.c_int, C.c_int, C.c_int,
                                _P, _P, _P, _I64P, _DP, _DP]),
    "itg_svd_trunc_ex": (C.c_int, [_P, C.c_int64, C.c_int64, _P, C.c_int64,
                                   C.c_int64, C.c_int64, C.c_double, C.c_int, C.c_int, C.c_int,
                                   _P, _P, _P, _I64P, _DP, _DP, C.c_int, C.c_int]),
    "itg_eigh_trunc": (C.c_int, [_P, C.c_int64, _P, C.c_int64,
                                 C.c_int64, C.c_int64, C.c_double, C.c_int, C.c_int, C.c_int,
                                 _P, _P, _I64P, _DP, _DP]),
    "itg_qr": (C.c_int, [_P, C.c_int64, C.c_int64, _P, C.c_int64, _P, _P]),
    "itg_matmul": (C.c_int, [_P, C.c_int64, C.c_int64, C.c_int64, _P, _P, _P, C.c_int]),
    "itg_set_autotune": (C.c_int, [_P, C.c_int]),
    "itg_autotune_info": (C.c_int, [_P, _I64P, _I64P]),
    "itg_autotune_clear": (C.c_int, [_P]),
    "itg_autotune_query": (C.c_int, [_P, C.c_int, _I64P, _I32P, C.c_int, _I64P, _I32P, C.c_int, _I64P, _I32P,
                                     C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "itg_autotune_force": (C.c_int, [_P, C.c_int, _I64P, _I32P, C.c_int, _I64P, _I32P, C.c_int, _I64P, _I32P,
                                     C.c_int, C.c_int]),
    "itg_svd_info": (C.c_int, [_P, C.POINTER(C.c_int), C.POINTER(C.c_int), _I64P]),
    "itg_factorize_trunc": (C.c_int, [_P, C.c_int64, C.c_int64, _P, C.c_int64, C.c_int64, C.c_int64, C.c_double,
                                      C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _P, _P, _P, _I64P,
                                      C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "itg_set_svd_options": (C.c_int, [_P, C.c_int, C.c_int]),
    "itg_mlp_create": (C.c_int, [_P, C.c_int, C.c_uint64, C.POINTER(_P)]),
    "itg_mlp_destroy": (C.c_int, [_P, _P]),
    "itg_mlp_num_params": (C.c_int, [_P, _I64P]),
    "itg_mlp_get_params": (C.c_int, [_P, _P, _P]),
    "itg_mlp_set_params": (C.c_int, [_P, _P, _P]),
    "itg_mlp_forward": (C.c_int, [_P, _P, C.c_int64, _P, _P]),
    "itg_mlp_train_step": (C.c_int, [_P, _P, C.c_int64, _P, _P, _P, C.c_float, _P, C.POINTER(C.c_float)]),
    "itg_heff2_features": (C.c_int, [_P, C.c_int64, C.c_int64, C.c_int64, _P, _P, C.c_double, _P, _P, _P,
                                     _P]),
    "itg_davidson_heff2_learned": (C.c_int, [_P, C.c_int64, C.c_int64, C.c_int64, C.c_int64, C.c_int64,
                                             C.c_int64, _P, _P, _P, _P, _P, C.c_int, C.c_int, C.c_double,
                                             C.c_int, _P, _P, _P, _DP, C.POINTER(C.c_int),
                                             C.POINTER(C.c_int)]),
    "itg_contract_grouped": (C.c_int, [_P, C.c_int, C.c_double, _P, C.c_int, _I64P, _I32P,
                                       _P, C.c_int, _I64P, _I32P, C.c_double, _P, C.c_int, _I64P, _I32P]),
    "itg_svd_trunc_batched": (C.c_int, [_P, C.c_int, _I64P, _I64P, _P, _I64P, C.c_int64, C.c_double,
                                        C.c_int, C.c_int, C.c_int, _P, _P, _P, _I64P, _DP]),
    "itg_davidson_heff2_batched": (C.c_int, [_P, C.c_int, _I64P, _I64P, C.c_int64, C.c_int64, C.c_int64,
                                             C.c_int64, _P, _P, _P, _P, _P, C.c_int, C.c_int, C.c_double,
                                             _DP, C.POINTER(C.c_int)]),
    "itg_heff2_apply": (C.c_int, [_P, C.c_int64, C.c_int64, C.c_int64, C.c_int64, C.c_int64,
                                  C.c_int64, _P, _P, _P, _P, _P, _P, C.c_int]),
    "itg_heff2_apply_noalloc": (C.c_int, [_P, C.c_int64, C.c_int64, C.c_int64, C.c_int64,
                                          C.c_int64, C.c_int64, _P, _P, _P, _P, _P, _P]),
    "itg_heff2_diag": (C.c_int, [_P, C.c_int64, C.c_int64, C.c_int64, C.c_int64, C.c_int64,
                                 C.c_int64, _P, _P, _P, _P, _P]),
    "itg_davidson_heff2": (C.c_int, [_P, C.c_int64, C.c_int64, C.c_int64, C.c_int64, C.c_int64,
                                     C.c_int64, _P, _P, _P, _P, _P, C.c_int, C.c_int,
                                     C.c_double, C.c_int, _DP, C.POINTER(C.c_int)]),
}

_lib = None
_lib_lock = threading.Lock()


def load_library(path: Path | None = None) -> C.CDLL:
    """Load libitg.so and attach signatures.  Raises if it was not built."""
    global _lib
    with _lib_lock:
        if _lib is not None:
            return _lib
        p = Path(path) if path else LIB_PATH
        if not p.exists():
            raise ImportError(
                f"{p} is missing: build the CUDA library first "
                "(python -c 'import __graft_entry__ as g; g.build()')")
        lib = C.CDLL(str(p))
        for name, (res, args) in SIGNATURES.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
        return lib


def i64arr(vals):
    a = (C.c_int64 * max(1, len(vals)))(*[int(v) for v in vals])
    return a


def i32arr(vals):
    a = (C.c_int32 * max(1, len(vals)))(*[int(v) for v in vals])
    return a


class Handle:
    """Owns one itg_handle on one device (the library's per-thread context)."""

    def __init__(self, device: int = 0):
        self.lib = load_library()
        h = C.c_void_p()
        st = self.lib.itg_create(int(device), C.byref(h))
        if st != ITG_OK:
            raise ITGError(st, f"itg_create({device}) failed: "
                               f"{self.lib.itg_status_string(st).decode()} (is a GPU present?)")
        self.ptr = h
        self.device = device

    def check(self, st: int, what: str = ""):
        if st == ITG_OK:
            return
        msg = self.lib.itg_last_error(self.ptr).decode(errors="replace")
        name = self.lib.itg_status_string(st).decode()
        text = f"{what}: {name}: {msg}"
        if st == ITG_ERR_SHAPE:
            raise DimensionMismatch(st, text)
        if st == ITG_ERR_NOTCONVERGED:
            raise NotConverged(st, text)
        raise ITGError(st, text)

    def call(self, name: str, *args):
        st = getattr(self.lib, name)(self.ptr, *args)
        self.check(st, name)

    def close(self):
        if getattr(self, "ptr", None):
            self.lib.itg_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_handles: dict[tuple[int, int], Handle] = {}


def handle(device: int = 0) -> Handle:
    """Per-thread, per-device handle (handles are not thread-safe)."""
    key = (threading.get_ident(), device)
    h = _handles.get(key)
    if h is None:
        h = Handle(device)
        _handles[key] = h
    return h


def f64_host_ptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"] or a.flags["F_CONTIGUOUS"]
    return C.c_void_p(a.ctypes.data)
