"""ITensor-level mirror of ITensorsGPU.jl's storage plugin, on libitg.so.

Mirrors the reference's user-facing surface for dense real tensors:

* ``Index``, ``ITensor`` with ``Dense`` (flat column-major) or ``Diag`` storage
  (src/tensor/cudense.jl:1-2, src/tensor/cudiag.jl:3-4),
* ``cuITensor``, ``randomCuITensor``, ``cu``, ``cpu`` (src/cuitensor.jl:1-49),
* ``A * B`` contraction (contract!!, src/tensor/cudense.jl:83-110 and the
  CuDiag methods, src/tensor/cudiag.jl:105-161), ``permute``, ``+``, ``-``,
  scalar ``*`` and ``/``, ``norm`` (src/tensor/cudense.jl:22-27,333-502),
* ``svd``, ``eigen``, ``qr`` with the truncation keywords
  (src/tensor/culinearalgebra.jl:33-121, src/tensor/cutruncate.jl).

Device storage is a 1-D float64 CUDA tensor from torch (used only as an
allocator); every arithmetic operation is a libitg.so call.  Host storage is a
1-D numpy array and only supports transfer (``cu``) and inspection.
"""
from __future__ import annotations

import ctypes as C
import itertools
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import DimensionMismatch, PREC_FP64, PREC_SPLIT, ITG_C64, ITG_F64, i32arr, i64arr

try:
    import torch
except ImportError:  # pragma: no cover - torch is part of the supported environment
    torch = None

_id_counter = itertools.count(1)
_seed_counter = itertools.count(1)

_state = {"precision": PREC_FP64, "device": 0}


def set_precision(p: str | int):
    """Arithmetic of ITensor contractions: "fp64" (default) or "split"."""
    if isinstance(p, str):
        p = {"fp64": PREC_FP64, "split": PREC_SPLIT}[p.lower()]
    _state["precision"] = int(p)


def get_precision() -> int:
    return _state["precision"]


def _precision_code(p: str | int) -> int:
    if isinstance(p, str):
        return {"fp64": PREC_FP64, "split": PREC_SPLIT}[p.lower()]
    return int(p)


def _h():
    return _lib.handle(_state["device"])


def _dev():
    return torch.device("cuda", _state["device"])


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def empty_dev(n: int, cplx: bool = False):
    return torch.empty(int(n), dtype=torch.complex128 if cplx else torch.float64, device=_dev())


def _is_cplx(data) -> bool:
    if torch is not None and isinstance(data, torch.Tensor):
        return data.is_complex()
    return np.iscomplexobj(data)


def _dt(t) -> int:
    """Element-type code of an ITensor's storage (ITG_F64 / ITG_C64)."""
    return ITG_C64 if t.is_complex else ITG_F64


def _to_complex_data(d):
    """Complex copy of real device data through itg_real_to_complex."""
    out = empty_dev(len(d), True)
    if len(d):
        _h().call("itg_real_to_complex", C.c_int64(len(d)), _ptr(d), _ptr(out))
    return out


# ----------------------------------------------------------------- Index
class Index:
    """A tensor index: identity (id, prime level), dimension and tags."""

    __slots__ = ("id", "dim", "tags", "plev")

    def __init__(self, dim: int, tags: str = "", plev: int = 0, id: int | None = None):
        self.dim = int(dim)
        self.tags = tags
        self.plev = int(plev)
        self.id = next(_id_counter) if id is None else id

    def prime(self, n: int = 1) -> "Index":
        return Index(self.dim, self.tags, self.plev + n, self.id)

    def noprime(self) -> "Index":
        return Index(self.dim, self.tags, 0, self.id)

    def sim(self) -> "Index":
        return Index(self.dim, self.tags, self.plev)

    def __eq__(self, o):
        return isinstance(o, Index) and self.id == o.id and self.plev == o.plev

    def __hash__(self):
        return hash((self.id, self.plev))

    def __repr__(self):
        return f"Index(dim={self.dim}, id={self.id}, tags={self.tags!r}, plev={self.plev})"


def dim(inds) -> int:
    d = 1
    for i in inds:
        d *= i.dim
    return d


def prime(x, n: int = 1):
    """Raise every index of an Index, ITensor, MPS or MPO by n prime levels."""
    if isinstance(x, Index):
        return x.prime(n)
    if not isinstance(x, ITensor) and hasattr(x, "prime"):
        return x.prime(n)
    return x.replaceinds(x.inds, [i.prime(n) for i in x.inds])


# --------------------------------------------------------------- storage
@dataclass
class Dense:
    data: object  # torch.Tensor (cuda, 1-D float64 or complex128) or numpy 1-D

    @property
    def is_cuda(self):
        return torch is not None and isinstance(self.data, torch.Tensor) and self.data.is_cuda


@dataclass
class Diag:
    data: object   # diagonal values (length = min dim), or length-1 for uniform
    uniform: bool = False

    @property
    def is_cuda(self):
        return torch is not None and isinstance(self.data, torch.Tensor) and self.data.is_cuda


# ---------------------------------------------------------------- ITensor
class ITensor:
    def __init__(self, store, inds):
        self.store = store
        self.inds = tuple(inds)
        if isinstance(store, Dense):
            n = len(store.data)
            if n != dim(self.inds):
                raise DimensionMismatch(2, f"storage length {n} != dim(inds) {dim(self.inds)}")

    # -- basic properties
    @property
    def is_cuda(self) -> bool:
        return self.store.is_cuda

    @property
    def dims(self):
        return tuple(i.dim for i in self.inds)

    @property
    def is_complex(self) -> bool:
        """ComplexF64 storage (interleaved re, im)."""
        return _is_cplx(self.store.data)

    def order(self) -> int:
        return len(self.inds)

    def isdiag(self) -> bool:
        return isinstance(self.store, Diag)

    def copy(self) -> "ITensor":
        d = self.store.data
        d2 = d.clone() if (torch is not None and isinstance(d, torch.Tensor)) else np.array(d, copy=True)
        st = Dense(d2) if isinstance(self.store, Dense) else Diag(d2, self.store.uniform)
        return ITensor(st, self.inds)

    def replaceinds(self, old, new) -> "ITensor":
        old = list(old)
        new = list(new)
        m = {o: n for o, n in zip(old, new)}
        return ITensor(self.store, [m.get(i, i) for i in self.inds])

    def __repr__(self):
        kind = "CuDense" if self.is_cuda and not self.isdiag() else (
            "CuDiag" if self.is_cuda else type(self.store).__name__)
        return f"ITensor({kind}, dims={self.dims})"

    # -- host access
    def array(self, *inds) -> np.ndarray:
        """Host n-d array (numpy, index order `inds` or the tensor's own)."""
        t = self if not self.isdiag() else dense(self)
        if inds:
            t = permute(t, *inds) if t.is_cuda else _host_permute(t, inds)
        d = t.store.data
        flat = d.detach().cpu().numpy() if (torch is not None and isinstance(d, torch.Tensor)) else np.asarray(d)
        return flat.reshape(t.dims if t.dims else (), order="F")

    def scalar(self):
        """T[] for an order-0 tensor; one device->host read (cudense.jl:25-26)."""
        if self.order() != 0:
            raise DimensionMismatch(2, "scalar() needs an order-0 tensor")
        d = self.store.data
        v = d[0].item() if (torch is not None and isinstance(d, torch.Tensor)) else d[0]
        return complex(v) if self.is_complex else float(v)

    def norm(self) -> float:
        return norm(self)

    # -- arithmetic
    def __mul__(self, other):
        if isinstance(other, ITensor):
            return contract(self, other)
        return _scale(self, other)

    def __rmul__(self, other):
        return _scale(self, other)

    def __truediv__(self, x):
        return _scale(self, 1.0 / x)

    def __neg__(self):
        return _scale(self, -1.0)

    def __add__(self, other):
        return _axpby(1.0, other, 1.0, self)

    def __sub__(self, other):
        return _axpby(-1.0, other, 1.0, self)


def _require_cuda(*ts):
    for t in ts:
        if not t.is_cuda:
            raise TypeError("operation needs CuDense/CuDiag storage: call cu(...) first "
                            "(this library has no CPU arithmetic path)")


def _host_permute(t: ITensor, inds) -> ITensor:
    perm = [t.inds.index(i) for i in inds]
    arr = np.asarray(t.store.data).reshape(t.dims, order="F").transpose(perm)
    return ITensor(Dense(np.asfortranarray(arr).ravel(order="F")), inds)


# --------------------------------------------------------- constructors
def ITensor_host(arr: np.ndarray, *inds) -> ITensor:
    """CPU ITensor holding `arr` (n-d, index order `inds`; float64 or complex128)."""
    arr = np.asarray(arr)
    arr = arr.astype(np.complex128 if np.iscomplexobj(arr) else np.float64, copy=False)
    if tuple(arr.shape) != tuple(i.dim for i in inds):
        raise DimensionMismatch(2, f"array shape {arr.shape} != index dims")
    return ITensor(Dense(arr.ravel(order="F").copy()), inds)


def cuITensor(x=None, *inds) -> ITensor:
    """Device ITensor: from an ITensor, an n-d array with inds, a number (filled), or zeros.

    A leading element type (float or complex) makes zeros of that type
    (cuITensor(SType, inds...)).  Mirrors src/cuitensor.jl:1-27.
    """
    if isinstance(x, ITensor):
        return cu(x)
    if x is float or x is complex:
        tdt = torch.complex128 if x is complex else torch.float64
        return ITensor(Dense(torch.zeros(dim(inds), dtype=tdt, device=_dev())), inds)
    if isinstance(x, Index):
        inds = (x,) + inds
        return ITensor(Dense(torch.zeros(dim(inds), dtype=torch.float64, device=_dev())), inds)
    if x is None:
        return ITensor(Dense(torch.zeros(dim(inds), dtype=torch.float64, device=_dev())), inds)
    if np.isscalar(x):
        tdt = torch.complex128 if np.iscomplexobj(x) else torch.float64
        return ITensor(Dense(torch.full((dim(inds),), x, dtype=tdt, device=_dev())), inds)
    arr = np.asarray(x)
    arr = arr.astype(np.complex128 if np.iscomplexobj(arr) else np.float64, copy=False)
    if arr.ndim == 1 and len(inds) != 1:
        if arr.size != dim(inds):
            raise DimensionMismatch(2, "flat data length != dim(inds)")
        flat = arr
    else:
        if tuple(arr.shape) != tuple(i.dim for i in inds):
            raise DimensionMismatch(2, f"array shape {arr.shape} != index dims")
        flat = arr.ravel(order="F")
    return ITensor(Dense(torch.from_numpy(np.ascontiguousarray(flat)).to(_dev())), inds)


def randomCuITensor(*inds, seed: int | None = None) -> ITensor:
    """Entries i.i.d. N(0,1) from the library's Philox generator (src/cuitensor.jl:35-49).

    A leading `complex` (randomCuITensor(ComplexF64, inds...)) draws complex
    entries with independent N(0, 1/2) real and imaginary parts.
    """
    cplx = False
    if inds and (inds[0] is complex or inds[0] is float):
        cplx = inds[0] is complex
        inds = inds[1:]
    n = dim(inds)
    s = next(_seed_counter) if seed is None else int(seed)
    if not cplx:
        t = torch.empty(max(n, 1), dtype=torch.float64, device=_dev())
        _h().call("itg_random_normal", C.c_int64(n), C.c_uint64(s), C.c_uint64(0), _ptr(t))
        return ITensor(Dense(t[:n]), inds)
    t = torch.empty(max(n, 1), dtype=torch.complex128, device=_dev())
    _h().call("itg_random_normal", C.c_int64(2 * n), C.c_uint64(s), C.c_uint64(0), _ptr(t))
    if n:
        _h().call("itg_scal", C.c_int64(2 * n), C.c_double(0.5 ** 0.5), _ptr(t))
    return ITensor(Dense(t[:n]), inds)


def diagITensor(d, *inds, uniform: bool = False) -> ITensor:
    """Device Diag ITensor (CuDiag).  `d` is the diagonal (or one value if
    uniform), real or complex."""
    arr = np.atleast_1d(np.asarray(d))
    arr = arr.astype(np.complex128 if np.iscomplexobj(arr) else np.float64, copy=False)
    return ITensor(Diag(torch.from_numpy(arr.copy()).to(_dev()), uniform), inds)


def delta(*inds, value: float = 1.0) -> ITensor:
    """UniformDiag tensor (every diagonal entry = value)."""
    return diagITensor([value], *inds, uniform=True)


def cu(x):
    """Move an ITensor / MPS / MPO to the device (cu, src/cuitensor.jl:28-33)."""
    if isinstance(x, ITensor):
        if x.is_cuda:
            return x
        hd = np.asarray(x.store.data)
        hd = hd.astype(np.complex128 if np.iscomplexobj(hd) else np.float64, copy=False)
        d = torch.from_numpy(np.ascontiguousarray(hd)).to(_dev())
        st = Dense(d) if isinstance(x.store, Dense) else Diag(d, x.store.uniform)
        return ITensor(st, x.inds)
    if hasattr(x, "_cu"):
        return x._cu()
    raise TypeError(f"cu: unsupported type {type(x)}")


def cpu(x):
    """Copy an ITensor / MPS / MPO back to the host (cpu, src/tensor/cudense.jl:12)."""
    if isinstance(x, ITensor):
        if not x.is_cuda:
            return x
        d = x.store.data.detach().cpu().numpy().copy()
        st = Dense(d) if isinstance(x.store, Dense) else Diag(d, x.store.uniform)
        return ITensor(st, x.inds)
    if hasattr(x, "_cpu"):
        return x._cpu()
    raise TypeError(f"cpu: unsupported type {type(x)}")


# ----------------------------------------------------------- operations
def _labels(*indsets):
    lab = {}
    for s in indsets:
        for i in s:
            if i not in lab:
                lab[i] = len(lab) + 1
    return lab


def _scale(t: ITensor, x) -> ITensor:
    """x * t for a real or complex number x (itg_scal / itg_zscal)."""
    _require_cuda(t)
    cx = isinstance(x, complex) or np.iscomplexobj(x)
    if cx and t.isdiag():
        raise TypeError("complex scaling of Diag storage is not supported")
    if t.is_complex or cx:
        out = t.store.data.clone() if t.is_complex else _to_complex_data(t.store.data)
        if len(out):
            a = (C.c_double * 2)(complex(x).real, complex(x).imag)
            _h().call("itg_zscal", C.c_int64(len(out)), a, _ptr(out))
        return ITensor(Dense(out), t.inds)
    out = t.store.data.clone()
    if len(out):
        _h().call("itg_scal", C.c_int64(len(out)), C.c_double(float(x)), _ptr(out))
    st = Dense(out) if isinstance(t.store, Dense) else Diag(out, t.store.uniform)
    return ITensor(st, t.inds)


def dag(x):
    """Complex conjugate (dag); a real tensor is returned as is.  For an MPS or
    MPO every site tensor is conjugated."""
    if not isinstance(x, ITensor):
        if hasattr(x, "tensors"):
            y = x.copy()
            y.tensors = [dag(t) for t in x.tensors]
            return y
        return x
    if not x.is_complex:
        return x
    _require_cuda(x)
    out = torch.empty_like(x.store.data)
    if len(out):
        _h().call("itg_conj", C.c_int64(len(out)), _ptr(x.store.data), _ptr(out))
    return ITensor(Dense(out), x.inds)


def complex_(t: ITensor) -> ITensor:
    """ComplexF64 copy of a tensor (complex(::ITensor), test/test_cuitensor.jl:77-81)."""
    _require_cuda(t)
    if t.isdiag():
        t = dense(t)
    if t.is_complex:
        return t.copy()
    return ITensor(Dense(_to_complex_data(t.store.data)), t.inds)


def permute(t: ITensor, *inds) -> ITensor:
    """Copy of `t` with its storage reordered to `inds` (permute!, cudense.jl:447-500)."""
    if len(inds) == 1 and isinstance(inds[0], (list, tuple)):
        inds = tuple(inds[0])
    if set(inds) != set(t.inds) or len(inds) != len(t.inds):
        raise DimensionMismatch(2, "permute: index sets differ")
    if t.isdiag():
        return ITensor(t.store, inds)
    _require_cuda(t)
    lab = _labels(t.inds)
    out = empty_dev(dim(inds), t.is_complex)
    if dim(inds) > 0:
        _h().call("itg_permute", _dt(t), C.c_double(1.0), _ptr(t.store.data), len(t.inds),
                  i64arr(t.dims), i32arr([lab[i] for i in t.inds]), _ptr(out),
                  i32arr([lab[i] for i in inds]))
    return ITensor(Dense(out), inds)


def _axpby(alpha: float, a: ITensor, beta: float, b: ITensor) -> ITensor:
    """alpha*a + beta*b, result in b's index order (Base.:+ / :-, cudense.jl:333-445)."""
    _require_cuda(a, b)
    if set(a.inds) != set(b.inds) or len(a.inds) != len(b.inds):
        raise DimensionMismatch(2, "ITensor +/-: index sets differ")
    a = dense(a) if a.isdiag() else a
    b = dense(b) if b.isdiag() else b
    if a.is_complex != b.is_complex:
        a, b = (a, complex_(b)) if a.is_complex else (complex_(a), b)
    lab = _labels(b.inds)
    out = empty_dev(dim(b.inds), b.is_complex)
    if dim(b.inds) > 0:
        _h().call("itg_axpby_permuted", _dt(b), C.c_double(alpha), _ptr(a.store.data), len(a.inds),
                  i64arr(a.dims), i32arr([lab[i] for i in a.inds]), C.c_double(beta),
                  _ptr(b.store.data), i32arr([lab[i] for i in b.inds]), _ptr(out))
    return ITensor(Dense(out), b.inds)


def norm(t: ITensor) -> float:
    """Frobenius norm of an ITensor, or the norm of an MPS."""
    if not isinstance(t, ITensor):
        from .mpsops import norm as _norm_chain
        return _norm_chain(t)
    _require_cuda(t)
    if t.isdiag():
        d = t.store.data
        if t.store.uniform:
            return abs(float(d[0].item())) * np.sqrt(min(t.dims) if t.dims else 1)
        t = ITensor(Dense(d), (Index(len(d)),))
    r = C.c_double()
    n = len(t.store.data) * (2 if t.is_complex else 1)
    _h().call("itg_nrm2", C.c_int64(n), _ptr(t.store.data), C.byref(r))
    return r.value


def dense(t: ITensor) -> ITensor:
    """Dense copy of a Diag tensor (dense(::CuDiagTensor), src/tensor/cudiag.jl:8-13)."""
    if not t.isdiag():
        return t
    _require_cuda(t)
    if t.is_complex:
        Dr, Di = _diag_parts(t)
        return _axpby(1.0, _scale(dense(Di), 1j), 1.0, complex_(dense(Dr)))
    out = empty_dev(dim(t.inds))
    if dim(t.inds) > 0:
        _h().call("itg_diag_to_dense", _ptr(t.store.data), int(t.store.uniform), len(t.inds),
                  i64arr(t.dims), _ptr(out))
    return ITensor(Dense(out), t.inds)


def contract(A: ITensor, B: ITensor, precision: int | None = None, **kw) -> ITensor:
    """A * B: contract all common indices; result indices = A's uncommon then B's.

    With an MPO first argument this is the MPO x MPS / MPO x MPO product of
    itg.mpsops.contract (keywords method, maxdim, cutoff, ...).
    """
    if not isinstance(A, ITensor):
        from .mpsops import contract as _contract_chain
        return _contract_chain(A, B, **kw)
    _require_cuda(A, B)
    common = [i for i in A.inds if i in B.inds]
    out_inds = tuple([i for i in A.inds if i not in common] + [i for i in B.inds if i not in common])
    prec = _state["precision"] if precision is None else precision
    if A.isdiag() and B.isdiag():
        return _diag_diag(A, B, common, out_inds)
    if A.isdiag() or B.isdiag():
        D, T = (A, B) if A.isdiag() else (B, A)
        return _diag_dense(D, T, out_inds)
    lab = _labels(A.inds, B.inds)
    if A.is_complex or B.is_complex:
        out = empty_dev(dim(out_inds), True)
        if dim(out_inds) > 0:
            one = (C.c_double * 2)(1.0, 0.0)
            zero = (C.c_double * 2)(0.0, 0.0)
            _h().call("itg_contract_z", _dt(A), _dt(B), one,
                      _ptr(A.store.data), len(A.inds), i64arr(A.dims), i32arr([lab[i] for i in A.inds]),
                      _ptr(B.store.data), len(B.inds), i64arr(B.dims), i32arr([lab[i] for i in B.inds]),
                      zero, _ptr(out), len(out_inds), i64arr([i.dim for i in out_inds]),
                      i32arr([lab[i] for i in out_inds]), int(prec))
        return ITensor(Dense(out), out_inds)
    out = empty_dev(dim(out_inds))
    if dim(out_inds) > 0:
        _h().call("itg_contract", ITG_F64, C.c_double(1.0),
                  _ptr(A.store.data), len(A.inds), i64arr(A.dims), i32arr([lab[i] for i in A.inds]),
                  _ptr(B.store.data), len(B.inds), i64arr(B.dims), i32arr([lab[i] for i in B.inds]),
                  C.c_double(0.0),
                  _ptr(out), len(out_inds), i64arr([i.dim for i in out_inds]),
                  i32arr([lab[i] for i in out_inds]), int(prec))
    return ITensor(Dense(out), out_inds)


def _split_cplx(d):
    """Real parts (re, im) of complex device data: the interleaved vector, read
    as the real (2, n) array, permuted to (n, 2) (itg_permute)."""
    n = len(d)
    out = empty_dev(2 * n)
    if n:
        _h().call("itg_permute", ITG_F64, C.c_double(1.0), _ptr(d), 2, i64arr([2, n]), i32arr([1, 2]), _ptr(out),
                  i32arr([2, 1]))
    return out[:n], out[n:]


def _join_cplx(re, im):
    """Complex device data re + i im (the inverse permutation of _split_cplx)."""
    n = len(re)
    buf = torch.cat([re, im]) if n else re
    out = empty_dev(n, True)
    if n:
        _h().call("itg_permute", ITG_F64, C.c_double(1.0), _ptr(buf), 2, i64arr([n, 2]), i32arr([1, 2]), _ptr(out),
                  i32arr([2, 1]))
    return out


def _diag_parts(D: ITensor):
    """(real part, imaginary part or None) of a Diag tensor, as real Diags."""
    if not D.is_complex:
        return D, None
    re, im = _split_cplx(D.store.data)
    return ITensor(Diag(re, D.store.uniform), D.inds), ITensor(Diag(im, D.store.uniform), D.inds)


def _diag_dense(D: ITensor, T: ITensor, out_inds) -> ITensor:
    if D.is_complex:
        # (Dr + i Di) T = Dr T + i (Di T)
        Dr, Di = _diag_parts(D)
        return _axpby(1.0, _scale(_diag_dense(Di, T, out_inds), 1j), 1.0, complex_(_diag_dense(Dr, T, out_inds)))
    lab = _labels(D.inds, T.inds)
    out = empty_dev(dim(out_inds), T.is_complex)
    if dim(out_inds) > 0:
        _h().call("itg_diag_contract", _dt(T), C.c_double(1.0), _ptr(D.store.data),
                  int(D.store.uniform), len(D.inds), i64arr(D.dims), i32arr([lab[i] for i in D.inds]),
                  _ptr(T.store.data), len(T.inds), i64arr(T.dims), i32arr([lab[i] for i in T.inds]),
                  C.c_double(0.0), _ptr(out), len(out_inds), i64arr([i.dim for i in out_inds]),
                  i32arr([lab[i] for i in out_inds]))
    return ITensor(Dense(out), out_inds)


def _diag_diag(A: ITensor, B: ITensor, common, out_inds) -> ITensor:
    if A.is_complex or B.is_complex:
        # (Ar + i Ai)(Br + i Bi) elementwise, from real products
        Ar, Ai = _diag_parts(A)
        Br, Bi = _diag_parts(B)
        parts = [(1.0, Ar, Br, 0)]
        if Ai is not None and Bi is not None:
            parts.append((-1.0, Ai, Bi, 0))
        if Bi is not None:
            parts.append((1.0, Ar, Bi, 1))
        if Ai is not None:
            parts.append((1.0, Ai, Br, 1))
        acc = [None, None]
        for sgn, X, Y, k in parts:
            Z = _diag_diag(X, Y, common, out_inds)
            Zd = ITensor(Dense(Z.store.data), (Index(len(Z.store.data)),))
            if acc[k] is None:
                acc[k] = _scale(Zd, sgn) if sgn != 1.0 else Zd
            else:
                acc[k] = _axpby(sgn, Zd, 1.0, acc[k].replaceinds(acc[k].inds, Zd.inds))
        re = acc[0].store.data
        im = acc[1].store.data if acc[1] is not None else torch.zeros_like(re)
        z = _join_cplx(re, im)
        if len(out_inds) == 0:
            return ITensor(Dense(z), ())
        uni = A.store.uniform and B.store.uniform
        return ITensor(Diag(z, uni), out_inds)
    na = 1 if A.store.uniform else len(A.store.data)
    nb = 1 if B.store.uniform else len(B.store.data)
    lens = [n for n, u in ((na, A.store.uniform), (nb, B.store.uniform)) if not u]
    dims_all = [i.dim for i in A.inds] + [i.dim for i in B.inds]
    n = min(lens) if lens else min(dims_all)
    out = empty_dev(max(n, 1))
    _h().call("itg_diag_diag", C.c_int64(n), C.c_double(1.0), _ptr(A.store.data),
              int(A.store.uniform), _ptr(B.store.data), int(B.store.uniform), _ptr(out))
    if len(out_inds) == 0:
        # full contraction of two diagonals: the sum of the products
        ones = torch.ones(max(n, 1), dtype=torch.float64, device=_dev())
        r = C.c_double()
        _h().call("itg_dot", C.c_int64(n), _ptr(out), _ptr(ones), C.byref(r))
        return ITensor(Dense(torch.full((1,), r.value, dtype=torch.float64, device=_dev())), ())
    uni = A.store.uniform and B.store.uniform
    return ITensor(Diag(out[: (1 if uni else n)], uni), out_inds)


# ------------------------------------------------------- factorisations
@dataclass
class Spectrum:
    """Kept eigenvalues of the density matrix (P = S^2) and the truncation error."""
    eigs: np.ndarray
    truncerr: float


def _trunc_args(m, n, kw):
    maxdim = int(kw.get("maxdim", min(m, n)) or 0)
    mindim = int(kw.get("mindim", 1))
    cutoff = float(kw.get("cutoff", 0.0) or 0.0)
    absolute = int(bool(kw.get("absoluteCutoff", kw.get("use_absolute_cutoff", False))))
    rel = int(bool(kw.get("doRelCutoff", kw.get("use_relative_cutoff", True))))
    legacy = int(bool(kw.get("legacy_gpu", False)))
    return maxdim, mindim, cutoff, absolute, rel, legacy


def svd(A: ITensor, *left_inds, **kw):
    """U, S, V, spec with A ~ U * S * V (culinearalgebra.jl:33-72 + cutruncate.jl).

    Keywords: maxdim, mindim, cutoff, absoluteCutoff, doRelCutoff and
    legacy_gpu (reproduce the reference GPU truncation rule instead of the
    ITensors CPU rule).  S is returned as a CuDiag tensor with indices (u, v).
    """
    _require_cuda(A)
    if len(left_inds) == 1 and isinstance(left_inds[0], (list, tuple)):
        left_inds = tuple(left_inds[0])
    left = [i for i in A.inds if i in left_inds]
    if len(left) != len(left_inds):
        raise DimensionMismatch(2, "svd: left index not in tensor")
    right = [i for i in A.inds if i not in left_inds]
    Am = permute(A, *left, *right) if A.isdiag() or tuple(left + right) != A.inds else A
    if Am.isdiag():
        Am = dense(Am)
    m, n = dim(left), dim(right)
    r = min(m, n)
    cplx = Am.is_complex
    U = empty_dev(m * r, cplx)
    S = empty_dev(r)
    V = empty_dev(n * r, cplx)
    k = C.c_int64()
    te = C.c_double()
    dc = C.c_double()
    maxdim, mindim, cutoff, ab, rel, legacy = _trunc_args(m, n, kw)
    # complex: A ~ U S V^H (so U * S * dag(V) rebuilds A, test/test_cuitensor.jl:100-106)
    _h().call("itg_svd_trunc_z" if cplx else "itg_svd_trunc", C.c_int64(m), C.c_int64(n), _ptr(Am.store.data),
              C.c_int64(m),
              C.c_int64(maxdim), C.c_int64(mindim), C.c_double(cutoff), ab, rel, legacy,
              _ptr(U), _ptr(S), _ptr(V), C.byref(k), C.byref(te), C.byref(dc))
    kk = int(k.value)
    u = Index(kk, kw.get("lefttags", "Link,u"))
    v = Index(kk, kw.get("righttags", "Link,v"))
    Ut = ITensor(Dense(U[: m * kk].clone()), (*left, u))
    St = ITensor(Diag(S[:kk].clone(), False), (u, v))
    Vt = ITensor(Dense(V[: n * kk].clone()), (*right, v))
    P = (S[:kk] ** 2).detach().cpu().numpy()
    return Ut, St, Vt, Spectrum(P, te.value)


def factorize(A: ITensor, *left_inds, ortho: str = "left", **kw):
    """L, R with A ~ L * R and one orthonormal factor (ITensors' factorize with
    which_decomp = "svd"; the two-site bond split of dmrg).

    ortho="left": L (left_inds..., l) has orthonormal columns, R = S V^T.
    ortho="right": R (l, right inds...) has orthonormal rows, L = U S.
    Keywords as svd, plus method (0 auto, 1 FP64 Jacobi, 2 mixed) and
    precision ("fp64" / "split") of the products.  Returns (L, R, spec).
    """
    _require_cuda(A)
    if len(left_inds) == 1 and isinstance(left_inds[0], (list, tuple)):
        left_inds = tuple(left_inds[0])
    if A.is_complex:
        # complex: through the complex SVD, A = U S V^H
        if ortho not in ("left", "right"):
            raise ValueError("factorize: ortho must be 'left' or 'right'")
        skw = {k: v for k, v in kw.items() if k not in ("method", "precision", "tags")}
        U, S, V, spec = svd(A, *left_inds, **skw)
        u, v = U.inds[-1], V.inds[-1]
        l = Index(u.dim, kw.get("tags", "Link,fac"))
        right = [i for i in A.inds if i not in left_inds]
        if ortho == "left":
            Rt = contract(S, dag(V))                              # (u, right...)
            return U.replaceinds([u], [l]), permute(Rt.replaceinds([u], [l]), l, *right), spec
        Lt = contract(U, S)                                       # (left..., v)
        return Lt.replaceinds([v], [l]), dag(V).replaceinds([v], [l]), spec
    left = [i for i in A.inds if i in left_inds]
    if len(left) != len(left_inds):
        raise DimensionMismatch(2, "factorize: left index not in tensor")
    right = [i for i in A.inds if i not in left_inds]
    Am = permute(A, *left, *right) if A.isdiag() or tuple(left + right) != A.inds else A
    if Am.isdiag():
        Am = dense(Am)
    if ortho not in ("left", "right"):
        raise ValueError("factorize: ortho must be 'left' or 'right'")
    m, n = dim(left), dim(right)
    r = min(m, n)
    big = max(m, n) * r
    Lb = empty_dev(big)
    S = empty_dev(r)
    Cb = empty_dev(big)
    k = C.c_int64()
    te = C.c_double()
    dc = C.c_double()
    maxdim, mindim, cutoff, ab, rel, legacy = _trunc_args(m, n, kw)
    prec = _precision_code(kw.get("precision", get_precision()))
    _h().call("itg_factorize_trunc", C.c_int64(m), C.c_int64(n), _ptr(Am.store.data), C.c_int64(m),
              C.c_int64(maxdim), C.c_int64(mindim), C.c_double(cutoff), ab, rel, legacy,
              0 if ortho == "left" else 1, int(kw.get("method", 0)), prec,
              _ptr(Lb), _ptr(S), _ptr(Cb), C.byref(k), C.byref(te), C.byref(dc))
    kk = int(k.value)
    l = Index(kk, kw.get("tags", "Link,fac"))
    if ortho == "left":
        Lt = ITensor(Dense(Lb[: m * kk].clone()), (*left, l))
        Rt = ITensor(Dense(Cb[: kk * n].clone()), (l, *right))
    else:
        Lt = ITensor(Dense(Cb[: m * kk].clone()), (*left, l))
        Rt = ITensor(Dense(Lb[: n * kk].clone()), (*right, l))
    P = (S[:kk] ** 2).detach().cpu().numpy()
    return Lt, Rt, Spectrum(P, te.value)


def eigen(A: ITensor, left_inds, right_inds, **kw):
    """Hermitian eigendecomposition (culinearalgebra.jl:74-108).

    A is viewed as the matrix M[left, right] (symmetric, or Hermitian for
    ComplexF64).  Returns (D, U, spec) with D a real CuDiag tensor on (l, r)
    holding descending eigenvalues, and U with indices (*right_inds, r), so
    that M ~ U D U^H (M U = U D).
    """
    _require_cuda(A)
    left, right = list(left_inds), list(right_inds)
    Am = permute(A, *left, *right)
    n = dim(left)
    if dim(right) != n:
        raise DimensionMismatch(2, "eigen: square matrix required")
    cplx = Am.is_complex
    if "maxdim" not in kw and "cutoff" not in kw:
        kw = dict(kw, mindim=n)   # no truncation keywords: keep every eigenvalue, negative ones too
    D = empty_dev(n)
    U = empty_dev(n * n, cplx)
    k = C.c_int64()
    te = C.c_double()
    dc = C.c_double()
    maxdim, mindim, cutoff, ab, rel, legacy = _trunc_args(n, n, kw)
    _h().call("itg_eigh_trunc_z" if cplx else "itg_eigh_trunc", C.c_int64(n), _ptr(Am.store.data), C.c_int64(n),
              C.c_int64(maxdim), C.c_int64(mindim), C.c_double(cutoff), ab, rel, legacy,
              _ptr(D), _ptr(U), C.byref(k), C.byref(te), C.byref(dc))
    kk = int(k.value)
    l = Index(kk, "Link,eigen,l")
    r = Index(kk, "Link,eigen,r")
    Dt = ITensor(Diag(D[:kk].clone(), False), (l, r))
    Ut = ITensor(Dense(U[: n * kk].clone()), (*right, r))
    return Dt, Ut, Spectrum(D[:kk].detach().cpu().numpy(), te.value)


def qr(A: ITensor, *left_inds):
    """Q, R with A = Q * R (culinearalgebra.jl:110-121); new index dim = min(m, n)."""
    _require_cuda(A)
    if len(left_inds) == 1 and isinstance(left_inds[0], (list, tuple)):
        left_inds = tuple(left_inds[0])
    left = [i for i in A.inds if i in left_inds]
    right = [i for i in A.inds if i not in left_inds]
    Am = permute(A, *left, *right)
    m, n = dim(left), dim(right)
    r = min(m, n)
    cplx = Am.is_complex
    Q = empty_dev(m * r, cplx)
    R = empty_dev(r * n, cplx)
    _h().call("itg_qr_z" if cplx else "itg_qr", C.c_int64(m), C.c_int64(n), _ptr(Am.store.data), C.c_int64(m),
              _ptr(Q), _ptr(R))
    q = Index(r, "Link,qr")
    return ITensor(Dense(Q), (*left, q)), ITensor(Dense(R), (q, *right))
