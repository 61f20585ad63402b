"""itg — Python mirror of ITensorsGPU.jl's API on the GB300 library libitg.so.

Every tensor operation runs in libitg.so (hand-written sm_103a CUDA behind the
C ABI in include/itg.h).  There is no CPU arithmetic path: calling an
operation on host storage raises, and a missing libitg.so raises on import of
the first operation.
"""
from ._lib import (DimensionMismatch, ITGError, NotConverged, PREC_FP64, PREC_SPLIT, Handle,
                   handle, load_library)
from .tensor import (Diag, Dense, ITensor, ITensor_host, Index, Spectrum, contract, cpu, cu,
                     cuITensor, dag, delta, dense, diagITensor, dim, eigen, factorize, get_precision, norm, permute,
                     prime, qr, randomCuITensor, set_precision, svd)
from .mps import (MPO, MPS, cuMPO, cuMPS, heisenberg_mpo, j1j2_mpo, op, ops,
                  productCuMPS, productMPS_host, randomCuMPS, siteinds, spin_ops, tfim_mpo, xxz_mpo)
from .dmrg import (DMRGResult, Sweeps, cutoff_, dmrg, expect_energy, inner, maxdim_, mindim_,
                   noise_, sweepnext)
from .batched import dmrg_batched
from .mpsops import (ArgumentError, add, apply, inner, leftlim, linkind, maxlinkdim, normalize_,
                     orthogonalize_, randomCuMPO, replacebond_, rightlim, siteind, truncate_)

from .solvers import ITensorMap, davidson
from .tensor import complex_

__all__ = [n for n in dir() if not n.startswith("_")]
# complex(A) as in the reference (kept out of __all__: it would shadow the builtin on star imports)
complex = complex_  # noqa: A001
