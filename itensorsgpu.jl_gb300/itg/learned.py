"""Learned Davidson preconditioner: data from the plain solver, training, use.

The network (itg_mlp_*, hand-written BF16/FP32 kernels in csrc/itg_mlp.cu)
maps per-element features of the two-site problem (normalised residual,
shifted diagonal, clipped inverse diagonal, left/right Schmidt values) to a
correction g of the diagonal preconditioner: t = (1 + g) m with m the
diagonally preconditioned residual, so the untrained network (zero output
layer) is the diagonal preconditioner.  Training samples come from the plain
solver itself: at every bond of a plain DMRG run the starting vector x0 is
refined to the converged eigenvector x* with the plain Davidson; the
normalised ideal correction d = x* - (x0.x*) x0 (oriented so that d.r >= 0) is
split into its best fit c m by the diagonal correction and the rest d - c m,
and the network learns g with g (c m) ~ d - c m.  In use, convergence is judged by the exact residual of
the plain matvec and the diagonal preconditioner takes over when a learned
step stalls (itg_davidson_heff2_learned).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import tensor as T
from ._lib import PREC_FP64

NFEAT = 5


def _p(t):
    return C.c_void_p(t.data_ptr())


class LearnedPreconditioner:
    def __init__(self, seed: int = 7):
        self.h = T._h()
        p = C.c_void_p()
        self.h.call("itg_mlp_create", NFEAT, C.c_uint64(seed), C.byref(p))
        self.ptr = p
        n = C.c_int64()
        st = self.h.lib.itg_mlp_num_params(self.ptr, C.byref(n))
        self.h.check(st, "itg_mlp_num_params")
        self.nparams = n.value
        self.history = []

    def close(self):
        if self.ptr:
            self.h.call("itg_mlp_destroy", self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self) -> np.ndarray:
        out = np.empty(self.nparams, dtype=np.float32)
        self.h.call("itg_mlp_get_params", self.ptr, C.c_void_p(out.ctypes.data))
        return out

    def set_params(self, w: np.ndarray):
        w = np.ascontiguousarray(w, dtype=np.float32)
        assert w.size == self.nparams
        self.h.call("itg_mlp_set_params", self.ptr, C.c_void_p(w.ctypes.data))

    def forward(self, X):
        import torch
        n = X.numel() // NFEAT
        g = torch.empty(n, dtype=torch.float32, device=X.device)
        self.h.call("itg_mlp_forward", self.ptr, C.c_int64(n), _p(X), _p(g))
        return g

    def step(self, X, mult, target, lr: float, grad=None):
        """One training step on (X, mult, target) device tensors; returns the loss."""
        loss = C.c_float()
        n = mult.numel()
        self.h.call("itg_mlp_train_step", self.ptr, C.c_int64(n), _p(X), _p(mult), _p(target), C.c_float(lr),
                    _p(grad) if grad is not None else None, C.byref(loss))
        return loss.value

    def train(self, data, steps: int = 600, lr: float = 1e-3, batch: int = 32768, seed: int = 0):
        """Adam on contiguous minibatches of the concatenated samples."""
        X, mult, target = data
        n = mult.numel()
        rng = np.random.default_rng(seed)
        for it in range(steps):
            if n <= batch:
                lo, hi = 0, n
            else:
                lo = int(rng.integers(0, n - batch))
                hi = lo + batch
            loss = self.step(X[lo * NFEAT: hi * NFEAT], mult[lo:hi], target[lo:hi], lr)
            self.history.append(loss)
        return self.history[-1]


class SampleCollector:
    """bond_hook for itg.dmrg that records (features, multiplier, target) samples."""

    def __init__(self, max_elements: int = 4_000_000, solve_krylov: int = 8, solve_iters: int = 40,
                 solve_tol: float = 1e-9):
        self.h = T._h()
        self.X, self.M, self.Y = [], [], []
        self.count = 0
        self.max_elements = max_elements
        self.kd, self.mi, self.tol = solve_krylov, solve_iters, solve_tol

    def __call__(self, ctx):
        import torch
        if self.count >= self.max_elements:
            return
        h = self.h
        chiL, chiR, d = ctx["chiL"], ctx["chiR"], ctx["d"]
        n = chiL * d * d * chiR
        args = (C.c_int64(chiL), C.c_int64(chiR), C.c_int64(d), C.c_int64(ctx["wL"]), C.c_int64(ctx["wM"]),
                C.c_int64(ctx["wR"]), _p(ctx["L"]), _p(ctx["W1"]), _p(ctx["W2"]), _p(ctx["R"]))
        x0 = ctx["phi"].clone()
        nrm = C.c_double()
        h.call("itg_nrm2", C.c_int64(n), _p(x0), C.byref(nrm))
        h.call("itg_scal", C.c_int64(n), C.c_double(1.0 / nrm.value), _p(x0))
        hx = torch.empty_like(x0)
        h.call("itg_heff2_apply", *args, _p(x0), _p(hx), PREC_FP64)
        th = C.c_double()
        h.call("itg_dot", C.c_int64(n), _p(x0), _p(hx), C.byref(th))
        r = hx.clone()
        h.call("itg_axpy", C.c_int64(n), C.c_double(-th.value), _p(x0), _p(r))
        dg = torch.empty_like(x0)
        h.call("itg_heff2_diag", *args, _p(dg))
        # ideal correction from the converged plain solve
        xs = x0.clone()
        e = C.c_double()
        nmv = C.c_int()
        h.call("itg_davidson_heff2", *args, _p(xs), self.kd, self.mi, C.c_double(self.tol), PREC_FP64,
               C.byref(e), C.byref(nmv))
        ov = C.c_double()
        h.call("itg_dot", C.c_int64(n), _p(x0), _p(xs), C.byref(ov))
        dvec = xs.clone()
        h.call("itg_axpy", C.c_int64(n), C.c_double(-ov.value), _p(x0), _p(dvec))
        dn = C.c_double()
        h.call("itg_nrm2", C.c_int64(n), _p(dvec), C.byref(dn))
        if not dn.value > 1e-12:
            return
        sr = C.c_double()
        h.call("itg_dot", C.c_int64(n), _p(dvec), _p(r), C.byref(sr))
        sgn = 1.0 if sr.value >= 0 else -1.0
        h.call("itg_scal", C.c_int64(n), C.c_double(sgn * np.sqrt(n) / dn.value), _p(dvec))
        X = torch.empty(n * NFEAT, dtype=torch.float32, device=x0.device)
        M = torch.empty(n, dtype=torch.float32, device=x0.device)
        lamL, lamR = ctx["lamL"], ctx["lamR"]
        h.call("itg_heff2_features", C.c_int64(chiL), C.c_int64(chiR), C.c_int64(d), _p(r), _p(dg),
               C.c_double(th.value), _p(lamL) if lamL is not None else None,
               _p(lamR) if lamR is not None else None, _p(X), _p(M))
        # best scale of the diagonal correction, then the part it misses
        y = dvec.float()
        mm = float((M.double() * M.double()).sum())
        c = float((M.double() * dvec).sum()) / mm if mm > 0 else 0.0
        Mc = M * c
        self.X.append(X)
        self.M.append(Mc)
        self.Y.append(y - Mc)
        self.count += n

    def data(self):
        import torch
        return torch.cat(self.X), torch.cat(self.M), torch.cat(self.Y)
