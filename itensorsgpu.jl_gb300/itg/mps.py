"""MPS / MPO containers, site indices, product/random states and Hamiltonian MPOs.

Mirrors src/mps/cumps.jl and src/mps/cumpo.jl: ``cuMPS``, ``randomCuMPS``,
``productCuMPS``, ``cuMPO``, ``cu(psi)``, ``cpu(psi)``.  AutoMPO/OpSum lives in
ITensors.jl, outside the reference, so the Hamiltonians DMRG needs are built
here as explicit finite-state-machine MPOs:

* S=1/2 or S=1 Heisenberg / XXZ chain (bond dimension 5),
* transverse-field Ising chain (bond dimension 3),
* J1-J2 Heisenberg chain (bond dimension 8).

Layout: site tensor j of an MPS has indices (l_{j-1}, s_j, l_j) with dimension-1
links at the two ends; MPO tensor j has (w_{j-1}, s_j', s_j, w_j) where s' is
the bra (output) index.  Both are column-major flat storage.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import tensor as T
from ._lib import DimensionMismatch
from .tensor import ITensor, Index, Dense, cu, cpu


# -------------------------------------------------------------- operators
def spin_ops(d: int):
    """Spin operators for S=(d-1)/2 in the basis m = S, S-1, ..., -S."""
    S = (d - 1) / 2.0
    m = S - np.arange(d)
    Sz = np.diag(m)
    Sp = np.zeros((d, d))
    for k in range(1, d):  # <m+1|S+|m>
        Sp[k - 1, k] = np.sqrt(S * (S + 1) - m[k] * (m[k] + 1))
    Sm = Sp.T.copy()
    Sx = 0.5 * (Sp + Sm)
    return {"Id": np.eye(d), "Sz": Sz, "S+": Sp, "S-": Sm, "Sx": Sx}


_QUBIT_GATES = {
    "X": np.array([[0.0, 1.0], [1.0, 0.0]]),
    "Z": np.diag([1.0, -1.0]),
    "H": np.array([[1.0, 1.0], [1.0, -1.0]]) / np.sqrt(2.0),
    "I": np.eye(2),
}


def _two_site_gate(name: str) -> np.ndarray:
    """4 x 4 matrix on (s1 s2) with s1 the slower index, basis |0>, |1>."""
    if name in ("CNOT", "CX"):
        g = np.eye(4)
        g[2:, 2:] = [[0.0, 1.0], [1.0, 0.0]]
        return g
    if name == "CZ":
        return np.diag([1.0, 1.0, 1.0, -1.0])
    if name == "SWAP":
        return np.eye(4)[[0, 2, 1, 3]]
    raise KeyError(name)


def op(name: str, *sites, matrix=None):
    """Device operator ITensor with indices (s1', ..., sk', s1, ..., sk).

    One-site names: the spin operators "Id", "Sz", "S+", "S-", "Sx" of the
    site's spin and the qubit gates "X", "Z", "H", "I"; two-site qubit gates:
    "CNOT" ("CX"), "CZ", "SWAP".  `matrix` gives any real d^k x d^k matrix
    instead, rows and columns ordered with s1 the slowest index (the order of
    a Kronecker product).  Mirrors op / op_matrix of examples/gate_evolution.jl.
    """
    k = len(sites)
    d = [s.dim for s in sites]
    if matrix is None:
        if k == 1:
            tab = dict(spin_ops(d[0]))
            if d[0] == 2:
                tab.update(_QUBIT_GATES)
            matrix = tab[name]
        elif k == 2 and d == [2, 2]:
            matrix = _two_site_gate(name)
        else:
            raise KeyError(f"op: no built-in {name!r} on {k} sites of dimensions {d}")
    M = np.asarray(matrix, dtype=np.float64).reshape(d + d)    # [s1'..sk', s1..sk], s1 slowest
    return T.cuITensor(M, *[s.prime() for s in sites], *sites)


def ops(sites, specs):
    """[op(name, sites[n]) for (name, n) in specs] (n 0-based; a tuple of
    site numbers for multi-site gates)."""
    out = []
    for name, n in specs:
        ns = n if isinstance(n, (tuple, list)) else (n,)
        out.append(op(name, *[sites[j] for j in ns]))
    return out


def siteinds(kind, N: int | None = None):
    """N site indices of a named kind ("S=1/2", "S=1", "Qubit"), or the site
    indices of an MPS / MPO when called with one."""
    if isinstance(kind, (MPS, MPO)):
        return list(kind.sites)
    d = {"S=1/2": 2, "S=1": 3, "Qubit": 2, "qubit": 2}[kind]
    return [Index(d, f"{kind},Site,n={j + 1}") for j in range(N)]


_STATE_NAMES = {
    2: {"Up": 0, "Dn": 1, "↑": 0, "↓": 1, "0": 0, "1": 1},
    3: {"Up": 0, "Z0": 1, "Dn": 2, "↑": 0, "0": 1, "↓": 2},
}


# ------------------------------------------------------------------- MPS
class MPS:
    def __init__(self, tensors, sites, llim: int = -1, rlim: int | None = None):
        self.tensors = list(tensors)
        self.sites = list(sites)
        self.llim = llim
        self.rlim = len(self.tensors) if rlim is None else rlim

    def __len__(self):
        return len(self.tensors)

    def __getitem__(self, j):
        return self.tensors[j]

    def __setitem__(self, j, v):
        self.tensors[j] = v

    @property
    def is_cuda(self):
        return all(t.is_cuda for t in self.tensors)

    def links(self):
        return [t.inds[2] for t in self.tensors[:-1]]

    def linkdims(self):
        return [t.dims[2] for t in self.tensors[:-1]]

    def maxlinkdim(self):
        return max(self.linkdims(), default=1)

    def copy(self):
        return MPS([t.copy() for t in self.tensors], self.sites, self.llim, self.rlim)

    def _cu(self):
        return MPS([cu(t) for t in self.tensors], self.sites, self.llim, self.rlim)

    def _cpu(self):
        return MPS([cpu(t) for t in self.tensors], self.sites, self.llim, self.rlim)

    def prime(self, n: int = 1):
        """Every index (sites and links) raised n prime levels."""
        return MPS([T.prime(t, n) for t in self.tensors], [s.prime(n) for s in self.sites],
                   self.llim, self.rlim)

    def __str__(self):
        return _show("MPS", self.tensors)

    def __add__(self, other):
        from .mpsops import add
        return add(self, other)


class MPO:
    def __init__(self, tensors, sites, llim: int = -1, rlim: int | None = None):
        self.tensors = list(tensors)
        self.sites = list(sites)
        self.llim = llim
        self.rlim = len(self.tensors) if rlim is None else rlim

    def __len__(self):
        return len(self.tensors)

    def __getitem__(self, j):
        return self.tensors[j]

    def __setitem__(self, j, v):
        self.tensors[j] = v

    @property
    def is_cuda(self):
        return all(t.is_cuda for t in self.tensors)

    def linkdims(self):
        return [t.dims[-1] for t in self.tensors[:-1]]

    def maxlinkdim(self):
        return max(self.linkdims(), default=1)

    def copy(self):
        return MPO([t.copy() for t in self.tensors], self.sites, self.llim, self.rlim)

    def prime(self, n: int = 1):
        """Every index (sites and links) raised n prime levels."""
        return MPO([T.prime(t, n) for t in self.tensors], [s.prime(n) for s in self.sites],
                   self.llim, self.rlim)

    def __str__(self):
        return _show("MPO", self.tensors)

    def __add__(self, other):
        from .mpsops import add
        return add(self, other)

    def _cu(self):
        return MPO([cu(t) for t in self.tensors], self.sites, self.llim, self.rlim)

    def _cpu(self):
        return MPO([cpu(t) for t in self.tensors], self.sites, self.llim, self.rlim)


def _show(kind, tensors):
    """One header line, one line per site, and a closing newline (show(::MPS))."""
    lines = [kind] + [f"[{j + 1}] " + ", ".join(f"({i.dim}|{i.tags}|{i.plev})" for i in t.inds)
                      for j, t in enumerate(tensors)]
    return "\n".join(lines) + "\n"


def cuMPS(x=None, states=None):
    """Device MPS (src/mps/cumps.jl:1-43,99-134).

    cuMPS() is empty; cuMPS(psi) copies an MPS to the device; cuMPS(sites) is
    the zero MPS with dimension-1 links; cuMPS(sites, states) is a product
    state, and a states list of the wrong length raises DimensionMismatch.
    """
    if x is None:
        return MPS([], [])
    if isinstance(x, MPS):
        return cu(x)
    sites = list(x)
    if states is not None:
        return productCuMPS(sites, states)
    N = len(sites)
    L = _links(N, [1] * (N - 1))
    return MPS([T.cuITensor(L[j], s, L[j + 1]) for j, s in enumerate(sites)], sites, -1, N)


def cuMPO(x=None):
    """Device MPO (src/mps/cumpo.jl:1-13): cuMPO() is empty, cuMPO(H) copies
    an MPO to the device, cuMPO(sites) is the zero MPO with dimension-1 links."""
    if x is None:
        return MPO([], [])
    if isinstance(x, MPO):
        return cu(x)
    sites = list(x)
    N = len(sites)
    W = [Index(1, f"Link,w={j}") for j in range(N + 1)]
    return MPO([T.cuITensor(W[j], s.prime(), s, W[j + 1]) for j, s in enumerate(sites)], sites)


def _links(N, dims):
    return [Index(1, "Link,l=0")] + [Index(dims[j], f"Link,l={j + 1}") for j in range(N - 1)] + \
           [Index(1, f"Link,l={N}")]


def random_linkdims(sites, linkdim: int):
    N = len(sites)
    out = []
    for j in range(N - 1):
        left = int(np.prod([s.dim for s in sites[: j + 1]], dtype=np.float64)) if j < 40 else 1 << 60
        right = int(np.prod([s.dim for s in sites[j + 1:]], dtype=np.float64)) if N - j - 1 < 40 else 1 << 60
        out.append(int(min(linkdim, left, right)))
    return out


def randomCuMPS(sites, linkdim: int = 1, seed: int = 1234):
    """Random device MPS (randomCuMPS, src/mps/cumps.jl:44-53).

    Site j is filled with N(0,1) numbers from the library's Philox stream
    (seed, offset j), so the CPU oracle can rebuild the same tensors, and is
    then scaled to unit norm (randn! + normalize! per site).  The state as a
    whole is not normalised or orthogonalised here; dmrg() does both.
    """
    N = len(sites)
    ld = random_linkdims(sites, linkdim)
    L = _links(N, ld)
    h = T._h()
    ts = []
    for j in range(N):
        inds = (L[j], sites[j], L[j + 1])
        n = T.dim(inds)
        t = T.empty_dev(n)
        h.call("itg_random_normal", C.c_int64(n), C.c_uint64(seed), C.c_uint64(j), T._ptr(t))
        nrm = C.c_double()
        h.call("itg_nrm2", C.c_int64(n), T._ptr(t), C.byref(nrm))
        h.call("itg_scal", C.c_int64(n), C.c_double(1.0 / nrm.value), T._ptr(t))
        ts.append(ITensor(Dense(t), inds))
    return MPS(ts, sites, -1, N)


def productMPS_host(sites, states):
    """Host product state; states are names ("Up", "Dn", "Z0"), ints (1-based) or a function."""
    N = len(sites)
    if callable(states):
        states = [states(j + 1) for j in range(N)]
    if isinstance(states, str):
        states = [states] * N
    if len(states) != N:
        raise DimensionMismatch(2, f"{len(states)} initial states for {N} sites")
    L = _links(N, [1] * (N - 1))
    ts = []
    for j, s in enumerate(sites):
        k = _STATE_NAMES[s.dim][s_] if isinstance((s_ := states[j]), str) else int(s_) - 1
        arr = np.zeros((1, s.dim, 1))
        arr[0, k, 0] = 1.0
        ts.append(T.ITensor_host(arr, L[j], s, L[j + 1]))
    return MPS(ts, sites)


def productCuMPS(sites, states):
    """Device product state (productCuMPS, src/mps/cumps.jl:58-134)."""
    return cu(productMPS_host(sites, states))


# ------------------------------------------------------------------- MPOs
def _mpo_from_W(sites, W_of_site, first_row: int, last_col: int) -> MPO:
    """Build an MPO from per-site operator-valued matrices W[a][b] (d x d each).

    H = e_first^T W_1 W_2 ... W_N e_last, with the left boundary selecting row
    `first_row` of W_1 and the right boundary column `last_col` of W_N.
    """
    N = len(sites)
    tens = []
    wdims = []
    for j in range(N):
        Wj = W_of_site(j)  # array (wl, wr, d, d) : Wj[a, b] = operator matrix [s', s]
        if j == 0:
            Wj = Wj[first_row: first_row + 1]
        if j == N - 1:
            Wj = Wj[:, last_col: last_col + 1]
        tens.append(Wj)
        wdims.append(Wj.shape[1])
    links = [Index(1, "Link,w=0")] + [Index(wdims[j], f"Link,w={j + 1}") for j in range(N - 1)] + \
            [Index(1, f"Link,w={N}")]
    out = []
    for j in range(N):
        Wj = tens[j]                                   # (wl, wr, s', s)
        arr = np.transpose(Wj, (0, 2, 3, 1))           # (wl, s', s, wr)
        s = sites[j]
        out.append(T.ITensor_host(arr, links[j], s.prime(), s, links[j + 1]))
    return MPO(out, sites)


def xxz_mpo(sites, J=1.0, Delta=1.0, h=0.0) -> MPO:
    """H = sum_i J_i (Sx Sx + Sy Sy + Delta_i Sz Sz)_{i,i+1} + h sum_i Sz_i.

    J and Delta may be scalars or per-bond sequences (length N-1).  Bond dim 5.
    States: 4 = nothing placed yet, 1..3 = S+, S-, Sz placed on the left,
    0 = term complete.
    """
    N = len(sites)
    Js = np.broadcast_to(np.asarray(J, dtype=float), (max(N - 1, 1),))
    Ds = np.broadcast_to(np.asarray(Delta, dtype=float), (max(N - 1, 1),))

    def W(j):
        o = spin_ops(sites[j].dim)
        d = sites[j].dim
        w = np.zeros((5, 5, d, d))
        w[0, 0] = o["Id"]
        w[4, 4] = o["Id"]
        w[1, 0] = o["S-"]
        w[2, 0] = o["S+"]
        w[3, 0] = o["Sz"]
        if j < N - 1:
            w[4, 1] = 0.5 * Js[j] * o["S+"]
            w[4, 2] = 0.5 * Js[j] * o["S-"]
            w[4, 3] = Js[j] * Ds[j] * o["Sz"]
        w[4, 0] = h * o["Sz"]
        return w

    return _mpo_from_W(sites, W, 4, 0)


def heisenberg_mpo(sites, J=1.0) -> MPO:
    """S=1/2 (or S=1) Heisenberg chain H = J sum_i S_i . S_{i+1}, open boundaries."""
    return xxz_mpo(sites, J=J, Delta=1.0)


def tfim_mpo(sites, h=0.5, J=1.0) -> MPO:
    """Transverse-field Ising chain H = -J sum Sz_i Sz_{i+1} - h sum Sx_i (test/dmrg.jl:62-69)."""

    def W(j):
        o = spin_ops(sites[j].dim)
        d = sites[j].dim
        w = np.zeros((3, 3, d, d))
        w[0, 0] = o["Id"]
        w[2, 2] = o["Id"]
        w[1, 0] = o["Sz"]
        w[2, 1] = -J * o["Sz"]
        w[2, 0] = -h * o["Sx"]
        return w

    return _mpo_from_W(sites, W, 2, 0)


def j1j2_mpo(sites, J1=1.0, J2=0.0) -> MPO:
    """H = J1 sum S_i.S_{i+1} + J2 sum S_i.S_{i+2}; bond dimension 8.

    States: 7 = nothing placed, 1..3 = (S+, S-, Sz) placed one site to the left,
    4..6 = the same placed two sites to the left, 0 = complete.
    """
    N = len(sites)

    def W(j):
        o = spin_ops(sites[j].dim)
        d = sites[j].dim
        A = [o["S+"], o["S-"], o["Sz"]]
        B = [0.5 * o["S-"], 0.5 * o["S+"], o["Sz"]]
        w = np.zeros((8, 8, d, d))
        w[0, 0] = o["Id"]
        w[7, 7] = o["Id"]
        for k in range(3):
            w[7, 1 + k] = A[k]
            w[1 + k, 0] = J1 * B[k]
            w[1 + k, 4 + k] = o["Id"]
            w[4 + k, 0] = J2 * B[k]
        return w

    return _mpo_from_W(sites, W, 7, 0)
