"""MPS / MPO operations either side of the DMRG sweep, on device storage.

Mirrors the MPS/MPO functions the reference's tests drive through its storage
plugin (test/test_cumps.jl:76-246, test/test_cumpo.jl:31-173); their
algorithms live in ITensors 0.2 (mps/abstractmps.jl, mps/mpo.jl):

* ``orthogonalize_`` (orthogonalize!): QR gauge moves, or truncating SVD
  moves when maxdim / cutoff is given;
* ``replacebond_`` (replacebond!): split a two-site tensor back into the chain
  with ITensors' gauge-limit bookkeeping;
* ``truncate_`` (truncate!): left-orthogonalise, then a right-to-left sweep of
  truncated SVDs;
* ``inner(phi, psi)`` and ``inner(phi, A, psi)``;
* ``contract(A::MPO, psi::MPS)`` and ``contract(A::MPO, B::MPO)``: exact
  site-by-site products with fused links, then ``truncate_`` when maxdim or
  cutoff is given;
* ``add`` / ``+`` for MPS and MPO: direct sum of the link spaces through 0/1
  embedding tensors, then ``truncate_`` with the caller's keywords;
* ``normalize_``, ``randomCuMPO``, ``linkind``, ``siteind``, ``leftlim``,
  ``rightlim``, ``maxlinkdim``, ``dag``.

Python spells Julia's in-place ``f!`` as ``f_``.  Sites and bonds are 0-based:
bond j joins sites j and j+1.  The gauge limits are ITensors' shifted by one:
llim = -1 and rlim = N mean nothing is known to be orthogonal, and an
orthogonality centre at site c has llim = c-1, rlim = c+1.

Layout: MPS site tensor (l, s, r); MPO site tensor (wl, x, y, wr) with two
site indices in the middle.  End links have dimension 1.  Every product and
sum is a libitg.so call (itg_contract, itg_axpby_permuted, itg_qr,
itg_factorize_trunc, itg_nrm2); torch only allocates.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import tensor as T
from ._lib import PREC_FP64, DimensionMismatch, i32arr, i64arr
from .dmrg import _contract_raw, inner as _inner2
from .mps import MPO, MPS
from .tensor import Dense, ITensor, Index


class ArgumentError(ValueError):
    """Raised where the reference raises Julia's ArgumentError."""


# ------------------------------------------------------------------ helpers
def _pc(A: ITensor, la, B: ITensor, lb, lc):
    """Contract A and B by positional labels; the result's modes are `lc`.

    Labels shared by A and B and absent from `lc` are summed.  Returns the flat
    device buffer and its dims.
    """
    dims = {}
    for t, ls in ((A, la), (B, lb)):
        if len(ls) != len(t.inds):
            raise DimensionMismatch(2, "label count != tensor order")
        for lab, d in zip(ls, t.dims):
            if dims.setdefault(lab, d) != d:
                raise DimensionMismatch(2, f"dimension of {lab!r} differs between operands")
    code = {lab: k + 1 for k, lab in enumerate(dims)}
    dC = tuple(dims[lab] for lab in lc)
    if A.is_complex or B.is_complex:
        out = T.empty_dev(int(np.prod(dC)) if dC else 1, True)
        one, zero = (C.c_double * 2)(1.0, 0.0), (C.c_double * 2)(0.0, 0.0)
        T._h().call("itg_contract_z", T._dt(A), T._dt(B), one, T._ptr(A.store.data), len(la), i64arr(A.dims),
                    i32arr([code[x] for x in la]), T._ptr(B.store.data), len(lb), i64arr(B.dims),
                    i32arr([code[x] for x in lb]), zero, T._ptr(out), len(lc), i64arr(dC),
                    i32arr([code[x] for x in lc]), PREC_FP64)
        return out, dC
    out = _contract_raw(T._h(), A.store.data, A.dims, [code[x] for x in la], B.store.data, B.dims,
                        [code[x] for x in lb], dC, [code[x] for x in lc])
    return out, dC


def _check_len(A, B, what):
    if len(A) != len(B):
        raise DimensionMismatch(2, f"{what}: lengths {len(A)} and {len(B)} differ")


def _mid(t: ITensor):
    return t.inds[1:-1]


from .tensor import dag  # noqa: E402  (re-exported: conjugates complex site tensors)


def linkind(M, j: int) -> Index:
    """Index of bond j (between sites j and j+1)."""
    return M[j].inds[-1]


def siteind(M: MPS, j: int) -> Index:
    return M[j].inds[1]


def leftlim(M) -> int:
    return M.llim


def rightlim(M) -> int:
    return M.rlim


def maxlinkdim(M) -> int:
    return max((t.inds[-1].dim for t in M.tensors[:-1]), default=1)


def _with_inds(t: ITensor, inds) -> ITensor:
    return ITensor(t.store, inds)


# --------------------------------------------------------------- gauge moves
def _move_right(M, b: int, trunc: dict | None):
    """Make site b left-orthogonal and push the remainder into site b+1."""
    A = M[b]
    r = A.inds[-1]
    left = A.inds[:-1]
    if trunc is None:
        Q, R = T.qr(A, *left)
        q = Q.inds[-1]
    else:
        Q, R, _ = T.factorize(A, *left, ortho="left", **trunc)
        q = Q.inds[-1]
    nq = Index(q.dim, r.tags)
    M[b] = Q.replaceinds([q], [nq])
    R = R.replaceinds([q], [nq])                       # (nq, r)
    nxt = M[b + 1]
    out, dC = _pc(R, ("q", "r"), nxt, ("r",) + tuple(range(len(nxt.inds) - 1)),
                  ("q",) + tuple(range(len(nxt.inds) - 1)))
    M[b + 1] = ITensor(Dense(out), (nq,) + nxt.inds[1:])


def _move_left(M, b: int, trunc: dict | None):
    """Make site b right-orthogonal and push the remainder into site b-1."""
    A = M[b]
    l = A.inds[0]
    right = A.inds[1:]
    if trunc is None:
        Q, R = T.qr(A, *right)                       # Q (right..., q), R (q, l)
        q = Q.inds[-1]
        Lf = R
    else:
        Lf, Q, _ = T.factorize(A, l, ortho="right", **trunc)   # Lf (l, q), Q (right..., q)
        q = Q.inds[-1]
    nq = Index(q.dim, l.tags)
    Q = Q.replaceinds([q], [nq])
    M[b] = T.permute(Q, nq, *right)
    Lf = Lf.replaceinds([q], [nq])
    prv = M[b - 1]
    n = len(prv.inds)
    out, dC = _pc(prv, tuple(range(n - 1)) + ("l",), Lf, ("l", "q") if Lf.inds[0] == l else ("q", "l"),
                  tuple(range(n - 1)) + ("q",))
    M[b - 1] = ITensor(Dense(out), prv.inds[:-1] + (nq,))


def _trunc_kw(kw):
    keys = ("maxdim", "mindim", "cutoff", "absoluteCutoff", "doRelCutoff", "use_absolute_cutoff",
            "use_relative_cutoff", "method", "precision")
    t = {k: v for k, v in kw.items() if k in keys and v is not None}
    return t if ("maxdim" in t or "cutoff" in t) else None


def orthogonalize_(M, j: int, *, normalize: bool = False, **kw):
    """Move the orthogonality centre of an MPS or MPO to site j (orthogonalize!).

    Without maxdim / cutoff each move is a QR (itg_qr); with them it is a
    truncated SVD (itg_factorize_trunc).  Gauge limits follow ITensors:
    afterwards llim = j-1 and rlim = j+1.  normalize=True scales the centre
    tensor to unit norm.
    """
    N = len(M)
    if not 0 <= j < N:
        raise DimensionMismatch(2, f"orthogonalize: site {j} outside 0..{N - 1}")
    trunc = _trunc_kw(kw)
    while M.llim < j - 1:
        b = M.llim + 1
        _move_right(M, b, trunc)
        M.llim = b
        if M.rlim < M.llim + 2:
            M.rlim = M.llim + 2
    while M.rlim > j + 1:
        b = M.rlim - 1
        _move_left(M, b, trunc)
        M.rlim = b
        if M.llim > M.rlim - 2:
            M.llim = M.rlim - 2
    if normalize:
        M[j] = M[j] / T.norm(M[j])
    return M


def replacebond_(M: MPS, b: int, phi: ITensor, *, ortho: str = "left", **kw):
    """Split the two-site tensor phi on bond b into sites b, b+1 (replacebond!).

    The new link keeps the old link's tags.  ortho="left" leaves site b
    left-orthogonal, "right" leaves site b+1 right-orthogonal; the gauge
    limits move only when they bordered the bond, as in ITensors.  Returns the
    truncation spectrum.
    """
    if ortho not in ("left", "right"):
        raise ArgumentError(f"replacebond!: ortho must be 'left' or 'right', not {ortho!r}")
    l, s1 = M[b].inds[0], M[b].inds[1]
    s2, r = M[b + 1].inds[1], M[b + 1].inds[2]
    old = linkind(M, b)
    if set(phi.inds) != {l, s1, s2, r}:
        raise DimensionMismatch(2, "replacebond!: phi must carry the indices of sites b and b+1")
    tkw = {k: v for k, v in kw.items() if v is not None}
    L, R, spec = T.factorize(phi, l, s1, ortho=ortho, **tkw)   # L (l, s1, q), R (q, s2, r)
    q = L.inds[-1]
    nq = Index(q.dim, old.tags)
    M[b] = T.permute(L.replaceinds([q], [nq]), l, s1, nq)
    M[b + 1] = T.permute(R.replaceinds([q], [nq]), nq, s2, r)
    if ortho == "left":
        if M.llim == b - 1:
            M.llim = b
        if M.rlim == b + 1:
            M.rlim = b + 2
    else:
        if M.llim == b:
            M.llim = b - 1
        if M.rlim == b + 2:
            M.rlim = b + 1
    return spec


def truncate_(M, **kw):
    """Truncate every bond of an MPS or MPO (truncate!).

    Left-orthogonalise by QR, then sweep right to left with truncated SVDs
    (maxdim, mindim, cutoff, ...); afterwards the centre is site 0
    (llim = -1, rlim = 1).
    """
    N = len(M)
    orthogonalize_(M, N - 1)
    tkw = {k: v for k, v in kw.items() if v is not None}
    for j in range(N - 1, 0, -1):
        _move_left(M, j, tkw if tkw else {"cutoff": 0.0})
        M.rlim = j
        M.llim = min(M.llim, j - 2)
    return M


def normalize_(M):
    """Scale an MPS to unit norm (normalize!); the scale lands on the centre
    site when the gauge is known, else on site 0."""
    nrm = np.sqrt(abs(inner(M, M)))
    c = M.llim + 1 if M.llim + 2 == M.rlim else 0
    M[c] = M[c] / nrm
    return M


def norm(M) -> float:
    return float(np.sqrt(abs(inner(M, M))))


# ------------------------------------------------------------------- inner
def inner(*args):
    """inner(phi, psi) = <phi|psi>, or inner(phi, A, psi) = <phi|A|psi>.

    For <phi|A|psi> the MPO's input index at each site is psi's site index and
    its output index is phi's site index or its prime (test/test_cumpo.jl:42-98).
    Lengths or site indices that do not line up raise DimensionMismatch.
    """
    if len(args) == 2:
        phi, psi = args
        _check_len(phi, psi, "inner")
        for j in range(len(psi)):
            if phi[j].inds[1].dim != psi[j].inds[1].dim:
                raise DimensionMismatch(2, f"inner: site {j} dimensions differ")
        phi, psi = T.cu(phi), T.cu(psi)
        if not any(t.is_complex for t in phi.tensors + psi.tensors):
            return _inner2(phi, psi)
        # complex: E[a, b] -> sum conj(phi[a, s, a2]) E[a, b] psi[b, s, b2]
        E = ITensor(Dense(T.empty_dev(1).fill_(1.0)), (Index(1), Index(1)))
        for j in range(len(psi)):
            t1, d1 = _pc(E, ("a", "b"), psi[j], ("b", "s", "b2"), ("a", "s", "b2"))
            t1 = ITensor(Dense(t1), tuple(Index(d) for d in d1))
            e, de = _pc(T.dag(phi[j]), ("a", "s", "a2"), t1, ("a", "s", "b2"), ("a2", "b2"))
            E = ITensor(Dense(e), tuple(Index(d) for d in de))
        return complex(E.store.data[0].item())
    if len(args) != 3:
        raise ArgumentError("inner takes (phi, psi) or (phi, A, psi)")
    phi, A, psi = (T.cu(x) for x in args)
    _check_len(phi, psi, "inner")
    _check_len(A, psi, "inner")
    E = ITensor(Dense(T.empty_dev(1).fill_(1.0)), (Index(1), Index(1), Index(1)))
    for j in range(len(psi)):
        P, W, X = phi[j], A[j], psi[j]
        ket, bra = _mpo_roles(W, X.inds[1], phi_site=P.inds[1])
        wl = ["wl", "o", "k", "wr"] if (W.inds[1] == bra) else ["wl", "k", "o", "wr"]
        t1, d1 = _pc(E, ("a", "wl", "b"), X, ("b", "k", "b2"), ("a", "wl", "k", "b2"))
        t1 = ITensor(Dense(t1), tuple(Index(d) for d in d1))
        t2, d2 = _pc(t1, ("a", "wl", "k", "b2"), W, tuple(wl), ("a", "o", "b2", "wr"))
        t2 = ITensor(Dense(t2), tuple(Index(d) for d in d2))
        e, de = _pc(t2, ("a", "o", "b2", "wr"), T.dag(P), ("a", "o", "a2"), ("a2", "wr", "b2"))
        E = ITensor(Dense(e), tuple(Index(d) for d in de))
    v = E.store.data[0].item()
    return complex(v) if E.is_complex else float(v)


def _mpo_roles(W: ITensor, ket_site: Index, phi_site: Index | None = None):
    """(input, output) site indices of MPO tensor W acting on ket_site."""
    x, y = W.inds[1], W.inds[2]
    if y == ket_site:
        ket, bra = y, x
    elif x == ket_site:
        ket, bra = x, y
    elif x.id == ket_site.id and y.id == ket_site.id and x.plev != y.plev:
        # both are prime levels of the MPS's site index (a primed MPO such as
        # prime(K) acting on an unprimed MPS): the lower level is the input
        ket, bra = (x, y) if x.plev < y.plev else (y, x)
    else:
        raise DimensionMismatch(2, "MPO and MPS site indices do not match")
    if phi_site is not None and not (bra == phi_site or bra == phi_site.prime(1)):
        raise DimensionMismatch(2, "MPO output index does not match the bra's site index")
    return ket, bra


# --------------------------------------------------------------- products
def _fused_links(N, dl, tags):
    return [Index(int(dl[j]), tags[j]) for j in range(N + 1)]


def contract(A, B, *, method: str = "densitymatrix", **kw):
    """contract(A::MPO, psi::MPS) or contract(A::MPO, B::MPO).

    The product is formed exactly, site by site (one itg_contract per site
    into fused links of dimension dim(A link) * dim(B link)).  When maxdim or
    cutoff is given it is then truncated by ``truncate_``: a canonical
    right-to-left SVD sweep, which keeps at every bond the leading eigenvectors
    of the reduced density matrix of the product given the bonds already
    truncated — the truncation the density-matrix algorithm makes.  Both
    method names run this path; any other raises ArgumentError.

    MPO x MPS: the MPO's input index matches psi's site index (or, for an
    MPO whose two site indices are both prime levels of it, the lower one);
    the result lives on the unprimed output index.  MPO x MPO: the one site index the two
    share is summed (if they share both, A's input is summed with B's output);
    an output index at prime level 2 over an input at level 0 is mapped to
    level 1.
    """
    if method not in ("densitymatrix", "naive"):
        raise ArgumentError(f"contract: unknown method {method!r}")
    A, B = T.cu(A), T.cu(B)
    _check_len(A, B, "contract")
    if isinstance(B, MPS):
        R = _mpo_mps(A, B)
    elif isinstance(B, MPO):
        R = _mpo_mpo(A, B)
    else:
        raise ArgumentError("contract: second argument must be an MPS or an MPO")
    tkw = _trunc_kw(kw)
    if tkw is not None:
        truncate_(R, **tkw)
    return R


def _mpo_mps(A: MPO, psi: MPS) -> MPS:
    N = len(psi)
    dl = [A[0].inds[0].dim * psi[0].inds[0].dim] + \
         [A[j].inds[-1].dim * psi[j].inds[-1].dim for j in range(N)]
    links = _fused_links(N, dl, ["Link,l=0"] + [psi[j].inds[-1].tags for j in range(N)])
    out, sites = [], []
    for j in range(N):
        W, X = A[j], psi[j]
        ket, bra = _mpo_roles(W, X.inds[1])
        wl = ("wl", "o", "k", "wr") if W.inds[1] == bra else ("wl", "k", "o", "wr")
        buf, d = _pc(W, wl, X, ("l", "k", "r"), ("l", "wl", "o", "r", "wr"))
        s = bra.noprime()
        sites.append(s)
        out.append(ITensor(Dense(buf), (links[j], s, links[j + 1])))
    return MPS(out, sites, -1, N)


def _mpo_mpo(A: MPO, B: MPO) -> MPO:
    N = len(A)
    dl = [A[0].inds[0].dim * B[0].inds[0].dim] + [A[j].inds[-1].dim * B[j].inds[-1].dim for j in range(N)]
    links = _fused_links(N, dl, ["Link,w=0"] + [A[j].inds[-1].tags for j in range(N)])
    out = []
    for j in range(N):
        Wa, Wb = A[j], B[j]
        a1, a2 = Wa.inds[1], Wa.inds[2]
        b1, b2 = Wb.inds[1], Wb.inds[2]
        common = [i for i in (a1, a2) if i in (b1, b2)]
        if len(common) == 1:
            c = common[0]
            ka = a2 if a1 == c else a1
            kb = b2 if b1 == c else b1
            la = ("wl", "c", "ka", "wr") if a1 == c else ("wl", "ka", "c", "wr")
            lb = ("vl", "c", "kb", "vr") if b1 == c else ("vl", "kb", "c", "vr")
        elif len(common) == 2:
            # both carry (x', x): operator product, A's input against B's output
            hi_a, lo_a = (a1, a2) if a1.plev > a2.plev else (a2, a1)
            hi_b, lo_b = (b1, b2) if b1.plev > b2.plev else (b2, b1)
            ka, kb = hi_a, lo_b
            la = ("wl", "ka", "c", "wr") if a1 == hi_a else ("wl", "c", "ka", "wr")
            lb = ("vl", "c", "kb", "vr") if b1 == hi_b else ("vl", "kb", "c", "vr")
        else:
            raise DimensionMismatch(2, f"contract: MPO site indices at site {j} do not match")
        buf, d = _pc(Wa, la, Wb, lb, ("wl", "vl", "ka", "kb", "wr", "vr"))
        if ka.plev == 2 and kb.plev == 0 and ka.id == kb.id:
            ka = ka.prime(-1)
        out.append(ITensor(Dense(buf), (links[j], ka, kb, links[j + 1])))
    R = MPO(out, A.sites)
    return R


# -------------------------------------------------------------------- sums
def _embed(n_from: int, n_to: int, offset: int) -> ITensor:
    e = np.zeros((n_from, n_to))
    e[np.arange(n_from), offset + np.arange(n_from)] = 1.0
    return T.cu(T.ITensor_host(e, Index(n_from), Index(n_to)))


def add(A, B, **kw):
    """A + B for two MPS or two MPO on the same site indices (add / +).

    Direct sum of the link spaces: every site tensor of A and of B is placed
    into its block of the summed links by contraction with 0/1 embedding
    tensors (exact in FP64) and the two placements are added; the end sites
    share their dimension-1 outer links.  The sum is then passed through
    ``truncate_`` with the caller's keywords (maxdim, cutoff, ...).
    """
    A, B = T.cu(A), T.cu(B)
    _check_len(A, B, "add")
    if type(A) is not type(B):
        raise ArgumentError("add: both arguments must be MPS or both MPO")
    N = len(A)
    for j in range(N):
        if set(_mid(A[j])) != set(_mid(B[j])):
            raise DimensionMismatch(2, f"add: site indices at site {j} differ")
    if N == 1:
        t = T._axpby(1.0, T.permute(B[0].replaceinds([B[0].inds[0], B[0].inds[-1]],
                                                     [A[0].inds[0], A[0].inds[-1]]), *A[0].inds),
                     1.0, A[0])
        C = A.copy() if isinstance(A, MPS) else MPO([t], A.sites)
        C[0] = t
        return C
    da = [A[j].inds[-1].dim for j in range(N - 1)]
    db = [B[j].inds[-1].dim for j in range(N - 1)]
    links = [A[0].inds[0]] + [Index(da[j] + db[j], A[j].inds[-1].tags) for j in range(N - 1)] + \
            [A[N - 1].inds[-1]]
    out = []
    for j in range(N):
        mid = _mid(A[j])
        parts = []
        for X, dims, off in ((A[j], da, 0), (B[j], db, None)):
            t = X
            labels = ["L"] + [mid.index(i) for i in _mid(X)] + ["R"]
            cur = list(labels)
            if j < N - 1:
                o = 0 if off == 0 else da[j]
                E = _embed(dims[j], da[j] + db[j], o)
                buf, d = _pc(t, tuple(cur), E, ("R", "Rn"), tuple(x if x != "R" else "Rn" for x in cur))
                cur = [x if x != "R" else "Rn" for x in cur]
                t = ITensor(Dense(buf), tuple(Index(k) for k in d))
            if j > 0:
                o = 0 if off == 0 else da[j - 1]
                E = _embed(dims[j - 1], da[j - 1] + db[j - 1], o)
                buf, d = _pc(E, ("L", "Ln"), t, tuple(cur), tuple(x if x != "L" else "Ln" for x in cur))
                cur = [x if x != "L" else "Ln" for x in cur]
                t = ITensor(Dense(buf), tuple(Index(k) for k in d))
            # order the modes as (L, mid..., R) of A
            want = [cur[0]] + list(range(len(mid))) + [cur[-1]]
            if cur != want:
                src = ITensor(t.store, tuple(Index(k) for k in t.dims))
                pos = [cur.index(w) for w in want]
                t = T.permute(src, *[src.inds[p] for p in pos])
            parts.append(_with_inds(t, (links[j],) + tuple(mid) + (links[j + 1],)))
        out.append(T._axpby(1.0, parts[1], 1.0, parts[0]) if parts[0].is_complex == parts[1].is_complex
                   else T._axpby(1.0, T.complex_(parts[1]), 1.0, T.complex_(parts[0])))
    if isinstance(A, MPS):
        C = MPS(out, A.sites, -1, N)
    else:
        C = MPO(out, A.sites)
    tkw = {k: v for k, v in kw.items() if v is not None}
    return truncate_(C, **tkw)


# ------------------------------------------------------- gate application
def apply(gates, psi: MPS, **kw) -> MPS:
    """Apply operator ITensors to an MPS in order (ITensors' apply / product,
    used by examples/gate_evolution.jl:43-46).

    Each gate carries primed output and unprimed input copies of the site
    indices it acts on (op(...)); its sites must be contiguous.  The
    orthogonality centre is first moved to the gate's first site, the sites'
    tensors are contracted with the gate, the output indices unprimed, and a
    multi-site result is split back site by site through itg_factorize_trunc
    with the caller's maxdim / cutoff (the centre ends on the gate's last
    site).  A one-site gate is applied in place.  Returns a new MPS.
    """
    if isinstance(gates, ITensor):
        gates = [gates]
    psi = T.cu(psi).copy()
    site_pos = {psi[j].inds[1]: j for j in range(len(psi))}
    tkw = {k: v for k, v in kw.items() if v is not None}
    for G in gates:
        ns = sorted(site_pos[i] for i in G.inds if i in site_pos)
        if not ns or len(ns) * 2 != len(G.inds):
            raise DimensionMismatch(2, "apply: gate indices must be (s', s) pairs of the MPS's sites")
        if ns != list(range(ns[0], ns[0] + len(ns))):
            raise ArgumentError("apply: gates on non-contiguous sites are not supported")
        for j in ns:
            if psi[j].inds[1].prime() not in G.inds:
                raise DimensionMismatch(2, "apply: gate lacks the primed output index of a site")
        if len(ns) == 1:
            j = ns[0]
            l, s, r = psi[j].inds
            t = T.contract(G, psi[j])                          # (s', l, r)
            t = t.replaceinds([s.prime()], [s])
            psi[j] = T.permute(t, l, s, r)
            psi.llim = min(psi.llim, j - 1)
            psi.rlim = max(psi.rlim, j + 1)
            continue
        orthogonalize_(psi, ns[0])
        phi = psi[ns[0]]
        for j in ns[1:]:
            phi = T.contract(phi, psi[j])
        phi = T.contract(G, phi)
        phi = phi.replaceinds([psi[j].inds[1].prime() for j in ns], [psi[j].inds[1] for j in ns])
        # split left to right: each site left-orthogonal, the centre moves along
        for j in ns[:-1]:
            l, s = psi[j].inds[0], psi[j].inds[1]
            old = psi[j].inds[2]
            L, R, _ = T.factorize(phi, l, s, ortho="left", **tkw)
            q = L.inds[-1]
            nq = Index(q.dim, old.tags)
            psi[j] = T.permute(L.replaceinds([q], [nq]), l, s, nq)
            phi = R.replaceinds([q], [nq])
        last = ns[-1]
        psi[last] = T.permute(phi, phi.inds[0], psi[last].inds[1], psi[last].inds[2])
        psi.llim, psi.rlim = last - 1, last + 1
    return psi


# ------------------------------------------------------------ constructors
def randomCuMPO(sites, *, seed: int | None = None) -> MPO:
    """Random link-dimension-1 MPO: each site tensor (1, s', s, 1) has N(0,1)
    entries (library Philox stream) scaled to unit norm (randomMPO, used by
    test/test_cumpo.jl:23-24)."""
    N = len(sites)
    links = [Index(1, f"Link,w={j}") for j in range(N + 1)]
    ts = []
    for j, s in enumerate(sites):
        t = T.randomCuITensor(links[j], s.prime(), s, links[j + 1], seed=seed if seed is None else seed + j)
        ts.append(t / T.norm(t))
    return MPO(ts, sites)
