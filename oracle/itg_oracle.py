"""CPU oracle for the two-site DMRG hot path — TEST INFRASTRUCTURE ONLY.

This module is test infrastructure.  Only tests/, __graft_entry__.smoke() and the
cpu_baseline / --impl reference legs of bench.py may import it.  The product
(libitg.so and the itg package) never calls it.

It restates, in NumPy/SciPy FP64, what the reference path computes:

* mode-labelled pairwise contraction with column-major storage: the label
  rules of _contract! (src/tensor/cudense.jl:255-283) and the scalar / outer /
  general split of contract!! (src/tensor/cudense.jl:83-110);
* permute! and permuted +/- (src/tensor/cudense.jl:333-500);
* Diag x Dense / Diag x Diag contraction (src/tensor/cudiag.jl:105-161);
* truncate! in two forms: the reference GPU rule, step by step
  (src/tensor/cutruncate.jl:1-93), and ITensors' CPU rule (cumulative discarded
  weight; NDTensors truncate!, ITensors 0.2 — an external dependency pinned at
  "0.2" in Project.toml:21, restated from its documented behaviour);
* svd / eigen / qr output conventions (src/tensor/culinearalgebra.jl:33-121);
* ITensors 0.2's dmrg two-site sweep (external; restated) with the same
  Davidson eigensolver the library uses;
* exact diagonalisation in the Sz = 0 sector for N <= 20 and the closed-form
  critical TFIM energy of test/dmrg.jl:79.

Pinning: the truncation restatement is checked against the reference's only
golden vectors (test/test_cutruncate.jl:9-17) and the DMRG restatement against
the known answers of test/dmrg.jl (TFIM closed form, S=1 Heisenberg bound)
and exact diagonalisation.  Contraction, permutation and factorisation are
pinned by einsum / LAPACK on the same inputs and by the reference's exact
identities (test/test_cuitensor.jl:29-54,89-130).  DMRG energies at 1e-10 are
not pinned by any reference number (none exists); they are pinned by ED.
"""
from __future__ import annotations

import math
import string

import numpy as np

# ------------------------------------------------------------- Philox normals
_M0, _M1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
_W0, _W1 = np.uint64(0x9E3779B9), np.uint64(0xBB67AE85)
_MASK32 = np.uint64(0xFFFFFFFF)


def philox_normal(n: int, seed: int, offset: int = 0) -> np.ndarray:
    """Same stream as itg_random_normal: Philox-4x32-10 (Salmon et al. 2011) + Box-Muller."""
    npairs = (n + 1) // 2
    p = np.arange(npairs, dtype=np.uint64)
    c0 = p & _MASK32
    c1 = p >> np.uint64(32)
    c2 = np.full(npairs, np.uint64(offset) & _MASK32, dtype=np.uint64)
    c3 = np.full(npairs, np.uint64(offset) >> np.uint64(32), dtype=np.uint64)
    k0 = np.uint64(seed) & _MASK32
    k1 = np.uint64(seed) >> np.uint64(32)
    for _ in range(10):
        p0 = _M0 * c0
        p1 = _M1 * c2
        hi0, lo0 = p0 >> np.uint64(32), p0 & _MASK32
        hi1, lo1 = p1 >> np.uint64(32), p1 & _MASK32
        c0, c1, c2, c3 = (hi1 ^ c1 ^ k0) & _MASK32, lo1, (hi0 ^ c3 ^ k1) & _MASK32, lo0
        k0 = (k0 + _W0) & _MASK32
        k1 = (k1 + _W1) & _MASK32
    a = ((c0 << np.uint64(32)) | c1) >> np.uint64(11)
    b = ((c2 << np.uint64(32)) | c3) >> np.uint64(11)
    u = (a.astype(np.float64) + 0.5) * 2.0 ** -53
    v = (b.astype(np.float64) + 0.5) * 2.0 ** -53
    r = np.sqrt(-2.0 * np.log(u))
    out = np.empty(2 * npairs)
    out[0::2] = r * np.cos(2.0 * np.pi * v)
    out[1::2] = r * np.sin(2.0 * np.pi * v)
    return out[:n]


# ---------------------------------------------------------------- contraction
def _letters(labels_list):
    m = {}
    for labs in labels_list:
        for x in labs:
            if x not in m:
                m[x] = string.ascii_letters[len(m)]
    return m


def contract(A: np.ndarray, la, B: np.ndarray, lb, lc) -> np.ndarray:
    """C[lc] = sum A[la] B[lb] over labels not in lc (n-d arrays, index order = labels)."""
    m = _letters([la, lb, lc])
    spec = "".join(m[x] for x in la) + "," + "".join(m[x] for x in lb) + "->" + "".join(m[x] for x in lc)
    return np.einsum(spec, A, B, optimize=True)


def _exact_slices(X: np.ndarray, axis: int, nslices: int = 4, bits: int = 14):
    """Row (axis=1: rows of an M x K matrix) or column (axis=0) scaled integer
    slices of X: X = 2^e * sum_p s_p 2^(-bits (p + 1)) up to 2^(-bits nslices - 1)
    relative to the row maximum.  Balanced digits (round to nearest), so
    |s_0| <= 2^bits, |s_p| <= 2^(bits - 1) and the truncation residue has no
    bias; every s_p is an integer held exactly in FP64.  Returns (slices, e)."""
    mx = np.max(np.abs(X), axis=axis, keepdims=True)
    _, e = np.frexp(np.where(mx > 0, mx, 1.0))       # mx < 2^e
    r = np.ldexp(X, -e)                                # |r| < 1, exact (power-of-two scaling)
    out = []
    for _ in range(nslices):
        r = np.ldexp(r, bits)
        s = np.rint(r)
        out.append(s)
        r = r - s                                      # exact: |r - s| <= 1/2
    return out, e


def matmul_exact(A: np.ndarray, B: np.ndarray) -> np.ndarray:
    """A @ B for FP64 matrices with an error near one rounding of each output.

    Compensated checker for deep contractions (large K), where an FP64 BLAS
    product carries up to K * 2^-53 of rounding relative to |A| |B|.  Each row
    of A and column of B is split into balanced integer slices of 14 bits (4
    slices, truncation below 2^-57 of the row / column maximum); every slice
    product is a sum of integers below 2^(28 + log2 K), and each level's sum of
    at most four of them stays below 2^53 for K < 2^22, so BLAS computes them
    exactly in any summation order.  The levels p + q <= 3 are combined with
    Neumaier's compensated summation; the dropped levels are below 2^-54 of
    |A| |B| and, the digits being balanced, add up without bias."""
    K = A.shape[1]
    if K >= (1 << 22):
        raise ValueError("matmul_exact: K too large for exact slice products")
    sa, ea = _exact_slices(A, axis=1)
    sb, eb = _exact_slices(B, axis=0)
    terms = []
    for L in range(4):
        acc = None
        for p in range(L + 1):
            t = sa[p] @ sb[L - p]                      # exact integers
            acc = t if acc is None else acc + t        # exact: < 2^(30 + log2 K) <= 2^53
        terms.append(np.ldexp(acc, -14 * (L + 2)))
    s = terms[0].copy()
    c = np.zeros_like(s)
    for t in terms[1:]:
        u = s + t
        c += np.where(np.abs(s) >= np.abs(t), (s - u) + t, (t - u) + s)
        s = u
    return np.ldexp(s + c, ea + eb)


def contract_exact(A: np.ndarray, la, B: np.ndarray, lb, lc) -> np.ndarray:
    """contract() through matmul_exact: the same labels and output order, the
    contracted labels folded into one GEMM depth."""
    la, lb, lc = list(la), list(lb), list(lc)
    con = [x for x in la if x in lb and x not in lc]
    fa = [x for x in la if x in lc]
    fb = [x for x in lb if x in lc]
    dims = {x: A.shape[i] for i, x in enumerate(la)}
    dims.update({x: B.shape[i] for i, x in enumerate(lb)})
    M = int(np.prod([dims[x] for x in fa], dtype=np.int64))
    N = int(np.prod([dims[x] for x in fb], dtype=np.int64))
    K = int(np.prod([dims[x] for x in con], dtype=np.int64))
    A2 = np.transpose(A, [la.index(x) for x in fa + con]).reshape(M, K)
    B2 = np.transpose(B, [lb.index(x) for x in con + fb]).reshape(K, N)
    C2 = matmul_exact(A2, B2).reshape([dims[x] for x in fa + fb])
    return np.transpose(C2, [(fa + fb).index(x) for x in lc])


def permute(A: np.ndarray, la, lb) -> np.ndarray:
    return np.transpose(A, [list(la).index(x) for x in lb])


def diag_dense(d: np.ndarray, dims_d, la, uniform: bool, T: np.ndarray, lt, lc) -> np.ndarray:
    """Diag x Dense by densifying the diagonal (what cudiag.jl:147-157 does)."""
    n = min(dims_d)
    D = np.zeros(dims_d)
    vals = np.full(n, d[0]) if uniform else np.asarray(d[:n])
    idx = np.arange(n)
    D[tuple([idx] * len(dims_d))] = vals
    return contract(D, la, T, lt, lc)


def flat(A: np.ndarray) -> np.ndarray:
    """Column-major flat storage of an n-d array (NDTensors Dense layout)."""
    return np.asarray(A).ravel(order="F")


def unflat(x: np.ndarray, dims) -> np.ndarray:
    return np.asarray(x).reshape(tuple(dims), order="F")


# ---------------------------------------------------------------- truncation
def truncate_legacy_gpu(P, maxdim=None, mindim=1, cutoff=0.0, absoluteCutoff=False, doRelCutoff=True):
    """src/tensor/cutruncate.jl:1-93 step by step.  Returns (n_keep, truncerr, docut).

    Sums run sequentially.  cut_ind is the first index strictly below the
    threshold (cuBLAS iamax of the +-2/0 flags, cutruncate.jl:35-38,53-56), 0
    when none is; a value exactly at the threshold counts as not below.
    """
    P = np.asarray(P, dtype=np.float64)
    origm = len(P)
    maxdim = origm if (maxdim is None or maxdim <= 0) else min(int(maxdim), origm)
    mindim = min(max(int(mindim), 1), maxdim)
    maxP = P.max()
    if maxP == 0.0:
        return 1, 0.0, 0.0
    if origm == 1:
        return 1, 0.0, maxP / 2
    rP = np.where(np.signbit(P), 0.0, P)
    n = origm
    truncerr = 0.0
    if n > maxdim:
        for i in range(n - maxdim):
            truncerr += rP[i]
        n = maxdim
    cut_ind = 0
    if absoluteCutoff:
        for i in range(origm):
            if rP[i] - cutoff < 0.0:
                cut_ind = i
                break
        n = min(maxdim, origm - cut_ind)
        n = max(n, mindim)
        for i in range(cut_ind, origm):
            truncerr += rP[i]
    else:
        scale = 1.0
        if doRelCutoff:
            scale = 0.0
            for x in P:
                scale += x
            scale = scale if scale > 0.0 else 1.0
        for i in range(origm):
            if (rP[i] + truncerr) - cutoff * scale < 0.0:
                cut_ind = i
                break
        if cut_ind > 0:
            for i in range(cut_ind, origm):
                truncerr += rP[i]
        else:
            for i in range(maxdim):
                truncerr += rP[i]
        n = min(maxdim, origm - cut_ind)
        n = max(n, mindim)
        truncerr = 0.0 if scale == 0.0 else truncerr / scale
    if n < 1:
        n = 1
    docut = 0.0
    if n < origm:
        docut = (P[n - 1] + P[n]) / 2
        if abs(P[n - 1] - P[n]) < 1e-3 * P[n - 1]:
            docut += 1e-3 * P[n - 1]
    return n, truncerr, docut


def truncate_cpu(P, maxdim=None, mindim=1, cutoff=0.0, absoluteCutoff=False, doRelCutoff=True):
    """ITensors 0.2 (NDTensors) CPU truncate!: cumulative discarded weight.

    Returns (n_keep, truncerr, docut).  Sequential sums, in the order the
    documented loop uses.
    """
    P = np.asarray(P, dtype=np.float64)
    origm = len(P)
    if origm == 0:
        return 0, 0.0, 0.0
    maxdim = origm if (maxdim is None or maxdim <= 0) else min(int(maxdim), origm)
    mindim = max(int(mindim), 1)
    if origm == 1:
        return 1, 0.0, abs(P[0]) / 2
    s = -1.0 if P[0] < 0.0 else 1.0
    Q = s * P
    lastpos = origm
    for i in range(origm - 1, -1, -1):
        if Q[i] >= 0.0:
            break
        lastpos = i
    Q = Q.copy()
    Q[lastpos:] = 0.0
    n = origm
    truncerr = 0.0
    while n > maxdim:
        truncerr += Q[n - 1]
        n -= 1
    if absoluteCutoff:
        while Q[n - 1] <= cutoff and n > mindim:
            truncerr += Q[n - 1]
            n -= 1
    else:
        scale = 1.0
        if doRelCutoff:
            scale = 0.0
            for x in Q:
                scale += x
            if scale == 0.0:
                scale = 1.0
        while (truncerr + Q[n - 1] <= cutoff * scale) and n > mindim:
            truncerr += Q[n - 1]
            n -= 1
        truncerr /= scale
    if n < 1:
        n = 1
    docut = 0.0
    if n < origm:
        docut = (Q[n - 1] + Q[n]) / 2
        if abs(Q[n - 1] - Q[n]) < 1e-3 * Q[n - 1]:
            docut += 1e-3 * Q[n - 1]
    return n, truncerr, docut


# -------------------------------------------------------------- factorisation
def svd_trunc(M: np.ndarray, maxdim=None, mindim=1, cutoff=0.0, absoluteCutoff=False, doRelCutoff=True,
              legacy_gpu=False):
    """(U, S, V, truncerr, docut) with M ~ U diag(S) V^T (culinearalgebra.jl:33-72)."""
    U, S, Vt = np.linalg.svd(M, full_matrices=False)
    P = S ** 2
    f = truncate_legacy_gpu if legacy_gpu else truncate_cpu
    k, te, dc = f(P, maxdim=maxdim, mindim=mindim, cutoff=cutoff, absoluteCutoff=absoluteCutoff,
                  doRelCutoff=doRelCutoff)
    return U[:, :k], S[:k], Vt[:k].T, te, dc


def eigh_trunc(M: np.ndarray, **kw):
    """Descending eigenpairs of a symmetric matrix + truncation (culinearalgebra.jl:74-108)."""
    w, V = np.linalg.eigh(0.5 * (M + M.T))
    w, V = w[::-1], V[:, ::-1]
    legacy = kw.pop("legacy_gpu", False)
    f = truncate_legacy_gpu if legacy else truncate_cpu
    k, te, dc = f(w, **kw)
    return w[:k], V[:, :k], te, dc


def qr_pos(M: np.ndarray):
    """Thin QR with a non-negative diagonal of R."""
    Q, R = np.linalg.qr(M)
    s = np.sign(np.diag(R))
    s[s == 0] = 1.0
    return Q * s, R * s[:, None]


# --------------------------------------------------------------- DMRG pieces
def heff_apply(L, W1, W2, R, psi):
    """out[a',s1',s2',b'] = sum L[a,w,a'] W1[w,s1',s1,x] W2[x,s2',s2,y] R[b,y,b'] psi[a,s1,s2,b]."""
    t = np.tensordot(L, psi, axes=([0], [0]))                 # (w, a', s1, s2, b)
    t = np.tensordot(t, W1, axes=([0, 2], [0, 2]))            # (a', s2, b, s1', x)
    t = np.tensordot(t, W2, axes=([4, 1], [0, 2]))            # (a', b, s1', s2', y)
    t = np.tensordot(t, R, axes=([1, 4], [0, 1]))             # (a', s1', s2', b')
    return t


def heff_diag(L, W1, W2, R):
    Ld = np.einsum("awa->aw", L)
    Rd = np.einsum("byb->by", R)
    Wd = np.einsum("wssx,xtty->wsty", W1, W2)
    return np.einsum("aw,wsty,by->astb", Ld, Wd, Rd)


def davidson(matvec, x0: np.ndarray, dg: np.ndarray, krylovdim=3, maxiter=2, tol=1e-14):
    """The library's Davidson (itg_davidson_heff2), restated.  Returns (theta, x, nmatvec)."""
    kmax = min(max(krylovdim, 2), 32)
    maxiter = max(maxiter, 1)
    n = x0.size
    V = np.zeros((n, kmax))
    AV = np.zeros((n, kmax))
    V[:, 0] = x0.ravel(order="F") / np.linalg.norm(x0)
    AV[:, 0] = matvec(V[:, 0])
    nmv = 1
    k = 1
    theta, X, HX, rn = 0.0, None, None, 0.0
    for restart in range(maxiter):
        while True:
            G = V[:, :k].T @ AV[:, :k]
            G = 0.5 * (G + G.T)
            w, Y = np.linalg.eigh(G)
            theta = w[0]
            y = Y[:, 0]
            if y[np.argmax(np.abs(y))] < 0:
                y = -y
            X = V[:, :k] @ y
            HX = AV[:, :k] @ y
            r = HX - theta * X
            rn = np.linalg.norm(r)
            if rn < tol or k == kmax:
                break
            guard = 1e-8 * max(abs(theta), 1.0)
            den = dg - theta
            den = np.where(np.abs(den) < guard, np.where(den >= 0, guard, -guard), den)
            tn = 0.0
            for t in (r / den, r.copy()):
                t0 = np.linalg.norm(t)
                for _ in range(2):
                    t = t - V[:, :k] @ (V[:, :k].T @ t)
                tn = np.linalg.norm(t)
                if tn > 1e-6 * t0:
                    break
                tn = 0.0
            if not tn > 1e-14:
                break
            V[:, k] = t / tn
            AV[:, k] = matvec(V[:, k])
            nmv += 1
            k += 1
        if rn < tol or restart == maxiter - 1:
            break
        xn = np.linalg.norm(X)
        V[:, 0] = X / xn
        AV[:, 0] = HX / xn
        k = 1
    return theta, X / np.linalg.norm(X), nmv


# ------------------------------------------------------------------ MPOs
def spin_matrices(d):
    S = (d - 1) / 2.0
    m = S - np.arange(d)
    Sz = np.diag(m)
    Sp = np.zeros((d, d))
    for k in range(1, d):
        Sp[k - 1, k] = math.sqrt(S * (S + 1) - m[k] * (m[k] + 1))
    return np.eye(d), Sz, Sp, Sp.T.copy()


def mpo_terms(N, d, bonds):
    """MPO (list of (wl, s', s, wr) arrays) for H = sum_i c1 Sz_i + sum over two-site
    terms given as (i, j, coefficient, opname_i, opname_j), built by the generic
    'one channel per open term' construction (independent of the product's
    hand-coded MPOs)."""
    I, Sz, Sp, Sm = spin_matrices(d)
    ops = {"Sz": Sz, "S+": Sp, "S-": Sm, "Sx": 0.5 * (Sp + Sm), "Id": I}
    # channels: 0 = done, 1..K open terms, K+1 = start
    # open term t spans sites i < j; channel t carries identity on sites strictly between.
    terms = [b for b in bonds if len(b) == 5]
    singles = [b for b in bonds if len(b) == 3]
    K = len(terms)
    D = K + 2
    Ws = []
    for site in range(N):
        W = np.zeros((D, D, d, d))
        W[0, 0] = I
        W[D - 1, D - 1] = I
        for t, (i, j, c, oi, oj) in enumerate(terms, start=1):
            if site == i:
                W[D - 1, t] = c * ops[oi]
            elif i < site < j:
                W[t, t] = I
            elif site == j:
                W[t, 0] = ops[oj]
        for (i, c, o) in singles:
            if site == i:
                W[D - 1, 0] += c * ops[o]
        Ws.append(W)
    out = []
    for site in range(N):
        W = Ws[site]
        if site == 0:
            W = W[D - 1: D]
        if site == N - 1:
            W = W[:, 0:1]
        out.append(np.ascontiguousarray(np.transpose(W, (0, 2, 3, 1))))
    return out


def heisenberg_terms(N, J=1.0, Delta=1.0, nn2=0.0):
    Js = np.broadcast_to(np.asarray(J, float), (max(N - 1, 1),))
    Ds = np.broadcast_to(np.asarray(Delta, float), (max(N - 1, 1),))
    terms = []
    for i in range(N - 1):
        terms += [(i, i + 1, 0.5 * Js[i], "S+", "S-"), (i, i + 1, 0.5 * Js[i], "S-", "S+"),
                  (i, i + 1, Js[i] * Ds[i], "Sz", "Sz")]
    if nn2:
        for i in range(N - 2):
            terms += [(i, i + 2, 0.5 * nn2, "S+", "S-"), (i, i + 2, 0.5 * nn2, "S-", "S+"),
                      (i, i + 2, nn2, "Sz", "Sz")]
    return terms


def heisenberg_mpo(N, d=2, J=1.0, Delta=1.0, J2=0.0):
    return compress_mpo(mpo_terms(N, d, heisenberg_terms(N, J, Delta, J2)))


def tfim_mpo(N, h=0.5, J=1.0):
    terms = [(i, i + 1, -J, "Sz", "Sz") for i in range(N - 1)] + [(i, -h, "Sx") for i in range(N)]
    return compress_mpo(mpo_terms(N, 2, terms))


def compress_mpo(Ws):
    """Drop MPO channels that carry nothing on a bond (keeps the generic
    construction exact but removes empty rows/columns)."""
    Ws = [w.copy() for w in Ws]
    for b in range(len(Ws) - 1):
        left, right = Ws[b], Ws[b + 1]
        keep = [k for k in range(left.shape[3])
                if np.any(left[:, :, :, k] != 0) and np.any(right[k] != 0)]
        Ws[b] = left[:, :, :, keep]
        Ws[b + 1] = right[keep]
    return Ws


def mpo_matrix(Ws):
    M = Ws[0][0]                                    # (s', s, wr)
    for W in Ws[1:]:
        M = np.einsum("abw,wcdx->acbdx", M, W)
        a, c, b, dd, x = M.shape
        M = M.reshape(a * c, b * dd, x)
    return M[:, :, 0]


def mps_vector(As):
    """Full state vector of a small MPS given as (l, s, r) arrays; site 0 is the
    slowest index, as in mpo_matrix."""
    v = As[0][0]                                    # (s, r)
    for A in As[1:]:
        v = np.einsum("ar,rsb->asb", v, A)
        v = v.reshape(-1, A.shape[2])
    return v[:, 0]


# ------------------------------------------------------------ random MPS
def random_mps(dims_site, linkdim, seed):
    N = len(dims_site)
    ld = []
    for j in range(N - 1):
        left = float(np.prod(dims_site[: j + 1], dtype=np.float64))
        right = float(np.prod(dims_site[j + 1:], dtype=np.float64))
        ld.append(int(min(linkdim, left, right)))
    chis = [1] + ld + [1]
    out = []
    for j in range(N):
        shape = (chis[j], dims_site[j], chis[j + 1])
        x = philox_normal(int(np.prod(shape)), seed, j)
        out.append(unflat(x / np.linalg.norm(x), shape))   # randn! + normalize!, cumps.jl:44-53
    return out


# ------------------------------------------------------------------ DMRG
def _env_left(L, A, W):
    """L'[b, x, d] = sum L[a, w, c] A[a, s, b] W[w, t, s, x] A[c, t, d] (pairwise BLAS products)."""
    t = np.tensordot(L, A, axes=([0], [0]))                  # (w, c, s, b)
    t = np.tensordot(t, W, axes=([0, 2], [0, 2]))            # (c, b, t, x)
    return np.tensordot(t, A, axes=([0, 2], [0, 1]))         # (b, x, d)


def _env_right(R, A, W):
    """R'[a, w, c] = sum A[a, s, b] W[w, t, s, x] R[b, x, d] A[c, t, d] (pairwise BLAS products)."""
    t = np.tensordot(A, R, axes=([2], [0]))                  # (a, s, x, d)
    t = np.tensordot(t, W, axes=([1, 2], [2, 3]))            # (a, d, w, t)
    return np.tensordot(t, A, axes=([1, 3], [2, 1]))         # (a, w, c)


def _noise_split(M, phi, L, W1, W2, R, ha, noise, maxdim, mindim, cutoff, legacy):
    """Bond split through the perturbed reduced density matrix (ITensors 0.2's
    dmrg with noise > 0: noiseterm, then factorize with which_decomp="eigen").

    Left-moving half: rho = M M^T + noise * nt nt^T over (a d1), with
    nt[a', t, x, d2, c] = sum L[a, w, a'] W1[w, t, s, x] phi[a, s, d2, c].
    Right-moving half: rho = M^T M + noise * nt nt^T over (d2 c), with
    nt[t, c', a, d1, w] = sum phi[a, d1, s, c] W2[w, t, s, x] R[c, x, c'].
    Returns (left factor, right factor, truncerr).
    """
    a, d1, d2, c = phi.shape
    if ha == 1:
        nt = np.einsum("awc,wtsx,asdb->ctxdb", L, W1, phi, optimize=True)
        ntm = nt.reshape(a * d1, -1, order="F")
        rho = M @ M.T + noise * (ntm @ ntm.T)
        D, U, te, _ = eigh_trunc(rho, maxdim=maxdim, mindim=mindim, cutoff=cutoff, legacy_gpu=legacy)
        return U, U.T @ M, te
    nt = np.einsum("akdb,wtdx,bxe->tekaw", phi, W2, R, optimize=True)
    ntm = nt.reshape(d2 * c, -1, order="F")
    rho = M.T @ M + noise * (ntm @ ntm.T)
    D, V, te, _ = eigh_trunc(rho, maxdim=maxdim, mindim=mindim, cutoff=cutoff, legacy_gpu=legacy)
    return M @ V, V.T, te


def dmrg(Ws, As, maxdims, cutoffs, nsweep, mindim=1, krylovdim=3, maxiter=2, tol=1e-14,
         legacy_gpu_truncate=False, return_sweeps=False, noises=None):
    """Two-site DMRG, the same schedule and solver as itg.dmrg.dmrg; a sweep
    with noise > 0 splits bonds through the perturbed density matrix."""
    N = len(As)
    A = [a.copy() for a in As]
    # right-orthogonalise by QR from the right, normalise site 0
    for j in range(N - 1, 0, -1):
        a, d, b = A[j].shape
        M = A[j].reshape(a, d * b, order="F")
        Q, R = qr_pos(M.T)
        r = Q.shape[1]
        A[j] = Q.T.reshape(r, d, b, order="F")
        A[j - 1] = np.tensordot(A[j - 1], R, axes=([2], [1]))
    A[0] = A[0] / np.linalg.norm(A[0])
    Lenv = [None] * (N + 1)
    Renv = [None] * (N + 1)
    Lenv[0] = np.ones((1, 1, 1))
    Renv[N] = np.ones((1, 1, 1))
    for j in range(N - 1, 1, -1):
        Renv[j] = _env_right(Renv[j + 1], A[j], Ws[j])
    energy = 0.0
    hist = []
    at = lambda v, i: v[min(i, len(v) - 1)]
    for sw in range(nsweep):
        maxdim, cutoff = at(maxdims, sw), at(cutoffs, sw)
        maxerr = 0.0
        for b, ha in [(b, 1) for b in range(N - 1)] + [(b, 2) for b in range(N - 2, -1, -1)]:
            phi = np.tensordot(A[b], A[b + 1], axes=([2], [0]))      # (a, d1, d2, c)
            L, R = Lenv[b], Renv[b + 2]
            W1, W2 = Ws[b], Ws[b + 1]
            shape = phi.shape
            mv = lambda v: flat(heff_apply(L, W1, W2, R, unflat(v, shape)))
            dg = flat(heff_diag(L, W1, W2, R))
            energy, x, _ = davidson(mv, flat(phi), dg, krylovdim, maxiter, tol)
            a, d1, d2, c = shape
            M = unflat(x, (a * d1, d2 * c))
            nz = at(noises, sw) if noises else 0.0
            if nz > 0:
                Lf, Rf, te = _noise_split(M, unflat(x, shape), L, W1, W2, R, ha, nz, maxdim, mindim, cutoff,
                                          legacy_gpu_truncate)
                maxerr = max(maxerr, te)
                k = Lf.shape[1]
                A[b] = Lf.reshape(a, d1, k, order="F")
                A[b + 1] = Rf.reshape(k, d2, c, order="F")
                if ha == 1:
                    Lenv[b + 1] = _env_left(L, A[b], W1)
                else:
                    Renv[b + 1] = _env_right(R, A[b + 1], W2)
                continue
            U, S, V, te, _ = svd_trunc(M, maxdim=maxdim, mindim=mindim, cutoff=cutoff,
                                       legacy_gpu=legacy_gpu_truncate)
            maxerr = max(maxerr, te)
            k = len(S)
            if ha == 1:
                A[b] = U.reshape(a, d1, k, order="F")
                A[b + 1] = (S[:, None] * V.T).reshape(k, d2, c, order="F")
                Lenv[b + 1] = _env_left(L, A[b], W1)
            else:
                A[b] = (U * S[None, :]).reshape(a, d1, k, order="F")
                A[b + 1] = V.T.reshape(k, d2, c, order="F")
                Renv[b + 1] = _env_right(R, A[b + 1], W2)
        hist.append((energy, max(x.shape[2] for x in A[:-1]), maxerr))
    if return_sweeps:
        return energy, A, hist
    return energy, A


# -------------------------------------------------- exact diagonalisation
def heisenberg_ed_sz0(N: int, J=1.0, Delta=1.0, J2=0.0) -> float:
    """Ground energy of the open S=1/2 XXZ (+ J2) chain in the Sz=0 sector (scipy eigsh)."""
    import scipy.sparse as sp
    from scipy.sparse.linalg import eigsh
    from itertools import combinations

    states = np.array([sum(1 << i for i in c) for c in combinations(range(N), N // 2)], dtype=np.int64)
    index = {int(s): k for k, s in enumerate(states)}
    rows, cols, vals = [], [], []
    diag = np.zeros(len(states))
    bonds = [(i, i + 1, J) for i in range(N - 1)] + ([(i, i + 2, J2) for i in range(N - 2)] if J2 else [])
    for k, s in enumerate(states):
        s = int(s)
        for (i, j, c) in bonds:
            bi, bj = (s >> i) & 1, (s >> j) & 1
            diag[k] += c * Delta * (0.25 if bi == bj else -0.25)
            if bi != bj:
                t = s ^ ((1 << i) | (1 << j))
                rows.append(index[t])
                cols.append(k)
                vals.append(0.5 * c)
    H = sp.csr_matrix((vals, (rows, cols)), shape=(len(states), len(states))) + sp.diags(diag)
    w = eigsh(H, k=1, which="SA", tol=1e-14, return_eigenvectors=False)
    return float(w[0])


def tfim_closed_form(N: int) -> float:
    """test/dmrg.jl:79: E = 0.25 - 0.25 / sin(pi / (2 (2N + 1))) for H = -sum SzSz - 0.5 sum Sx."""
    return 0.25 - 0.25 / math.sin(math.pi / (2 * (2 * N + 1)))


# ------------------------------------------------- learned preconditioner MLP
MLP_W = 128


def bf16_round(x) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest even), returned as float32."""
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def mlp_unpack(params, F):
    p = np.asarray(params, dtype=np.float32)
    o = 0
    W1 = p[o: o + MLP_W * F].reshape(MLP_W, F); o += MLP_W * F
    b1 = p[o: o + MLP_W]; o += MLP_W
    W2 = p[o: o + MLP_W * MLP_W].reshape(MLP_W, MLP_W); o += MLP_W * MLP_W
    b2 = p[o: o + MLP_W]; o += MLP_W
    w3 = p[o: o + MLP_W]; o += MLP_W
    b3 = p[o]
    return W1, b1, W2, b2, w3, b3


def mlp_forward(params, F, X):
    """The library's per-element MLP: BF16 weights, FP32 arithmetic, ReLU."""
    W1, b1, W2, b2, w3, b3 = mlp_unpack(params, F)
    W1, W2, w3 = bf16_round(W1), bf16_round(W2), bf16_round(w3)
    X = np.asarray(X, dtype=np.float32).reshape(-1, F)
    z1 = X @ W1.T + b1
    a1 = np.maximum(z1, 0)
    z2 = a1 @ W2.T + b2
    a2 = np.maximum(z2, 0)
    return (a2 @ w3 + b3).astype(np.float32)


def mlp_loss_grad(params, F, X, mult, target):
    """(loss, gradient w.r.t. the master parameters) of mean (g*mult - target)^2."""
    W1, b1, W2, b2, w3, b3 = mlp_unpack(params, F)
    W1r, W2r, w3r = bf16_round(W1), bf16_round(W2), bf16_round(w3)
    X = np.asarray(X, dtype=np.float64).reshape(-1, F)
    n = X.shape[0]
    z1 = X @ W1r.T.astype(np.float64) + b1
    a1 = np.maximum(z1, 0)
    z2 = a1 @ W2r.T.astype(np.float64) + b2
    a2 = np.maximum(z2, 0)
    g = a2 @ w3r.astype(np.float64) + b3
    diff = g * mult - target
    loss = float(np.mean(diff ** 2))
    dg = 2.0 * diff * mult / n
    dw3 = a2.T @ dg
    db3 = dg.sum()
    dz2 = np.outer(dg, w3r) * (z2 > 0)
    dW2 = dz2.T @ a1
    db2 = dz2.sum(0)
    dz1 = (dz2 @ W2r.astype(np.float64)) * (z1 > 0)
    dW1 = dz1.T @ X
    db1 = dz1.sum(0)
    grad = np.concatenate([dW1.ravel(), db1, dW2.ravel(), db2, dw3, [db3]])
    return loss, grad
