"""MPS / MPO operations on the device, following the reference's cuMPS and
cuMPO tests (test/test_cumps.jl, test/test_cumpo.jl) with sites 0-based.

Each identity the reference checks between two routes (chain contraction vs
inner, contract vs inner(phi, A, psi), add vs inner) is checked here, and the
results are also compared with dense state vectors and operator matrices
built on the host by the oracle (mps_vector, mpo_matrix) for N <= 10.
"""
import numpy as np
import pytest

from oracle import itg_oracle as O

pytestmark = pytest.mark.gpu


def vec(gpu, psi):
    return O.mps_vector([t.array() for t in gpu.cpu(psi).tensors])


def mat(gpu, K):
    return O.mpo_matrix([t.array() for t in gpu.cpu(K).tensors])


def rel(a, b):
    return np.linalg.norm(np.ravel(a - b)) / max(np.linalg.norm(np.ravel(b)), 1e-300)


def _random_chain(gpu, sites, link_dim, seed, mpo=False):
    """Random MPS or MPO with every inner link of dimension link_dim."""
    I = gpu.Index
    N = len(sites)
    links = [I(1, "Link,l=0")] + [I(link_dim, f"r{j},Link") for j in range(1, N)] + [I(1, f"Link,l={N}")]
    ts = []
    for j, s in enumerate(sites):
        inds = (links[j], s.prime(), s, links[j + 1]) if mpo else (links[j], s, links[j + 1])
        ts.append(gpu.randomCuITensor(*inds, seed=seed + j))
    return gpu.MPO(ts, sites) if mpo else gpu.MPS(ts, sites, -1, N)


# ------------------------------------------------------------------- MPS
def test_cumps_basics(gpu):
    N = 10
    sites = [gpu.Index(2, "Site") for _ in range(N)]
    psi = gpu.cuMPS(sites)
    assert len(psi) == N and len(gpu.cuMPS()) == 0
    lines = str(psi).split("\n")
    assert lines[0] == "MPS" and len(lines) == len(psi) + 2
    assert gpu.siteind(psi, 1) == sites[1]
    assert gpu.linkind(psi, 1) in psi[2].inds and gpu.linkind(psi, 2) in psi[2].inds
    L = gpu.cpu(gpu.randomCuMPS(sites, 3, seed=4))
    K = gpu.cuMPS(L)
    assert all(np.array_equal(a.store.data, gpu.cpu(b).store.data) for a, b in zip(L.tensors, K.tensors))


@pytest.mark.parametrize("as_int", [False, True])
def test_product_state_sz(gpu, as_int):
    N = 10
    sites = gpu.siteinds("S=1/2", N)
    states = [(1 if j % 2 == 0 else 2) if as_int else ("Up" if j % 2 == 0 else "Dn") for j in range(N)]
    psi = gpu.productCuMPS(sites, states)
    Sz = gpu.spin_ops(2)["Sz"]
    for j in range(N):
        s = sites[j]
        op = gpu.cuITensor(Sz, s.prime(), s)
        bra = psi[j].replaceinds([s], [s.prime()])
        res = (psi[j] * op) * bra
        assert res.array().sum() == pytest.approx(0.5 if j % 2 == 0 else -0.5)
    with pytest.raises(gpu.DimensionMismatch):
        gpu.cuMPS(sites, ["Up"] * (N - 1))
    with pytest.raises(gpu.DimensionMismatch):
        gpu.productCuMPS(sites, ["Up"] * (N - 1))


def test_random_mps_sites_normalised(gpu):
    sites = [gpu.Index(2, "Site") for _ in range(10)]
    phi = gpu.randomCuMPS(sites, seed=9)
    assert sites[0] in phi[0].inds
    assert gpu.norm(phi[0]) == pytest.approx(1.0, abs=1e-14)
    assert gpu.norm(phi[3]) == pytest.approx(1.0, abs=1e-14)


def test_inner_different_mps(gpu):
    N = 10
    sites = [gpu.Index(2, "Site") for _ in range(N)]
    phi = gpu.randomCuMPS(sites, 4, seed=11)
    psi = gpu.randomCuMPS(sites, 4, seed=12)
    # the same number through a chain of ITensor contractions (links renamed
    # on the bra so that only site indices are shared between the layers)
    bra = [t.replaceinds([t.inds[0], t.inds[2]], [t.inds[0].prime(), t.inds[2].prime()]) for t in phi.tensors]
    E = bra[0] * psi[0]
    for j in range(1, N):
        E = E * bra[j] * psi[j]
    ref = float(np.dot(vec(gpu, phi), vec(gpu, psi)))
    assert E.array().sum() == pytest.approx(ref, rel=1e-12)
    assert gpu.inner(phi, psi) == pytest.approx(ref, rel=1e-12)
    bad = gpu.randomCuMPS([gpu.Index(2) for _ in range(N + 1)], seed=1)
    with pytest.raises(gpu.DimensionMismatch):
        gpu.inner(phi, bad)


def test_add_mps(gpu):
    N = 10
    sites = [gpu.Index(2, "Site") for _ in range(N)]
    for linkdim in (1, 4):
        psi = gpu.randomCuMPS(sites, linkdim, seed=20 + linkdim)
        phi = psi.copy()
        xi = gpu.add(psi, phi)
        assert gpu.inner(xi, xi) == pytest.approx(4.0 * gpu.inner(psi, psi), rel=1e-12)
        assert rel(vec(gpu, xi), 2 * vec(gpu, psi)) < 1e-12
    a = gpu.randomCuMPS(sites, 3, seed=30)
    b = gpu.randomCuMPS(sites, 5, seed=31)
    c = a + b
    assert rel(vec(gpu, c), vec(gpu, a) + vec(gpu, b)) < 1e-12
    # rank-deficient sums compress back under a cutoff
    d = gpu.add(a, a.copy(), cutoff=1e-13)
    assert d.maxlinkdim() <= a.maxlinkdim()
    assert rel(vec(gpu, d), 2 * vec(gpu, a)) < 1e-10


def test_orthogonalize_limits(gpu):
    N = 10
    sites = gpu.siteinds("S=1/2", N)
    psi = gpu.randomCuMPS(sites, 4, seed=40)
    v0 = vec(gpu, psi)
    gpu.orthogonalize_(psi, N - 2)
    assert (gpu.leftlim(psi), gpu.rightlim(psi)) == (N - 3, N - 1)
    gpu.orthogonalize_(psi, 1)
    assert (gpu.leftlim(psi), gpu.rightlim(psi)) == (0, 2)
    assert rel(vec(gpu, psi), v0) < 1e-12
    psi = gpu.randomCuMPS(sites, 4, seed=41)
    psi.rlim = N          # QR from the rightmost tensor
    gpu.orthogonalize_(psi, N // 2 - 1)
    assert (gpu.leftlim(psi), gpu.rightlim(psi)) == (N // 2 - 2, N // 2)


def test_replacebond(gpu):
    N = 10
    sites = gpu.siteinds("S=1/2", N)
    psi = gpu.randomCuMPS(sites, 4, seed=50)
    tags = gpu.linkind(psi, 0).tags
    gpu.replacebond_(psi, 0, psi[0] * psi[1])
    assert gpu.linkind(psi, 0).tags == tags
    gpu.orthogonalize_(psi, 4)
    v0 = vec(gpu, psi)
    gpu.replacebond_(psi, 4, psi[4] * psi[5], ortho="left")
    assert (gpu.leftlim(psi), gpu.rightlim(psi)) == (4, 6)
    gpu.replacebond_(psi, 4, psi[4] * psi[5], ortho="right")
    assert (gpu.leftlim(psi), gpu.rightlim(psi)) == (3, 5)
    psi.llim, psi.rlim = 2, 6
    gpu.replacebond_(psi, 4, psi[4] * psi[5], ortho="left")
    assert (gpu.leftlim(psi), gpu.rightlim(psi)) == (2, 6)
    assert rel(vec(gpu, psi), v0) < 1e-12


def _check_left_orth(gpu, t, tol):
    r = t.inds[-1]
    P = (t * t.replaceinds([r], [r.prime()])).array(r, r.prime())
    assert np.abs(P - np.eye(r.dim)).max() < tol


def _check_right_orth(gpu, t, tol):
    l = t.inds[0]
    P = (t * t.replaceinds([l], [l.prime()])).array(l, l.prime())
    assert np.abs(P - np.eye(l.dim)).max() < tol


def _basic_random(gpu, N, dim, seed):
    sites = [gpu.Index(2, "Site") for _ in range(N)]
    M = _random_chain(gpu, sites, dim, seed)
    M[0] = M[0] / np.sqrt(gpu.inner(M, M))
    return M


def test_orthogonalize_gauge(gpu):
    N, c = 30, 11
    M = _basic_random(gpu, N, 4, 60)
    gpu.orthogonalize_(M, c)
    assert (gpu.leftlim(M), gpu.rightlim(M)) == (c - 1, c + 1)
    for j in range(c):
        _check_left_orth(gpu, M[j], 1e-12)
    for j in range(c + 1, N):
        _check_right_orth(gpu, M[j], 1e-12)
    assert gpu.norm(M[c]) == pytest.approx(1.0, rel=1e-12)


def test_truncate(gpu):
    N = 30
    M = _basic_random(gpu, N, 10, 70)
    M0 = M.copy()
    gpu.truncate_(M, maxdim=5)
    assert gpu.rightlim(M) == 1
    assert M.maxlinkdim() <= 5
    for j in range(1, N):
        _check_right_orth(gpu, M[j], 1e-12)
    assert gpu.inner(M0, M) > 0.1


def test_truncate_exact_when_rank_allows(gpu):
    """maxdim at the true rank leaves the state unchanged."""
    N = 8
    sites = gpu.siteinds("S=1/2", N)
    a = gpu.randomCuMPS(sites, 3, seed=80)
    v = vec(gpu, a)
    s = gpu.add(a, a.copy())                   # bonds doubled, rank unchanged
    gpu.truncate_(s, maxdim=3)
    assert s.maxlinkdim() == 3
    assert rel(vec(gpu, s), 2 * v) < 1e-11


# ------------------------------------------------------------------- MPO
def test_cumpo_basics(gpu):
    N = 6
    sites = [gpu.Index(2, "Site") for _ in range(N)]
    assert len(gpu.cuMPO()) == 0
    O_ = gpu.cuMPO(sites)
    assert len(O_) == N
    lines = str(O_).split("\n")
    assert lines[0] == "MPO" and len(lines) == len(O_) + 2
    O_[0] = gpu.cuITensor(O_[0].inds[0], sites[0], sites[0].prime(), O_[0].inds[-1])
    P = O_.copy()
    assert sites[0] in P[0].inds and sites[0].prime() in P[0].inds
    K = gpu.randomCuMPO(gpu.siteinds("S=1/2", N), seed=3)
    Kc = gpu.cpu(K)
    K2 = gpu.cuMPO(Kc)
    assert all(np.array_equal(a.store.data, gpu.cpu(b).store.data) for a, b in zip(Kc.tensors, K2.tensors))
    assert K.maxlinkdim() == 1


def test_mpo_orthogonalize_keeps_expectation(gpu):
    N = 6
    sites = [gpu.Index(2, "Site") for _ in range(N)]
    phi = gpu.randomCuMPS(sites, 2, seed=90)
    K = _random_chain(gpu, sites, 3, 91, mpo=True)
    gpu.orthogonalize_(phi, 0)
    gpu.orthogonalize_(K, 0)
    e0 = gpu.inner(phi, K, phi)
    gpu.orthogonalize_(phi, N // 2)
    gpu.orthogonalize_(K, N // 2)
    assert gpu.inner(phi, K, phi) == pytest.approx(e0, rel=1e-12)
    v = vec(gpu, phi)
    assert e0 == pytest.approx(v @ mat(gpu, K) @ v, rel=1e-12)


def test_inner_mpo(gpu):
    N = 6
    sites = [gpu.Index(2, "Site") for _ in range(N)]
    phi = gpu.randomCuMPS(sites, seed=100)
    K = gpu.randomCuMPO(sites, seed=101)
    assert gpu.maxlinkdim(K) == 1
    psi = gpu.randomCuMPS(sites, seed=102)
    ref = vec(gpu, phi) @ mat(gpu, K) @ vec(gpu, psi)
    assert gpu.inner(phi, K, psi) == pytest.approx(ref, rel=1e-12)
    bad = gpu.randomCuMPS([gpu.Index(2, "Site") for _ in range(N + 1)], seed=1)
    with pytest.raises(gpu.DimensionMismatch):
        gpu.inner(phi, K, bad)
    for link_dim in range(2, 6):
        K = _random_chain(gpu, sites, link_dim, 200 + link_dim, mpo=True)
        psi = _random_chain(gpu, sites, link_dim, 300 + link_dim)
        phi = _random_chain(gpu, sites, link_dim, 400 + link_dim)
        gpu.orthogonalize_(psi, 0, maxdim=link_dim)
        gpu.orthogonalize_(K, 0, maxdim=link_dim)
        gpu.orthogonalize_(phi, 0, normalize=True, maxdim=link_dim)
        ref = vec(gpu, phi) @ mat(gpu, K) @ vec(gpu, psi)
        assert gpu.inner(phi, K, psi) == pytest.approx(ref, rel=1e-11)


def test_contract_mpo_mps(gpu):
    N = 6
    sites = [gpu.Index(2, "Site") for _ in range(N)]
    phi = gpu.randomCuMPS(sites, seed=110)
    K = gpu.randomCuMPO(sites, seed=111)
    psi = gpu.randomCuMPS(sites, seed=112)
    out = gpu.contract(K, psi, maxdim=1)
    assert gpu.inner(phi, out) == pytest.approx(gpu.inner(phi, K, psi), rel=1e-12)
    with pytest.raises(gpu.ArgumentError):
        gpu.contract(K, psi, method="fakemethod")
    bad = gpu.randomCuMPS([gpu.Index(2, "Site") for _ in range(N + 1)], seed=1)
    with pytest.raises(gpu.DimensionMismatch):
        gpu.contract(K, bad)
    for link_dim in range(2, 6):
        K = _random_chain(gpu, sites, link_dim, 500 + link_dim, mpo=True)
        psi = _random_chain(gpu, sites, link_dim, 600 + link_dim)
        phi = _random_chain(gpu, sites, link_dim, 700 + link_dim)
        gpu.orthogonalize_(psi, 0, maxdim=link_dim)
        gpu.orthogonalize_(K, 0, maxdim=link_dim)
        gpu.orthogonalize_(phi, 0, normalize=True, maxdim=link_dim)
        out = gpu.contract(K.copy(), psi.copy(), maxdim=10 * link_dim, cutoff=0.0)
        assert gpu.inner(phi, out) == pytest.approx(gpu.inner(phi, K, psi), rel=1e-10)
        assert rel(vec(gpu, out), mat(gpu, K) @ vec(gpu, psi)) < 1e-11
        exact = gpu.contract(K, psi)
        assert exact.maxlinkdim() <= link_dim * link_dim
        assert rel(vec(gpu, exact), mat(gpu, K) @ vec(gpu, psi)) < 1e-12


def test_add_mpo(gpu):
    N = 6
    s = gpu.siteinds("S=1/2", N)
    K = gpu.randomCuMPO(s, seed=120)
    L = gpu.randomCuMPO(s, seed=130)
    M = gpu.add(K, L)
    assert len(M) == N
    assert rel(mat(gpu, M), mat(gpu, K) + mat(gpu, L)) < 1e-12
    psi = gpu.randomCuMPS(s, seed=140)
    kp = gpu.contract(K, psi, maxdim=1)
    lp = gpu.contract(L, psi, maxdim=1)
    assert gpu.inner(psi, gpu.add(kp, lp)) == pytest.approx(gpu.inner(psi, M, psi), abs=5e-3)
    H = gpu.cuMPO(gpu.heisenberg_mpo(s))
    H2 = H + H
    assert rel(mat(gpu, H2), 2 * mat(gpu, H)) < 1e-12


def test_contract_mpo_mpo(gpu):
    N = 6
    sites = [gpu.Index(2, "Site") for _ in range(N)]
    psi = gpu.randomCuMPS(sites, seed=150)
    K = gpu.randomCuMPO(sites, seed=151)
    L = gpu.randomCuMPO(sites, seed=152)
    KL = gpu.contract(gpu.prime(K), L, maxdim=1)
    assert rel(mat(gpu, KL), mat(gpu, K) @ mat(gpu, L)) < 1e-12
    kl_psi = gpu.contract(gpu.prime(K), gpu.contract(L, psi, maxdim=1), maxdim=1)
    assert gpu.inner(psi, KL, psi) == pytest.approx(gpu.inner(psi, kl_psi), abs=5e-3)
    # both operators carry (s', s): the product is taken as an operator product
    assert rel(mat(gpu, gpu.contract(K, L)), mat(gpu, K) @ mat(gpu, L)) < 1e-12
    # differently labelled outputs: the shared input index is summed
    ok = [gpu.Index(2, "Site,aaa") for _ in range(N)]
    ol = [gpu.Index(2, "Site,bbb") for _ in range(N)]
    K = gpu.randomCuMPO(sites, seed=160)
    L = gpu.randomCuMPO(sites, seed=161)
    for j in range(N):
        K[j] = K[j].replaceinds([sites[j].prime()], [ok[j]])
        L[j] = L[j].replaceinds([sites[j].prime()], [ol[j]])
    KL = gpu.contract(K, L, maxdim=1)
    psik = gpu.randomCuMPS(ok, seed=170)
    psil = gpu.randomCuMPS(ol, seed=171)
    out = gpu.contract(K, gpu.contract(L, psil, maxdim=1), maxdim=1)
    assert gpu.inner(psik, KL, psil) == pytest.approx(gpu.inner(psik, out), abs=5e-3)
    badL = gpu.randomCuMPO([gpu.Index(2, "Site") for _ in range(N + 1)], seed=1)
    with pytest.raises(gpu.DimensionMismatch):
        gpu.contract(K, badL)


def test_heisenberg_expectation_through_contract(gpu):
    """<psi|H|psi> three ways: inner(psi, H, psi), inner(psi, H psi), dense."""
    N = 8
    s = gpu.siteinds("S=1/2", N)
    H = gpu.cuMPO(gpu.heisenberg_mpo(s))
    psi = gpu.randomCuMPS(s, 6, seed=180)
    e1 = gpu.inner(psi, H, psi)
    e2 = gpu.inner(psi, gpu.contract(H, psi))
    v = vec(gpu, psi)
    e3 = v @ O.mpo_matrix(O.heisenberg_mpo(N)) @ v
    assert e1 == pytest.approx(e3, rel=1e-12)
    assert e2 == pytest.approx(e3, rel=1e-12)
    assert gpu.expect_energy(H, psi) == pytest.approx(e3 / (v @ v), rel=1e-12)


# ------------------------------------------------------- gate application
def test_gate_evolution_example(gpu):
    """examples/gate_evolution.jl: X on every other qubit of |00...0>."""
    N = 10
    s = gpu.siteinds("Qubit", N)
    X = gpu.ops(s, [("X", n) for n in range(N)])
    psi0 = gpu.productCuMPS(s, ["0"] * N)
    psi = gpu.apply([X[n] for n in range(0, N, 2)], psi0)
    v = vec(gpu, psi)
    idx = int("".join("1" if n % 2 == 0 else "0" for n in range(N)), 2)   # site 0 is the slowest bit
    want = np.zeros(2 ** N)
    want[idx] = 1.0
    assert np.abs(v - want).max() < 1e-15
    assert np.abs(vec(gpu, psi0) - np.eye(2 ** N)[0]).max() == 0.0       # input untouched


def _dense_gate(G, n, N, d=2):
    left, right = np.eye(d ** n), np.eye(d ** (N - n - 2))
    return np.kron(np.kron(left, G), right)


def test_apply_two_site_gates_matches_dense(gpu):
    N = 8
    s = gpu.siteinds("Qubit", N)
    rng = np.random.default_rng(17)
    psi = gpu.randomCuMPS(s, 4, seed=190)
    v = vec(gpu, psi)
    gates, dense = [], []
    for n in [0, 3, 6, 2, 5, 1, 4]:
        G = rng.standard_normal((4, 4))
        gates.append(gpu.op("g", s[n], s[n + 1], matrix=G))
        dense.append((G, n))
    out = gpu.apply(gates, psi)
    for G, n in dense:
        v = _dense_gate(G, n, N) @ v
    assert rel(vec(gpu, out), v) < 1e-12
    # built-in gates, and a truncating application
    bell = gpu.apply([gpu.op("H", s[0]), gpu.op("CNOT", s[0], s[1])], gpu.productCuMPS(s, ["0"] * N))
    vb = vec(gpu, bell)
    assert vb[0] == pytest.approx(2 ** -0.5) and vb[3 << (N - 2)] == pytest.approx(2 ** -0.5)
    assert bell.maxlinkdim() == 2
    cut = gpu.apply(gates, psi, maxdim=2)
    assert cut.maxlinkdim() <= 2
    with pytest.raises(gpu.ArgumentError):
        gpu.apply([gpu.op("SWAP", s[0], s[2])], psi)
