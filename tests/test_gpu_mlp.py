"""Learned Davidson preconditioner on the GPU (itg_mlp_*, itg_davidson_heff2_learned).

* forward and gradient of the hand-written BF16/FP32 kernels against the
  oracle's numpy restatement (FP32 accumulation order differs: 1e-4 relative);
* the first Adam step against its closed form;
* training reduces the loss on a synthetic regression;
* the learned eigensolver reaches the same eigenvalue as the plain one, with
  a random network (the stall rule hands over to the diagonal
  preconditioner) and inside a full DMRG run with a trained network;
* a fresh network (zero output layer) is the diagonal preconditioner;
* the measured comparison on a held-out coupling: matvecs per bond of DMRG
  with the trained network against the diagonal preconditioner, at equal
  energy.
"""
import ctypes as C
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import itg_oracle as O

pytestmark = pytest.mark.gpu
GOLD = json.loads((Path(__file__).parent / "golden" / "reference_known_answers.json").read_text())
F = 5


def _p(t):
    return C.c_void_p(t.data_ptr())


def _net(seed=7):
    from itg.learned import LearnedPreconditioner
    return LearnedPreconditioner(seed=seed)


def _rand_params(net, seed, scale=0.15):
    rng = np.random.default_rng(seed)
    p = (rng.standard_normal(net.nparams) * scale).astype(np.float32)
    net.set_params(p)
    return p


@pytest.mark.parametrize("n", [1, 63, 1000, 152 * 64 * 2 + 37])
def test_mlp_forward_matches_oracle(gpu, n):
    import torch
    net = _net()
    p = _rand_params(net, n)
    assert np.array_equal(net.params(), p)
    rng = np.random.default_rng(100 + n)
    X = rng.standard_normal((n, F)).astype(np.float32)
    g = net.forward(torch.from_numpy(X.ravel()).cuda()).cpu().numpy()
    ref = O.mlp_forward(p, F, X)
    assert np.max(np.abs(g - ref)) < 1e-4 * max(1.0, np.max(np.abs(ref)))
    net.close()


@pytest.mark.parametrize("n", [50, 152 * 64 * 3 + 5])
def test_mlp_gradient_matches_oracle(gpu, n):
    import torch
    net = _net()
    p = _rand_params(net, 11 + n)
    rng = np.random.default_rng(n)
    X = rng.standard_normal((n, F)).astype(np.float32)
    mult = rng.standard_normal(n).astype(np.float32)
    target = rng.standard_normal(n).astype(np.float32)
    grad = torch.zeros(net.nparams, dtype=torch.float32, device="cuda")
    loss = net.step(torch.from_numpy(X.ravel()).cuda(), torch.from_numpy(mult).cuda(),
                    torch.from_numpy(target).cuda(), 0.0, grad)
    lo, go = O.mlp_loss_grad(p, F, X, mult, target)
    assert abs(loss - lo) < 1e-4 * lo
    g = grad.cpu().numpy()
    assert np.linalg.norm(g - go) < 1e-4 * np.linalg.norm(go)
    # lr = 0: parameters unchanged
    assert np.array_equal(net.params(), p)
    # deterministic: the same call gives the same bits
    grad2 = torch.zeros_like(grad)
    net.step(torch.from_numpy(X.ravel()).cuda(), torch.from_numpy(mult).cuda(),
             torch.from_numpy(target).cuda(), 0.0, grad2)
    assert torch.equal(grad, grad2)
    net.close()


def test_mlp_first_adam_step(gpu):
    import torch
    net = _net()
    p = _rand_params(net, 5)
    rng = np.random.default_rng(2)
    n = 700
    X = torch.from_numpy(rng.standard_normal(n * F).astype(np.float32)).cuda()
    m = torch.from_numpy(rng.standard_normal(n).astype(np.float32)).cuda()
    y = torch.from_numpy(rng.standard_normal(n).astype(np.float32)).cuda()
    grad = torch.zeros(net.nparams, dtype=torch.float32, device="cuda")
    lr = 1e-3
    net.step(X, m, y, lr, grad)
    g = grad.cpu().numpy().astype(np.float64)
    # first step: m = 0.1 g, v = 0.001 g^2, bias corrections 0.1 and 0.001
    expect = p - lr * g / (np.abs(g) + 1e-8)
    assert np.max(np.abs(net.params() - expect)) < 1e-6
    net.close()


def test_mlp_training_reduces_loss(gpu):
    """Regression target y = m * (0.3 + 0.5 tanh(x1)): learnable by the network."""
    import torch
    net = _net(seed=3)
    rng = np.random.default_rng(9)
    n = 20000
    X = rng.standard_normal((n, F)).astype(np.float32)
    m = rng.standard_normal(n).astype(np.float32)
    y = (m * (0.3 + 0.5 * np.tanh(X[:, 1]))).astype(np.float32)
    data = (torch.from_numpy(X.ravel()).cuda(), torch.from_numpy(m).cuda(), torch.from_numpy(y).cuda())
    l0 = net.step(*data, 0.0)
    net.train(data, steps=300, lr=2e-3, batch=8192)
    l1 = net.step(*data, 0.0)
    assert l1 < 0.05 * l0, (l0, l1)
    net.close()


def _sym_heff(chi, d, w, seed):
    rng = np.random.default_rng(seed)
    L = rng.standard_normal((chi, w, chi))
    R = rng.standard_normal((chi, w, chi))
    W1 = rng.standard_normal((w, d, d, w))
    W2 = rng.standard_normal((w, d, d, w))
    L = L + L.transpose(2, 1, 0)
    R = R + R.transpose(2, 1, 0)
    W1 = W1 + W1.transpose(0, 2, 1, 3)
    W2 = W2 + W2.transpose(0, 2, 1, 3)
    psi = rng.standard_normal((chi, d, d, chi))
    return L, W1, W2, R, psi


def test_learned_davidson_random_network_falls_back_and_converges(gpu):
    """A network with large random weights: its corrections stall, the
    diagonal preconditioner takes over (fallbacks counted) and the converged
    eigenvalue is exact."""
    import torch
    from itg import _lib
    chi, d, w = 12, 2, 5
    L, W1, W2, R, psi = _sym_heff(chi, d, w, seed=3)
    n = chi * d * d * chi
    H = np.stack([O.flat(O.heff_apply(L, W1, W2, R, O.unflat(np.eye(n)[:, i], psi.shape)))
                  for i in range(n)], axis=1)
    e0 = np.linalg.eigvalsh(0.5 * (H + H.T))[0]
    net = _net(seed=1)
    _rand_params(net, 99, scale=1.0)
    dev = lambda a: torch.from_numpy(O.flat(a).copy()).cuda()
    Ld, W1d, W2d, Rd, pd = map(dev, (L, W1, W2, R, psi))
    h = _lib.handle(0)
    e = C.c_double()
    nmv = C.c_int()
    fb = C.c_int()
    h.call("itg_davidson_heff2_learned", C.c_int64(chi), C.c_int64(chi), C.c_int64(d), C.c_int64(w),
           C.c_int64(w), C.c_int64(w), _p(Ld), _p(W1d), _p(W2d), _p(Rd), _p(pd), 10, 200, C.c_double(1e-9), 0,
           net.ptr, None, None, C.byref(e), C.byref(nmv), C.byref(fb))
    x = pd.cpu().numpy()
    assert abs(e.value - e0) < 1e-10 * abs(e0)
    assert np.linalg.norm(H @ x - e.value * x) < 1e-8 * abs(e0)
    assert fb.value >= 1
    net.close()


def test_learned_davidson_rejects_null_network(gpu):
    from itg import _lib
    import torch
    h = _lib.handle(0)
    z = torch.zeros(16, dtype=torch.float64, device="cuda")
    e = C.c_double()
    nmv = C.c_int()
    with pytest.raises(_lib.ITGError):
        h.call("itg_davidson_heff2_learned", C.c_int64(2), C.c_int64(2), C.c_int64(2), C.c_int64(1),
               C.c_int64(1), C.c_int64(1), _p(z), _p(z), _p(z), _p(z), _p(z), 3, 2, C.c_double(1e-10), 0,
               None, None, None, C.byref(e), C.byref(nmv), None)


def test_dmrg_with_trained_preconditioner(gpu):
    """Samples from a plain run of the Heisenberg N=12 chain train the network;
    DMRG with the learned preconditioner on a J1-J2 chain (not seen in
    training) reaches the energy of the plain solver."""
    from itg.learned import SampleCollector
    N = 12
    sites = gpu.siteinds("S=1/2", N)
    H = gpu.cuMPO(gpu.heisenberg_mpo(sites))
    col = SampleCollector(max_elements=2_000_000)
    sw = gpu.Sweeps(4, maxdim=[10, 20, 40], cutoff=[1e-12])
    gpu.dmrg(H, gpu.randomCuMPS(sites, 4, seed=5), sw, bond_hook=col)
    X, M, Y = col.data()
    assert col.count > 1000 and X.numel() == 5 * M.numel() == 5 * Y.numel()
    net = _net(seed=2)
    l0 = net.step(X, M, Y, 0.0)
    net.train((X, M, Y), steps=200, lr=1e-3, batch=16384)
    l1 = net.step(X, M, Y, 0.0)
    assert l1 < l0
    H2 = gpu.cuMPO(gpu.j1j2_mpo(sites, J2=0.5))
    sw2 = gpu.Sweeps(6, maxdim=[10, 20, 50, 100], cutoff=[1e-14])
    plain = gpu.dmrg(H2, gpu.randomCuMPS(sites, 4, seed=8), sw2, return_result=True)
    learned = gpu.dmrg(H2, gpu.randomCuMPS(sites, 4, seed=8), sw2, preconditioner=net, return_result=True)
    assert abs(plain.energy - learned.energy) < 1e-9 * abs(plain.energy)
    net.close()


def test_fresh_network_is_the_diagonal_preconditioner(gpu):
    """With the zero output layer of a new network, g = 0 and the learned
    correction is the diagonally preconditioned residual: the eigensolver takes
    the same number of matvecs as the plain one and reaches the same value."""
    import torch
    from itg import _lib
    chi, d, w = 12, 2, 5
    L, W1, W2, R, psi = _sym_heff(chi, d, w, seed=6)
    net = _net(seed=4)
    X = torch.randn(100 * F, dtype=torch.float32, device="cuda")
    assert torch.count_nonzero(net.forward(X)) == 0
    dev = lambda a: torch.from_numpy(O.flat(a).copy()).cuda()
    h = _lib.handle(0)
    res = []
    for learned in (False, True):
        Ld, W1d, W2d, Rd, pd = map(dev, (L, W1, W2, R, psi))
        e, nmv, fb = C.c_double(), C.c_int(), C.c_int()
        args = (C.c_int64(chi), C.c_int64(chi), C.c_int64(d), C.c_int64(w), C.c_int64(w), C.c_int64(w),
                _p(Ld), _p(W1d), _p(W2d), _p(Rd), _p(pd), 8, 50, C.c_double(1e-10), 0)
        if learned:
            h.call("itg_davidson_heff2_learned", *args, net.ptr, None, None, C.byref(e), C.byref(nmv), C.byref(fb))
        else:
            h.call("itg_davidson_heff2", *args, C.byref(e), C.byref(nmv))
        res.append((e.value, nmv.value))
    (e0, n0), (e1, n1) = res
    assert abs(e0 - e1) < 1e-9 * abs(e0)
    assert abs(n0 - n1) <= max(2, n0 // 5), (n0, n1)
    net.close()


def test_learned_vs_diagonal_matvecs_on_held_out_coupling(gpu, record_property):
    """Train on samples of the plain solver at J2 = 0.2, 0.3, 0.4 (J1-J2 chain,
    N = 24), then run DMRG at the held-out J2 = 0.5 from the same initial state
    with the diagonal and with the learned preconditioner (Davidson krylovdim 3,
    maxiter 4, residual tolerance 1e-9, maxdim 64, cutoff 1e-10).  Both reach
    the same energy (1e-10 relative); the matvecs per bond of both are recorded
    (record_property) as the measured gain of the trained network.  The
    stall rule bounds any loss: a learned step that does not cut the residual
    by 10% is redone with the diagonal preconditioner, so the learned run may
    not need more than 10% more matvecs."""
    from itg.learned import LearnedPreconditioner, SampleCollector
    N = 24
    sites = gpu.siteinds("S=1/2", N)
    col = SampleCollector(max_elements=1_000_000)
    for j2 in (0.2, 0.3, 0.4):
        H = gpu.cuMPO(gpu.j1j2_mpo(sites, J1=1.0, J2=j2))
        gpu.dmrg(H, gpu.randomCuMPS(sites, 8, seed=int(j2 * 100)), gpu.Sweeps(2, maxdim=[32], cutoff=[1e-10]),
                 bond_hook=col)
    X, M, Y = col.data()
    net = LearnedPreconditioner(seed=11)
    l0 = net.step(X, M, Y, 0.0)
    net.train((X, M, Y), steps=800, lr=1e-3, batch=65536)
    l1 = net.step(X, M, Y, 0.0)
    assert l1 < l0
    H = gpu.cuMPO(gpu.j1j2_mpo(sites, J1=1.0, J2=0.5))
    psi0 = gpu.randomCuMPS(sites, 8, seed=505)
    per_bond = {}
    energy = {}
    for name, pc in (("diag", None), ("learned", net)):
        r = gpu.dmrg(H, psi0, gpu.Sweeps(3, maxdim=[64], cutoff=[1e-10]), krylovdim=3, maxiter=4,
                     eigsolve_tol=1e-9, preconditioner=pc, return_result=True)
        per_bond[name] = sum(x.matvecs for x in r.sweeps) / (len(r.sweeps) * 2 * (N - 1))
        energy[name] = r.energy
    record_property("matvecs_per_bond_diag", per_bond["diag"])
    record_property("matvecs_per_bond_learned", per_bond["learned"])
    record_property("loss_before_after", (l0, l1))
    print(f"matvecs per bond: diagonal {per_bond['diag']:.3f}, learned {per_bond['learned']:.3f}")
    assert abs(energy["learned"] - energy["diag"]) < 1e-10 * abs(energy["diag"])
    assert per_bond["learned"] <= 1.10 * per_bond["diag"], per_bond
    net.close()
