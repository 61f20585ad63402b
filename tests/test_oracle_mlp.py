"""The oracle's MLP restatement on the CPU: BF16 rounding and the analytic gradient."""
import numpy as np

from oracle import itg_oracle as O


def test_bf16_round_nearest_even():
    x = np.array([1.0, 1.00390625, 1.001953125, 1.0058593750, -2.7182818, 0.0, 65504.0], dtype=np.float32)
    got = O.bf16_round(x)
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7 and rounds to the even mantissa (1.0);
    # 1 + 3*2^-9 is above the tie and rounds up to 1 + 2^-7
    assert got[0] == 1.0 and got[1] == 1.0 and got[2] == 1.0
    assert got[3] == np.float32(1.0078125)
    assert got[4] == np.float32(-2.71875)
    assert got[5] == 0.0
    # values with at most 8 significant bits are unchanged
    y = np.array([3.0, 0.5, -96.0, 2 ** -20], dtype=np.float32)
    assert np.array_equal(O.bf16_round(y), y)


def test_mlp_gradient_finite_differences():
    """The gradient is the exact derivative of the loss with the BF16-rounded
    weights held fixed (a straight-through gradient for the master weights):
    check it against central differences of the loss in FP64 with the
    rounded weights perturbed directly."""
    F = 5
    rng = np.random.default_rng(3)
    n = 40
    W = O.MLP_W
    npar = W * F + W + W * W + W + W + 1
    p = (rng.standard_normal(npar) * 0.2).astype(np.float32)
    p = O.bf16_round(p)  # rounded weights: rounding is then the identity
    X = rng.standard_normal((n, F))
    mult = rng.standard_normal(n)
    target = rng.standard_normal(n)
    loss, grad = O.mlp_loss_grad(p, F, X, mult, target)

    def loss64(q):
        # unpack in FP64 (mlp_unpack casts to FP32, which would round the perturbation)
        o = 0
        W1 = q[o: o + W * F].reshape(W, F); o += W * F
        b1 = q[o: o + W]; o += W
        W2 = q[o: o + W * W].reshape(W, W); o += W * W
        b2 = q[o: o + W]; o += W
        w3 = q[o: o + W]; o += W
        b3 = q[o]
        z1 = X @ W1.T + b1
        z2 = np.maximum(z1, 0) @ W2.T + b2
        g = np.maximum(z2, 0) @ w3 + b3
        return np.mean((g * mult - target) ** 2)

    assert abs(loss64(p.astype(np.float64)) - loss) < 1e-6 * max(1.0, loss)
    idx = np.concatenate([rng.choice(W * F, 6, replace=False),
                          W * F + rng.choice(W, 3, replace=False),
                          W * F + W + rng.choice(W * W, 8, replace=False),
                          [npar - 2, npar - 1]])
    base = p.astype(np.float64)
    for i in idx:
        e = np.zeros(npar)
        e[i] = 1e-5
        fd = (loss64(base + e) - loss64(base - e)) / 2e-5
        assert abs(fd - grad[i]) < 1e-5 * max(1.0, abs(grad[i])), (i, fd, grad[i])


def test_mlp_forward_matches_manual():
    F = 3
    rng = np.random.default_rng(1)
    W = O.MLP_W
    npar = W * F + W + W * W + W + W + 1
    p = rng.standard_normal(npar).astype(np.float32) * 0.1
    X = rng.standard_normal((7, F)).astype(np.float32)
    W1, b1, W2, b2, w3, b3 = O.mlp_unpack(p, F)
    ref = []
    for x in X:
        a1 = np.maximum(O.bf16_round(W1).astype(np.float64) @ x + b1, 0)
        a2 = np.maximum(O.bf16_round(W2).astype(np.float64) @ a1 + b2, 0)
        ref.append(O.bf16_round(w3).astype(np.float64) @ a2 + b3)
    assert np.allclose(O.mlp_forward(p, F, X), ref, rtol=1e-5, atol=1e-6)
