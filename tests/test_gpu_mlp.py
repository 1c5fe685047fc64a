"""The learned-state model's tensor-core kernels against FP64 references.

The GEMM (tcgen05 MMA, TMA-loaded BF16 operands, FP32 accumulation in tensor
memory) is compared with the FP64 product of the same BF16-rounded operands:
the only differences are FP32 accumulation errors, bounded by K * 2^-24 of the
sum of |terms|. The model's loss, outputs and every parameter gradient are
compared with an FP64 restatement of the same network that rounds to BF16 at the
same points (weights, hidden activations, output and hidden gradients); the
tolerance (0.5% of each block's norm) covers the rare BF16 rounding that an FP32
/ FP64 difference flips.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ls(gpu):
    import qpesim_gb300.learned_state as L
    return L


@pytest.mark.parametrize("M,N,K,tile", [(128, 16, 64, 16), (256, 64, 192, 64), (384, 256, 256, 256),
                                        (128, 512, 1024, 256), (256, 256, 4096, 256), (128, 64, 320, 64)])
def test_gemm_against_fp64(ls, M, N, K, tile):
    rng = np.random.default_rng(M + N + K)
    A = ls.round_bf16(rng.standard_normal((M, K)).astype(np.float32))
    B = ls.round_bf16(rng.standard_normal((N, K)).astype(np.float32))
    D = ls.gemm_bf16(A, B, tile)
    ref = A.astype(np.float64) @ B.astype(np.float64).T
    bound = K * 2.0 ** -23 * (np.abs(A).astype(np.float64) @ np.abs(B).astype(np.float64).T)
    assert np.all(np.abs(D - ref) <= bound + 1e-30)


def _gelu(x):
    from scipy.special import erf
    return 0.5 * x * (1 + erf(x / math.sqrt(2)))


def _gelu_grad(x):
    from scipy.special import erf
    return 0.5 * (1 + erf(x / math.sqrt(2))) + x * np.exp(-0.5 * x * x) / math.sqrt(2 * math.pi)


def _reference(ls, p, bits, n_bits, tla, tph, w, feats=None):
    """FP64 forward / backward with BF16 rounding where the device rounds (the
    extra input features, if any, are rounded to BF16 like the rest of X0)."""
    lay = ls.param_layout()
    P = {k: p[o:o + int(np.prod(s))].reshape(s).astype(np.float64) for k, (o, s) in lay.items()}
    rb = lambda x: ls.round_bf16(np.asarray(x, np.float32)).astype(np.float64)  # noqa: E731
    W = {k: rb(P[k]) for k in ("W1", "W2", "W3", "W4")}
    B = len(bits)
    X0 = np.zeros((B, 64))
    for j in range(n_bits):
        X0[:, j] = (bits >> np.uint64(j)) & np.uint64(1)
    if feats is not None:
        X0[:, n_bits:n_bits + feats.shape[1]] = rb(feats)
    Z1 = X0 @ W["W1"].T + P["b1"]
    H1 = rb(_gelu(Z1))
    Z2 = H1 @ W["W2"].T + P["b2"]
    H2 = rb(_gelu(Z2))
    Z3 = H2 @ W["W3"].T + P["b3"]
    H3 = rb(_gelu(Z3))
    Y = H3 @ W["W4"].T + P["b4"]
    dl, dp = Y[:, 0] - tla, Y[:, 1] - tph
    loss = float(np.sum(w * (dl * dl + 1 - np.cos(dp))) / B)
    dY = np.zeros((B, 16))
    dY[:, 0] = rb(2 * w * dl / B)
    dY[:, 1] = rb(w * np.sin(dp) / B)
    dZ3 = rb((dY @ W["W4"]) * _gelu_grad(Z3))
    dZ2 = rb((dZ3 @ W["W3"]) * _gelu_grad(Z2))
    dZ1 = rb((dZ2 @ W["W2"]) * _gelu_grad(Z1))
    g = {"W4": dY.T @ H3, "b4": dY.sum(0), "W3": dZ3.T @ H2, "b3": dZ3.sum(0), "W2": dZ2.T @ H1, "b2": dZ2.sum(0),
         "W1": dZ1.T @ X0, "b1": dZ1.sum(0)}
    return Y[:, :2], loss, g


@pytest.mark.parametrize("n_feat", [0, 2])
def test_mlp_forward_and_gradients_against_fp64(ls, n_feat):
    """Outputs, loss and every parameter gradient against the FP64 restatement;
    with n_feat > 0 the model also takes per-sample real features after the
    occupation bits."""
    n_bits, B = 20, 384
    m = ls.AmplitudeMLP(n_bits, batch=512, seed=3, n_feat=n_feat)
    rng = np.random.default_rng(5)
    p = m.get_params()
    lay = ls.param_layout()
    for k in ("b1", "b2", "b3", "b4"):  # nonzero biases so that their gradients and terms are exercised
        o, s = lay[k]
        p[o:o + int(np.prod(s))] = rng.standard_normal(int(np.prod(s))) * 0.1
    m.set_params(p)
    p = m.get_params()
    bits = rng.integers(0, 1 << n_bits, size=B).astype(np.uint64)
    tla = rng.standard_normal(B).astype(np.float32)
    tph = rng.uniform(-3, 3, B).astype(np.float32)
    w = rng.uniform(0.2, 2.0, B).astype(np.float32)
    feats = rng.uniform(-2, 2, (B, n_feat)).astype(np.float32) if n_feat else None
    y_ref, loss_ref, g_ref = _reference(ls, p, bits, n_bits, tla.astype(np.float64), tph.astype(np.float64),
                                        w.astype(np.float64), feats)
    y = m.forward(bits, feats)
    np.testing.assert_allclose(y, y_ref, rtol=0, atol=2e-2 * np.abs(y_ref).max())
    g, loss = m.gradients(bits, tla, tph, w, feats)
    assert abs(loss - loss_ref) <= 1e-2 * abs(loss_ref)
    for k, (o, s) in lay.items():
        got = g[o:o + int(np.prod(s))].reshape(s).astype(np.float64)
        want = np.zeros(s)
        if k == "W1":
            want[:, :] = g_ref[k]
        elif k in ("W4", "b4"):
            want[:2] = g_ref[k][:2]
        else:
            want = g_ref[k]
        err = np.linalg.norm(got - want) / max(np.linalg.norm(want), 1e-30)
        assert err < 5e-3, (k, err)
    # padding stays exactly zero
    o, s = lay["W1"]
    assert not np.any(g[o:o + 256 * 64].reshape(256, 64)[:, n_bits + n_feat:])


def test_mlp_training_fits_a_smooth_target(ls):
    n_bits = 12
    bits = np.arange(1 << n_bits, dtype=np.uint64)
    pop = np.array([bin(int(b)).count("1") for b in bits], np.float32)
    tla = (-0.5 * (pop - 6) ** 2 / 4).astype(np.float32)
    tph = (np.pi / 2 * (bits & np.uint64(3)).astype(np.float32) - 1.0).astype(np.float32)
    w = np.ones_like(tla)
    m = ls.AmplitudeMLP(n_bits, batch=1024, seed=11)
    m.set_data(bits, tla, tph, w)
    losses = m.train(400, lr=2e-3, seed=1)
    assert np.all(np.isfinite(losses))
    assert losses[-20:].mean() < 0.1 * losses[:5].mean()
