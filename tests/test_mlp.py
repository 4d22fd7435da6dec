"""The extrapolator network's hand-written kernels against the CPU oracle.

Tolerances: the GPU and the oracle round the same quantities to BF16 (weights in
the forward pass, hidden activations), but FP32 sums in a different order can
move an activation across a BF16 rounding boundary (2^-8 relative), so
forward outputs agree to 1e-2 relative and the gradient vector to 3e-2 relative
in the L2 norm; the loss agrees to 1e-3 relative.
"""
import numpy as np
import pytest

from oracle import mlp as omlp

pytestmark = pytest.mark.gpu

WIDTHS = (8, 256, 256, 256, 4)


def _data(m, seed):
    rng = np.random.default_rng(seed)
    X = rng.normal(size=(m, WIDTHS[0])).astype(np.float32)
    T = np.stack([np.sin(X[:, 0]) * X[:, 1], np.cos(X[:, 2]), X[:, 3] * X[:, 4], np.tanh(X[:, 5] - X[:, 6])],
                 axis=1).astype(np.float32)
    return X, T


def test_forward_matches_oracle():
    from macaw_gb300.capi import Mlp
    net = Mlp(WIDTHS, seed=3)
    X, _ = _data(700, 1)
    Y = net.predict(X)
    ref = omlp.forward(net.get_params(), WIDTHS, X)[-1]
    assert np.linalg.norm(Y - ref) <= 1e-2 * np.linalg.norm(ref)


def test_gradient_matches_oracle():
    from macaw_gb300.capi import Mlp
    net = Mlp(WIDTHS, seed=4)
    X, T = _data(513, 2)
    loss, g = net.grad(X, T)
    rloss, rg = omlp.loss_and_grad(net.get_params(), WIDTHS, X, T)
    assert abs(loss - rloss) <= 1e-3 * rloss
    assert np.linalg.norm(g - rg) <= 3e-2 * np.linalg.norm(rg)
    # every layer's block individually
    off = 0
    for k, n in zip(WIDTHS[:-1], WIDTHS[1:]):
        blk = slice(off, off + n * k + n)
        assert np.linalg.norm(g[blk] - rg[blk]) <= 5e-2 * np.linalg.norm(rg[blk]) + 1e-9
        off += n * k + n


def test_training_reduces_loss():
    from macaw_gb300.capi import Mlp
    net = Mlp(WIDTHS, seed=5)
    X, T = _data(20000, 3)
    l0, _ = net.grad(X[:4096], T[:4096])
    l1 = net.train(X, T, batch=2048, epochs=15, lr=2e-3)
    l2, _ = net.grad(X[:4096], T[:4096])
    assert l2 < 0.1 * l0, (l0, l1, l2)
