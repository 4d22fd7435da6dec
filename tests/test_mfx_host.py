"""Host side of the learned mean-field extrapolation: the Newton-increment inputs
and targets built from recorded snapshots (no GPU)."""
import numpy as np

from macaw_gb300 import mfx


def _poly_history(deg, n=12, E=7, seed=3):
    rng = np.random.default_rng(seed)
    c = rng.normal(size=(deg + 1, E)) + 1j * rng.normal(size=(deg + 1, E))
    h = 0.3 * 1.2 ** np.arange(n)
    t0 = np.concatenate([[0.0], np.cumsum(h)])[:n]

    def z(t):
        return sum(c[p] * t ** p for p in range(deg + 1))
    s0 = np.stack([z(t) for t in t0])
    sh = np.stack([z(t + 0.5 * hh) for t, hh in zip(t0, h)])
    return t0, h, s0, sh


def test_quartic_targets_vanish_for_quartic_fields():
    X, R, k = mfx.build_dataset(*_poly_history(4))
    assert np.abs(R).max() < 1e-8
    assert X.shape[1] == mfx.NFEAT and R.shape[1] == mfx.NOUT


def test_lower_orders_from_increments():
    """For quartic fields the quadratic residual is exactly the order-3 and order-4
    increments; for quadratic fields every order from 2 up is exact."""
    X, R, k = mfx.build_dataset(*_poly_history(4))
    r2 = mfx.poly_residual(X, R, 2)
    assert np.abs(r2).max() > 1e-6
    assert np.abs(mfx.poly_residual(X, R, 3)).max() > 1e-3 * np.abs(r2).max()
    Xq, Rq, _ = mfx.build_dataset(*_poly_history(2))
    assert np.abs(mfx.poly_residual(Xq, Rq, 2)).max() < 1e-9
    assert np.abs(mfx.poly_residual(Xq, Rq, 1)).max() > 1e-6


def test_ratios_and_scale():
    t0, h, s0, sh = _poly_history(3)
    X, R, k = mfx.build_dataset(t0, h, s0, sh)
    first = X[k == k.min()][0]
    j = int(k.min())
    s = t0 + 0.5 * h           # half-step times of the history
    d = s[j - 1] - s[j - 2]
    np.testing.assert_allclose(first[16:], [(s[j - 4] - s[j - 5]) / d, (s[j - 3] - s[j - 4]) / d,
                                            (s[j - 2] - s[j - 3]) / d, (t0[j] + 0.5 * h[j] - s[j - 1]) / d],
                               rtol=1e-12)
    # every entry's scale is |inc_1| + |inc_2| at the step end (plus a floor of
    # 1e-12 of the RMS of inc_1): the scaled pair sums to one
    rows = X[k == k.min()]
    pair = np.hypot(rows[:, 8], rows[:, 9]) + np.hypot(rows[:, 10], rows[:, 11])
    np.testing.assert_allclose(pair, 1.0, rtol=1e-9)
