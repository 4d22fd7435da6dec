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


def test_build_datasets_offsets_runs():
    """Several recorded runs: rows concatenated in run order, every run's step
    indices after the previous run's, so train()'s held-back part is the last run."""
    runs = [_poly_history(3, n=10, seed=s) for s in (1, 2, 3)]
    X, R, k = mfx.build_datasets(runs)
    parts = [mfx.build_dataset(*r) for r in runs]
    assert len(X) == sum(len(p[0]) for p in parts)
    np.testing.assert_array_equal(X[:len(parts[0][0])], parts[0][0])
    off, start = 0, 0
    for Xp, Rp, kp in parts:
        sl = slice(start, start + len(kp))
        np.testing.assert_array_equal(k[sl], kp + off)
        np.testing.assert_array_equal(R[sl], Rp)
        assert start == 0 or k[sl].min() > k[start - 1]
        off += int(kp.max()) + 1
        start += len(kp)


def test_variant_states_are_seeded_displacements():
    """Variant 0 is the model's own initial state; the others displace every
    initial Gaussian (normalised wavefunctions, reproducible from the seed, the
    model left unchanged)."""
    from macaw_gb300.model import initial_wavefunction
    from tests.helpers import small_qvc
    model = small_qvc()
    before = dict(model.init_spf)
    a = mfx.variant_states(model, 3, seed=5)
    b = mfx.variant_states(model, 3, seed=5)
    assert model.init_spf == before
    A0, p0 = initial_wavefunction(model)
    np.testing.assert_array_equal(a[0][1], p0)
    np.testing.assert_array_equal(a[0][0], A0)
    for (Aa, pa), (Ab, pb) in zip(a, b):
        np.testing.assert_array_equal(pa, pb)
    assert np.abs(a[1][1] - p0).max() > 1e-3 and np.abs(a[2][1] - a[1][1]).max() > 1e-3
