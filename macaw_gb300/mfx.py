"""Learned mean-field extrapolation for CMF2: data, training and evaluation.

A snapshot is every density matrix and mean field of the grid modes at one
time (``GpuCore.mfx_size()`` complex entries).  Plain CMF2 steps recorded with
``GpuCore.mfx_record`` give, per accepted step k, the snapshot at the step
start t_k and at its half step t_k + h_k/2.

The extrapolator replaces the step-start mean-field evaluation of CMF2
(cmf2_base.f90:78-87): from the half-step snapshots z_0..z_4 of the last five
steps (times s_j = t_j + h_j/2) it predicts the snapshot at the next step start
tau_0 = t_k and, for the check against the computed half-step fields, at its
half step tau_1 = t_k + h_k/2.  P_o(tau) is the Lagrange polynomial through the
last o+1 history values and inc_o = P_o - P_{o-1} (P_0 = z_4) its Newton
increment; the extrapolation without the network is P_4 (quartic).  The network
sees, per entry, Re/Im of inc_1..inc_4 at tau_0 and tau_1 divided by the
entry's own scale s = |inc_1(tau_1)| + |inc_2(tau_1)| + 1e-12 S (S the RMS over
all entries of |inc_1(tau_1)|), and the spacing ratios (s_1-s_0, s_2-s_1,
s_3-s_2, tau_1-s_4) / (s_4-s_3); every input column is divided by its scale
``fscale``.  It predicts the residual z(tau) - P_4(tau) at tau_0 and tau_1 in
units of s times the output column scale ``tscale``.  The per-entry scale keeps
every correction proportional to the entry's own variation: the mean fields of
weakly occupied SPFs are small, and the regularised inverse of rho in the SPF
equations magnifies any error of theirs.  The device builds the same inputs
(mfx_features_kernel).
"""
from __future__ import annotations

from typing import Tuple

import numpy as np

NHIST = 5
NFEAT = 20
NOUT = 4
WIDTHS = (NFEAT, 256, 256, 256, NOUT)
GATE_GAIN = 0.9   # a correction column is kept when it removes >= 10 % of the validation residual


def lagrange_tail(ts, first, tau):
    """Weights at tau of the polynomial through ts[first:] (zero for earlier points)."""
    n = len(ts)
    w = np.zeros(n)
    for j in range(first, n):
        p = 1.0
        for k in range(first, n):
            if k != j:
                p *= (tau - ts[k]) / (ts[j] - ts[k])
        w[j] = p
    return w


def coefficients(ts, taus):
    """Increment weights inc[tau][o-1][j], quartic weights base[tau][j] and the
    ratios for the history times ts and the two prediction times taus."""
    n = len(ts)
    inc = np.zeros((2, n - 1, n))
    base = np.zeros((2, n))
    for it, tau in enumerate(taus):
        prev = np.zeros(n)
        prev[-1] = 1.0
        for o in range(1, n):
            w = lagrange_tail(ts, n - 1 - o, tau)
            inc[it, o - 1] = w - prev
            prev = w
        base[it] = prev
    d = ts[-1] - ts[-2]
    ratio = np.array([(ts[j + 1] - ts[j]) / d for j in range(n - 2)] + [(taus[1] - ts[-1]) / d])
    return inc, base, ratio


def features(Z, ts, taus):
    """Unscaled inputs (E, 20), the quartic extrapolations (2, E) and the
    per-entry scales s (E) for the history Z (5, E) at times ts and the
    prediction times taus."""
    inc, base, ratio = coefficients(ts, taus)
    incs = np.einsum("toj,je->toe", inc, Z)          # (2, 4, E)
    Sg = max(float(np.sqrt(np.mean(np.abs(incs[1, 0]) ** 2))), 1e-300)
    S = np.abs(incs[1, 0]) + np.abs(incs[1, 1]) + 1e-12 * Sg + 1e-300
    E = Z.shape[1]
    X = np.empty((E, NFEAT))
    col = 0
    for it in range(2):
        for o in range(NHIST - 1):
            X[:, col] = incs[it, o].real / S
            X[:, col + 1] = incs[it, o].imag / S
            col += 2
    X[:, col:] = ratio[None, :]
    Q = base @ Z
    return X, Q, S


def build_dataset(t0, h, s0, sh) -> Tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Samples of consecutive recorded steps: for step k, the history is the
    half-step snapshots of steps k-5 .. k-1, the targets the snapshot at the step
    start t_k and at its half step.  Returns the unscaled inputs X, the residual
    targets R of the quartic extrapolation (Re/Im at the step start, Re/Im at the
    half step, in units of each entry's scale s) and the step index of every row."""
    Xs, Rs, ks = [], [], []
    for k in range(NHIST, len(t0)):
        ok = all(np.isclose(t0[j + 1], t0[j] + h[j], rtol=0, atol=1e-9 * max(1.0, abs(t0[j])))
                 for j in range(k - NHIST, k))
        if not ok:
            continue
        ts = t0[k - NHIST:k] + 0.5 * h[k - NHIST:k]
        taus = (t0[k], t0[k] + 0.5 * h[k])
        X, Q, S = features(sh[k - NHIST:k], ts, taus)
        r0 = (s0[k] - Q[0]) / S
        r1 = (sh[k] - Q[1]) / S
        Xs.append(X)
        Rs.append(np.stack([r0.real, r0.imag, r1.real, r1.imag], axis=1))
        ks.append(np.full(len(X), k))
    if not Xs:
        raise ValueError("not enough consecutive recorded steps")
    return np.concatenate(Xs), np.concatenate(Rs), np.concatenate(ks)


def variant_states(model, nvar, seed=0, shift=0.3):
    """`nvar` seeded variants of the model's initial wavefunction for training
    data: variant 0 is the model's own initial state; in the others the initial
    Gaussian of every DVR DOF is displaced by up to +-shift in position and in
    momentum (uniform, in the DOF's coordinate units).  Returns [(A, psi)]."""
    from .model import initial_wavefunction
    saved = dict(model.init_spf)
    rng = np.random.default_rng(seed)
    out = []
    try:
        for v in range(nvar):
            model.init_spf.clear()
            model.init_spf.update(saved)
            if v > 0:
                for d in range(model.ndof):
                    kind, par = saved.get(d, ("gauss", (0.0, 0.0, 0.707107)))
                    if kind != "gauss":
                        continue
                    x0, p0, dx = par
                    model.init_spf[d] = ("gauss", (x0 + rng.uniform(-shift, shift),
                                                   p0 + rng.uniform(-shift, shift), dx))
            out.append(initial_wavefunction(model))
    finally:
        model.init_spf.clear()
        model.init_spf.update(saved)
    return out


def build_datasets(records):
    """build_dataset over several recorded runs [(t0, h, s0, sh)]: rows
    concatenated in run order, step indices offset so that every run's steps
    follow the previous run's (the last run is then the held-back part of train)."""
    Xs, Rs, ks = [], [], []
    off = 0
    for rec in records:
        X, R, k = build_dataset(*rec)
        Xs.append(X)
        Rs.append(R)
        ks.append(k + off)
        off += int(k.max()) + 1
    return np.concatenate(Xs), np.concatenate(Rs), np.concatenate(ks)


def train(X, R, steps=None, seed=1, epochs=20, batch=4096, lr=1e-3, widths=WIDTHS, val_frac=0.2):
    """Train the GPU network; returns (net, fscale, tscale, loss).  Input columns
    are scaled to an RMS of 1/4 (keeping tanh near its linear range), targets to 1.

    The polynomial order (1-4) is chosen per prediction time on all rows
    (``net.orders``: the network learns the residual of that polynomial).  The
    last `val_frac` of the steps (or of the rows, without `steps`) are held back
    from the fit; on them, per output column the network's correction is shrunk
    by the factor
    beta in [0, 1] that minimises the residual on them (folded into tscale), and
    switched off (beta = 0) unless it removes at least 10 % of that residual, so
    a correction that does not generalise is not applied."""
    from .capi import Mlp
    if steps is not None:
        cut = np.quantile(np.unique(steps), 1.0 - val_frac)
        fit, val = steps <= cut, steps > cut
    else:
        n_fit = int(len(X) * (1.0 - val_frac))
        fit = np.zeros(len(X), dtype=bool)
        fit[:n_fit] = True
        val = ~fit
    # the polynomial order per prediction time (step start, half step) with the
    # smallest residual over all rows; the network learns the residual of that order
    orders = []
    for tau in range(2):
        cols = slice(2 * tau, 2 * tau + 2)
        rms = [np.mean(poly_residual(X, R, o)[:, cols] ** 2) for o in range(1, NHIST)]
        orders.append(1 + int(np.argmin(rms)))
    Ro = order_residual(X, R, orders)
    fscale = 4.0 * np.sqrt(np.mean(X[fit] ** 2, axis=0))
    fscale = np.where(fscale > 0, fscale, 1.0)
    tscale = np.sqrt(np.mean(Ro[fit] ** 2, axis=0))
    tscale = np.where(tscale > 0, tscale, 1.0)
    net = Mlp(widths, seed=seed)
    net.orders = tuple(orders)
    rng = np.random.default_rng(seed)
    idx = np.flatnonzero(fit)[rng.permutation(int(fit.sum()))]
    loss = net.train((X[idx] / fscale).astype(np.float32), (Ro[idx] / tscale).astype(np.float32),
                     batch=batch, epochs=epochs, lr=lr)
    if val.any():
        P = net_output(net, fscale, tscale, X[val])
        Rv = Ro[val]
        beta = np.clip(np.sum(P * Rv, axis=0) / np.maximum(np.sum(P * P, axis=0), 1e-300), 0.0, 1.0)
        before = np.sum(Rv ** 2, axis=0)
        after = np.sum((Rv - beta * P) ** 2, axis=0)
        beta = np.where(after < GATE_GAIN * before, beta, 0.0)   # keep only clear gains
        tscale = tscale * beta
    return net, fscale, tscale, loss


def net_output(net, fscale, tscale, X):
    """The network's correction (units of S) to the polynomial of its orders."""
    return net.predict((X / fscale).astype(np.float32)).astype(np.float64) * tscale


def order_residual(X, R, orders):
    """Targets relative to the polynomials of `orders` (step start, half step)
    instead of the quartic."""
    Ro = R.copy()
    for tau, o in enumerate(orders):
        cols = slice(2 * tau, 2 * tau + 2)
        Ro[:, cols] = poly_residual(X, R, o)[:, cols]
    return Ro


def predict(net, fscale, tscale, X):
    """The extrapolator's prediction as a correction to the quartic (units of S):
    the step from the quartic to the polynomial of the chosen order plus the
    network's correction -- what the device adds to the quartic."""
    orders = getattr(net, "orders", (NHIST - 1, NHIST - 1))
    P = net_output(net, fscale, tscale, X)
    shift = order_residual(X, np.zeros((len(X), NOUT)), orders)
    return P - shift


def poly_residual(X, R, order):
    """Residual of the polynomial through the last order+1 history snapshots
    (1 <= order <= 4), from the quartic residual R by adding back the increments
    above `order`."""
    P = np.zeros_like(R)
    for o in range(order + 1, NHIST):
        P[:, 0] += X[:, 2 * (o - 1)]
        P[:, 1] += X[:, 2 * (o - 1) + 1]
        P[:, 2] += X[:, 8 + 2 * (o - 1)]
        P[:, 3] += X[:, 8 + 2 * (o - 1) + 1]
    return R + P


def prediction_errors(net, fscale, tscale, X, R):
    """RMS per output column of the residual left by the quartic extrapolation
    alone (R) and by the learned extrapolator (polynomial of the chosen order plus
    the network), in units of S."""
    P = predict(net, fscale, tscale, X)
    base = np.sqrt(np.mean(R ** 2, axis=0))
    left = np.sqrt(np.mean((R - P) ** 2, axis=0))
    return base, left
