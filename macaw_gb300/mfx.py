"""Learned mean-field extrapolation for CMF2: data, training and use.

A snapshot is every density matrix and mean field of the grid modes at one
time (``GpuCore.mfx_size()`` complex entries).  Plain CMF2 steps recorded with
``GpuCore.mfx_record`` give, per accepted step k, the snapshot at the step
start t_k and at its half step t_k + h_k/2; the snapshot at the step end is
the next step's start.  For every entry z the network sees its last three
step-start values (z0, z1, z2 at t_{k-2}, t_{k-1}, t_k) scaled by
s = max|z_i|, and the ratios (t1-t0)/(t2-t1) and h/(t2-t1); it predicts the
correction to the quadratic extrapolation of z to t_k + h/2 and t_k + h, in
units of s * tscale.  The same features are built on the device
(mfx_features_kernel) when the trained network replaces the half-step mean
fields inside CMF2 (cmf2_base.f90:122-130).
"""
from __future__ import annotations

from typing import Tuple

import numpy as np

WIDTHS = (8, 256, 256, 256, 4)


def lagrange_weights(t0, t1, t2, tau):
    return np.array([(tau - t1) * (tau - t2) / ((t0 - t1) * (t0 - t2)),
                     (tau - t0) * (tau - t2) / ((t1 - t0) * (t1 - t2)),
                     (tau - t0) * (tau - t1) / ((t2 - t0) * (t2 - t1))])


def features(z0, z1, z2, t0, t1, t2, h):
    s = np.maximum(np.maximum(np.abs(z0), np.abs(z1)), np.maximum(np.abs(z2), 1e-300))
    X = np.empty((z0.size, 8), dtype=np.float32)
    for j, z in enumerate((z0, z1, z2)):
        X[:, 2 * j] = (z.real / s).astype(np.float32)
        X[:, 2 * j + 1] = (z.imag / s).astype(np.float32)
    X[:, 6] = np.float32((t1 - t0) / (t2 - t1))
    X[:, 7] = np.float32(h / (t2 - t1))
    return X, s


def quadratic(z0, z1, z2, t0, t1, t2, tau):
    w = lagrange_weights(t0, t1, t2, tau)
    return w[0] * z0 + w[1] * z1 + w[2] * z2


def build_dataset(t0, h, s0, sh) -> Tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Samples from consecutive recorded steps: features X, raw residual targets R
    (in units of s; columns Re/Im at the half step, Re/Im at the step end), and the
    step index of every row."""
    Xs, Rs, ks = [], [], []
    for k in range(2, len(t0) - 1):
        if not np.isclose(t0[k + 1], t0[k] + h[k], rtol=0, atol=1e-9 * max(1.0, abs(t0[k]))):
            continue
        ta, tb, tc = t0[k - 2], t0[k - 1], t0[k]
        z0, z1, z2 = s0[k - 2], s0[k - 1], s0[k]
        X, s = features(z0, z1, z2, ta, tb, tc, h[k])
        qh = quadratic(z0, z1, z2, ta, tb, tc, tc + 0.5 * h[k])
        qf = quadratic(z0, z1, z2, ta, tb, tc, tc + h[k])
        rh = (sh[k] - qh) / s
        rf = (s0[k + 1] - qf) / s
        R = np.stack([rh.real, rh.imag, rf.real, rf.imag], axis=1)
        Xs.append(X)
        Rs.append(R)
        ks.append(np.full(len(X), k))
    if not Xs:
        raise ValueError("not enough consecutive recorded steps")
    return np.concatenate(Xs), np.concatenate(Rs), np.concatenate(ks)


def train(X, R, seed=1, epochs=20, batch=8192, lr=1e-3, widths=WIDTHS):
    """Train the GPU network on residuals R scaled by their RMS; returns (net, tscale, loss)."""
    from .capi import Mlp
    tscale = float(np.sqrt(np.mean(R ** 2))) or 1.0
    net = Mlp(widths, seed=seed)
    rng = np.random.default_rng(seed)
    perm = rng.permutation(len(X))
    loss = net.train(X[perm], (R[perm] / tscale).astype(np.float32), batch=batch, epochs=epochs, lr=lr)
    return net, tscale, loss


def prediction_errors(net, tscale, X, R):
    """RMS of the half-step / step-end residual left by the quadratic extrapolation
    alone (R) and by quadratic + network (R - prediction), in units of s."""
    P = net.predict(X).astype(np.float64) * tscale
    base = np.sqrt(np.mean(R ** 2, axis=0))
    left = np.sqrt(np.mean((R - P) ** 2, axis=0))
    return base, left
