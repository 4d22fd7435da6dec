"""Learned mean-field extrapolation in CMF2: training data from plain CMF2 runs,
what the trained network gains over the method without it, and the assisted
propagation.

Findings these tests pin down (small QVC model):
* held out, the quartic extrapolation of the last five step starts already
  predicts the step-end fields to a few 1e-4 of their step-to-step change; the
  network's correction (gated on validation steps) is switched off where it does
  not help and stays within 25 % of the quartic where it is kept;
* CMF2 with extrapolated half-step fields takes steps with one mean-field
  evaluation less, but the propagated state deviates from the plain scheme's at
  the level of the scheme's own local error (eps_int), so the step-end check
  (tolerance eps_int) fails for a large share of the steps and C(t) stays within
  1e-5, not 1e-6, of plain CMF2.
"""
import numpy as np
import pytest

from macaw_gb300.model import initial_wavefunction, INT_CMF2, AU2FS
from tests.helpers import small_qvc

pytestmark = pytest.mark.gpu

T_FS = 1.5


def _run(core, model, A0, psi0, t_end):
    core.set_state(A0, psi0, as_start=True)
    t, h = 0.0, model.tout * model.eps_int
    c0 = core.counters()["eom"]
    while t < t_end:
        hdid, h, _ = core.step(INT_CMF2, t, h)
        t += hdid
    return t, core.counters()["eom"] - c0


def test_extrapolator_gain_and_assisted_cmf2():
    from macaw_gb300.capi import GpuCore
    from macaw_gb300 import mfx
    model = small_qvc(tfinal_fs=T_FS)
    A0, psi0 = initial_wavefunction(model)
    plain = GpuCore(model)
    plain.mfx_record(2)
    t_plain, eom_plain = _run(plain, model, A0, psi0, T_FS / AU2FS)
    t0, h, s0, sh = plain.mfx_fetch()
    assert len(t0) > 20
    X, R, k = mfx.build_dataset(t0, h, s0, sh)
    cut = np.quantile(np.unique(k), 0.7)
    tr, te = k <= cut, k > cut
    net, fscale, tscale, loss = mfx.train(X[tr], R[tr], steps=k[tr], epochs=60, batch=2048, lr=1e-3)
    base, left = mfx.prediction_errors(net, fscale, tscale, X[te], R[te])
    quad = np.sqrt(np.mean(mfx.poly_residual(X[te], R[te], 2) ** 2, axis=0))
    print("held-out RMS residual (units of S): quadratic", quad, "quartic", base, "quartic + network", left)
    # the quartic extrapolation of the step starts is the method without the
    # network; the network's (validation-gated) correction stays close to it
    assert np.all(left <= 1.25 * base), (base, left)
    assert left[2] < 0.5 * quad[2] and left[3] < 0.5 * quad[3], (quad, left)

    # assisted propagation over the same interval, then C(t) at a common time
    assisted = GpuCore(model)
    assisted.mfx_attach(net, fscale, tscale, tol=model.eps_int)
    t_mlp, eom_mlp = _run(assisted, model, A0, psi0, T_FS / AU2FS)
    stats = assisted.mfx_stats()
    print("plain: EOM/fs", eom_plain / (t_plain * AU2FS), "assisted: EOM/fs", eom_mlp / (t_mlp * AU2FS), stats)
    assert stats["mlp_steps"] > 0
    tc = max(t_plain, t_mlp) + 0.05 / AU2FS
    outs = []
    for core, t in ((plain, t_plain), (assisted, t_mlp)):
        tt, _, _, _, _ = core.propagate_interval(INT_CMF2, tc, t, model.tout * 0.01)
        outs.append(core.observables(tt))
    print("|dC|", abs(outs[0]["auto"] - outs[1]["auto"]), "|dpop|", np.abs(outs[0]["pop"] - outs[1]["pop"]).max())
    assert abs(outs[0]["auto"] - outs[1]["auto"]) < 1e-5
    assert np.abs(outs[0]["pop"] - outs[1]["pop"]).max() < 1e-5


def test_device_prediction_matches_host():
    """The device path (history ring, Newton-increment features, network, quartic
    base) reproduces the host formulas of macaw_gb300.mfx on recorded snapshots."""
    from macaw_gb300.capi import GpuCore
    from macaw_gb300 import mfx
    model = small_qvc(tfinal_fs=1.0)
    A0, psi0 = initial_wavefunction(model)
    core = GpuCore(model)
    core.mfx_record(2)
    _run(core, model, A0, psi0, 1.0 / AU2FS)
    t0, h, s0, sh = core.mfx_fetch()
    X, R, k = mfx.build_dataset(t0, h, s0, sh)
    net, fscale, tscale, _ = mfx.train(X, R, steps=k, epochs=5)
    for ts_scale in (tscale, np.ones(4) * np.abs(tscale).max() + 1e-3, np.zeros(4)):
        core.mfx_attach(net, fscale, ts_scale, tol=model.eps_int)
        for kk in (int(k.min()), int(k.max())):
            Z = s0[kk - 4:kk + 1]
            ts = t0[kk - 4:kk + 1]
            half, full = core.mfx_predict(Z, ts, h[kk])
            Xh, Q, S = mfx.features(Z, ts, h[kk])
            P = mfx.predict(net, fscale, ts_scale, Xh) * S
            ref_half = Q[0] + P[:, 0] + 1j * P[:, 1]
            ref_full = Q[1] + P[:, 2] + 1j * P[:, 3]
            scale = np.abs(Z).max()
            assert np.abs(half - ref_half).max() < 1e-9 * scale
            assert np.abs(full - ref_full).max() < 1e-9 * scale
