"""Learned mean-field extrapolation in CMF2: training data from plain CMF2 runs,
what the trained network adds to the extrapolation, and the assisted
propagation.

The extrapolator replaces the step-start mean-field evaluation of CMF2
(cmf2_base.f90:78-87) by a prediction from the half-step mean fields of the
last five steps; the half-step evaluation (:122-130) stays and checks the
prediction.  Training data are plain CMF2 runs of four seeded variants of the
initial state (displaced Gaussians); the model's own initial state is held out.
What these tests pin down (small QVC model, CMF2 tolerance 1e-5):
* on the held-out run, the learned extrapolator (polynomial order chosen per
  prediction time on the training runs, plus the gated network) leaves at least
  15 % less RMS residual over its four outputs than the better of the quadratic
  and quartic extrapolations, and no output more than 15 % above it;
* the assisted propagation of the held-out state, extrapolating only after
  steps whose first attempt used less than half the tolerance, needs fewer
  mean-field evaluations per simulated fs than plain CMF2 (one per extrapolated
  step instead of two) and stays within 1e-6 of it in C(t) and within 1e-5 in
  the populations.  Without that gate the extrapolation error, although ~1e-7
  of the mean fields, shifts the CMF2 error estimate of steps that the step
  control runs at error ~1, and the extra rejected attempts cost more than the
  saved evaluations.
"""
import numpy as np
import pytest

from macaw_gb300.model import initial_wavefunction, INT_CMF2, AU2FS
from tests.helpers import small_qvc

pytestmark = pytest.mark.gpu

T_FS = 1.5
NVAR = 5


def _run(core, model, A0, psi0, t_end):
    core.set_state(A0, psi0, as_start=True)
    t, h = 0.0, model.tout * model.eps_int
    c0 = core.counters()["eom"]
    while t < t_end:
        hdid, h, _ = core.step(INT_CMF2, t, h)
        t += hdid
    return t, h, core.counters()["eom"] - c0


def _recorded(model, A0, psi0, t_fs):
    from macaw_gb300.capi import GpuCore
    rec = GpuCore(model)
    rec.mfx_record(2)
    _run(rec, model, A0, psi0, t_fs / AU2FS)
    data = rec.mfx_fetch()
    rec.close()
    return data


@pytest.fixture(scope="module")
def trained():
    """Network trained on variants 1..4; the dataset of variant 0 held out."""
    from macaw_gb300 import mfx
    model = small_qvc(tfinal_fs=T_FS)
    states = mfx.variant_states(model, NVAR, seed=3)
    records = [_recorded(model, A, psi, T_FS) for A, psi in states]
    assert all(len(r[0]) > 20 for r in records)
    X, R, k = mfx.build_datasets(records[1:])
    net, fscale, tscale, _ = mfx.train(X, R, steps=k, epochs=60, batch=2048, lr=1e-3,
                                       val_frac=1.0 / (NVAR - 1))
    return model, states[0], (net, fscale, tscale), mfx.build_dataset(*records[0])


def test_extrapolator_held_out_variant(trained):
    from macaw_gb300 import mfx
    _, _, (net, fscale, tscale), (Xh, Rh, _) = trained
    base, left = mfx.prediction_errors(net, fscale, tscale, Xh, Rh)
    quad = np.sqrt(np.mean(mfx.poly_residual(Xh, Rh, 2) ** 2, axis=0))
    print("orders", net.orders, "held-out RMS residual (units of S): quadratic", quad,
          "quartic", base, "learned", left)
    best = np.minimum(base, quad)
    assert np.sqrt(np.mean(left ** 2)) <= 0.85 * np.sqrt(np.mean(best ** 2)), (quad, base, left)
    assert np.all(left <= 1.15 * best), (quad, base, left)


def test_assisted_cmf2_fewer_evaluations(trained):
    from macaw_gb300.capi import GpuCore
    model, (A0, psi0), (net, fscale, tscale), _ = trained
    # plain and assisted propagation over the same interval, then C(t) at a common time
    plain = GpuCore(model)
    t_plain, h_plain, eom_plain = _run(plain, model, A0, psi0, T_FS / AU2FS)
    assisted = GpuCore(model)
    assisted.mfx_attach(net, fscale, tscale, tol=model.eps_int)
    assisted.mfx_gate(0.5)
    t_mlp, h_mlp, eom_mlp = _run(assisted, model, A0, psi0, T_FS / AU2FS)
    stats = assisted.mfx_stats()
    rate_plain = eom_plain / (t_plain * AU2FS)
    rate_mlp = eom_mlp / (t_mlp * AU2FS)
    print("plain: EOM/fs", rate_plain, "assisted: EOM/fs", rate_mlp, stats)
    assert stats["mlp_steps"] > 0
    assert rate_mlp < rate_plain
    tc = max(t_plain, t_mlp) + 0.05 / AU2FS
    outs = []
    for core, t, hh in ((plain, t_plain, h_plain), (assisted, t_mlp, h_mlp)):
        tt, _, _, _, _ = core.propagate_interval(INT_CMF2, tc, t, hh)
        outs.append(core.observables(tt))
    dC = abs(outs[0]["auto"] - outs[1]["auto"])
    dpop = np.abs(outs[0]["pop"] - outs[1]["pop"]).max()
    print("|dC|", dC, "|dpop|", dpop)
    assert dC < 1e-6
    assert dpop < 1e-5


def test_device_prediction_matches_host():
    """The device path (history ring, Newton-increment features, network, quartic
    base) reproduces the host formulas of macaw_gb300.mfx on recorded snapshots."""
    from macaw_gb300.capi import GpuCore
    from macaw_gb300 import mfx
    model = small_qvc(tfinal_fs=1.0)
    A0, psi0 = initial_wavefunction(model)
    t0, h, s0, sh = _recorded(model, A0, psi0, 1.0)
    X, R, k = mfx.build_dataset(t0, h, s0, sh)
    net, fscale, tscale, _ = mfx.train(X, R, steps=k, epochs=5)
    core = GpuCore(model)
    for ts_scale in (tscale, np.ones(4) * np.abs(tscale).max() + 1e-3, np.zeros(4)):
        core.mfx_attach(net, fscale, ts_scale, tol=model.eps_int)
        for kk in (int(k.min()), int(k.max())):
            Z = sh[kk - 5:kk]
            ts = t0[kk - 5:kk] + 0.5 * h[kk - 5:kk]
            taus = (t0[kk], t0[kk] + 0.5 * h[kk])
            p0, p1 = core.mfx_predict(Z, ts, *taus)
            Xh, Q, S = mfx.features(Z, ts, taus)
            P = mfx.predict(net, fscale, ts_scale, Xh) * S[:, None]
            ref0 = Q[0] + P[:, 0] + 1j * P[:, 1]
            ref1 = Q[1] + P[:, 2] + 1j * P[:, 3]
            scale = np.abs(Z).max()
            assert np.abs(p0 - ref0).max() < 1e-9 * scale
            assert np.abs(p1 - ref1).max() < 1e-9 * scale
