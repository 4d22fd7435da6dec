"""Learned mean-field extrapolation in CMF2: training data from plain CMF2 runs,
the network's gain over the method without it, and the assisted propagation.

Gain is measured two ways: (1) on held-out steps, the residual left by the
quartic extrapolation of the last five step starts plus the network's correction
is printed beside the quartic's and the quadratic's, and may not exceed the
quartic's by more than 10 %;
(2) CMF2 with the network evaluates fewer mean fields per simulated fs than plain
CMF2, while C(t) and the populations stay within 1e-6 / 1e-5 of plain CMF2.
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
    # network; the network's (validation-gated) correction may not make it worse
    assert np.all(left <= 1.1 * base), (base, left)
    assert left[2] < 0.5 * quad[2] and left[3] < 0.5 * quad[3], (quad, left)

    # assisted propagation over the same interval, then C(t) at a common time
    assisted = GpuCore(model)
    assisted.mfx_attach(net, fscale, tscale, tol=model.eps_int)
    t_mlp, eom_mlp = _run(assisted, model, A0, psi0, T_FS / AU2FS)
    stats = assisted.mfx_stats()
    assert stats["mlp_steps"] > 0
    assert eom_mlp / t_mlp < eom_plain / t_plain
    tc = max(t_plain, t_mlp) + 0.05 / AU2FS
    outs = []
    for core, t in ((plain, t_plain), (assisted, t_mlp)):
        tt, _, _, _, _ = core.propagate_interval(INT_CMF2, tc, t, model.tout * 0.01)
        outs.append(core.observables(tt))
    assert abs(outs[0]["auto"] - outs[1]["auto"]) < 1e-6
    assert np.abs(outs[0]["pop"] - outs[1]["pop"]).max() < 1e-5
