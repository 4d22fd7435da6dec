"""Ensembles of wavepackets of uneven shape (mctdh_ens_*): every EOM stage is one
launch over all members, and adaptive RK runs the members in lockstep.

A member's descriptors keep their order inside the merged launches, so each
member's arithmetic is the same as in its own context: derivatives and whole
propagations agree with single-context runs to rounding (checked at 1e-13).
"""
import numpy as np
import pytest

from macaw_gb300.model import initial_wavefunction, INT_RK45, INT_DOPRI, AU2FS
from macaw_gb300.generate import ensemble
from tests.helpers import small_lvc, small_qvc, random_state

pytestmark = pytest.mark.gpu


def _members():
    return [small_lvc(), small_qvc(), small_qvc(nstates=2, ndof=6, grid=5, nspf=3),
            small_qvc(nstates=3, ndof=4, grid=7, nspf=3)]


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def test_ensemble_eom_matches_single_contexts():
    from macaw_gb300.capi import Ensemble, GpuCore
    models = _members()
    ens = Ensemble(models)
    states = [random_state(m, seed=10 + i) for i, m in enumerate(models)]
    for i, (A, psi) in enumerate(states):
        ens.set_state(i, A, psi)
    got = ens.calc_derivs()
    for m, (A, psi), (dA, dpsi) in zip(models, states, got):
        rA, rpsi = GpuCore(m).calc_derivs(A, psi)
        assert _rel(dA, rA) < 1e-13
        assert _rel(dpsi, rpsi) < 1e-13


@pytest.mark.parametrize("method,shapes", [(INT_RK45, False), (INT_DOPRI, False), (INT_RK45, "persistent")])
def test_ensemble_propagation_matches_single_contexts(method, shapes):
    """Lockstep RK with per-member step control: each member follows the step
    sequence its own context takes, so C(t), populations, norm and energy agree.
    With persistent CTAs (each walking the batch's blocks) the block partials and
    so the arithmetic are the same."""
    from macaw_gb300.capi import Ensemble, GpuCore
    models = _members()
    # the planned launch shapes: the autotuner may re-tile the contractions, which
    # reorders their partial sums
    ens = Ensemble(models, autotune=shapes)
    if shapes == "persistent":
        tn = ens.tuning()
        assert tn["persistent_prod_ctas"] > 0 and tn["persistent_hole_ctas"] > 0
    starts = [initial_wavefunction(m) for m in models]
    for i, (A, psi) in enumerate(starts):
        ens.set_state(i, A, psi, as_start=True)
    tnext = 0.5 / AU2FS
    t = np.zeros(len(models))
    step = np.array([m.tout * m.eps_int for m in models])
    rounds, neom = ens.propagate(method, tnext, t, step)
    assert rounds > 0 and neom > 0
    for i, (m, (A, psi)) in enumerate(zip(models, starts)):
        # ensemble members start every Jacobi eigen-decomposition cold
        core = GpuCore(m, warm_start=False)
        core.set_state(A, psi, as_start=True)
        ts, ss, _, _, _ = core.propagate_interval(method, tnext, 0.0, m.tout * m.eps_int)
        assert abs(ts - t[i]) < 1e-12 and abs(ss - step[i]) < 1e-12 * max(1.0, ss)
        ref = core.observables(ts)
        got = ens.observables(i, t[i])
        assert abs(got["auto"] - ref["auto"]) < 1e-13
        assert np.abs(got["pop"] - ref["pop"]).max() < 1e-13
        assert abs(got["energy"] - ref["energy"]) < 1e-13


def test_generated_ragged_ensemble_runs():
    """Members drawn like the batched-ensemble workload (2-4 states, 4-10 modes,
    4-10 SPFs, 16-48 points; capped configuration count): the lockstep run
    keeps every member's norm."""
    from macaw_gb300.capi import Ensemble
    models = ensemble(count=6, max_conf=1 << 12)
    ens = Ensemble(models)
    for i, m in enumerate(models):
        A, psi = initial_wavefunction(m)
        ens.set_state(i, A, psi, as_start=True)
    t = np.zeros(len(models))
    step = np.array([m.tout * m.eps_int for m in models])
    ens.propagate(INT_RK45, 0.2 / AU2FS, t, step)
    for i in range(len(models)):
        ob = ens.observables(i, t[i])
        assert abs(ob["norm"] - 1.0) < 1e-6


def test_autotuned_split_precision_ensemble():
    """Split-FP32 members (compensated contractions) with the launch-shape
    autotuner: the chosen shape is the fastest timed one, every member's EOM
    agrees with its own split-precision context to 1e-10 relative (re-tiling
    only reorders compensated partial sums), and a lockstep RK45 interval of
    0.1 fs agrees with single-context runs within 10 eps_int (free-running step
    control)."""
    from macaw_gb300.capi import Ensemble, GpuCore
    models = _members()
    ens = Ensemble(models, precision=1)
    states = [random_state(m, seed=70 + i) for i, m in enumerate(models)]
    for i, (A, psi) in enumerate(states):
        ens.set_state(i, A, psi, as_start=True)
    tun = ens.autotune()
    assert tun["candidates"] >= 12
    assert 0.0 < tun["eom_ms"] <= tun["default_eom_ms"]
    got = ens.calc_derivs()
    for m, (A, psi), (dA, dpsi) in zip(models, states, got):
        rA, rpsi = GpuCore(m, precision=1).calc_derivs(A, psi)
        assert _rel(dA, rA) < 1e-10
        assert _rel(dpsi, rpsi) < 1e-10
    starts = [initial_wavefunction(m) for m in models]
    for i, (A, psi) in enumerate(starts):
        ens.set_state(i, A, psi, as_start=True)
    tnext = 0.1 / AU2FS
    t = np.zeros(len(models))
    step = np.array([m.tout * m.eps_int for m in models])
    ens.propagate(INT_RK45, tnext, t, step)
    for i, (m, (A, psi)) in enumerate(zip(models, starts)):
        core = GpuCore(m, precision=1)
        core.set_state(A, psi, as_start=True)
        ts, _, _, _, _ = core.propagate_interval(INT_RK45, tnext, 0.0, m.tout * m.eps_int)
        ref = core.observables(ts)
        ob = ens.observables(i, t[i])
        assert abs(ob["auto"] - ref["auto"]) < 10 * m.eps_int
        assert np.abs(ob["pop"] - ref["pop"]).max() < 10 * m.eps_int
