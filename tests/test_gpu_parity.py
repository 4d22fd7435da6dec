"""GPU parity: the CUDA path through the C-ABI against the CPU oracle.

Tolerances: single EOM evaluations and overlaps agree to 1e-11 relative (FP64
with a different but fixed summation order); propagated observables (C(t),
populations, norm, energy) agree to 1e-10 absolute, the parity bar of the
FP64 path.
"""
import numpy as np
import pytest

from macaw_gb300.model import initial_wavefunction, INT_RK45, INT_DOPRI, INT_CMF2
from oracle.mctdh import Oracle
from tests.helpers import small_lvc, small_qvc, random_state

pytestmark = pytest.mark.gpu

EOM_RTOL = 1e-11
OBS_ATOL = 1e-10


@pytest.fixture(scope="module")
def core_cls():
    from macaw_gb300.capi import GpuCore
    return GpuCore


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("builder,seed", [(lambda: small_lvc(), 1), (lambda: small_qvc(), 2),
                                          (lambda: small_qvc(nstates=2, ndof=6, grid=5, nspf=3), 3)])
def test_calc_derivs_random_state(core_cls, builder, seed):
    model = builder()
    A, psi = random_state(model, seed=seed)
    ref_dA, ref_dpsi = Oracle(model).calc_derivs(A, psi, 0.0)
    gpu = core_cls(model)
    dA, dpsi = gpu.calc_derivs(A, psi, 0.0)
    assert _rel(dA, ref_dA) < EOM_RTOL
    assert _rel(dpsi, ref_dpsi) < EOM_RTOL


def test_calc_derivs_initial_state(core_cls):
    """The single-configuration start: rho is rank one, so the regularised
    inverse (eps_rho = 1e-8) carries the weight of the virtual SPFs."""
    model = small_lvc()
    A, psi = initial_wavefunction(model)
    ref_dA, ref_dpsi = Oracle(model).calc_derivs(A, psi, 0.0)
    dA, dpsi = core_cls(model).calc_derivs(A, psi, 0.0)
    assert _rel(dA, ref_dA) < EOM_RTOL
    assert np.abs(dpsi - ref_dpsi).max() < 1e-9 * max(np.abs(ref_dpsi).max(), 1.0)


def test_norm_and_overlap(core_cls):
    model = small_qvc()
    A1, p1 = random_state(model, seed=4)
    A2, p2 = random_state(model, seed=5)
    o = Oracle(model)
    gpu = core_cls(model)
    assert abs(gpu.norm_wf(A1, p1) - o.norm_wf(A1, p1)) < 1e-13
    assert abs(gpu.wf_ovl(A1, p1, A2, p2) - o.wf_ovl(A1, p1, A2, p2)) < 1e-13


@pytest.mark.parametrize("method", [INT_RK45, INT_DOPRI])
def test_rkqs_step(core_cls, method):
    """An accepted step reproduces the oracle to rounding.  The next-step
    proposal depends on errmax ** -0.2, and errmax comes from DeltaPsi
    (gmctdh_objects.f90:222), sqrt|2(1 - Re<1|2>/sqrt(<1|1><2|2>))|, which for
    an accepted small step cancels down to a few ulps of O(1) overlaps: errmax
    is then rounding noise in any FP64 implementation, the reference included."""
    model = small_lvc()
    A, psi = random_state(model, seed=6, spread=1.0)
    o = Oracle(model)
    dA, dpsi = o.calc_derivs(A, psi, 0.0)
    h = 0.2
    rA, rp, rdA, rdp, rhdid, rhnext, ratt = o.rkqs(A, psi, dA, dpsi, 0.0, h, method)
    assert ratt == 1
    gA, gp, gdA, gdp, ghdid, ghnext = core_cls(model).rkqs(A, psi, dA, dpsi, 0.0, h, method)
    assert ghdid == rhdid == h
    # errmax is at the rounding floor here: only the bounds of the controller hold
    assert 0.1 * h <= ghnext <= 5.0 * h
    assert np.abs(gA - rA).max() < 1e-12
    assert np.abs(gp - rp).max() < 1e-12
    if method == INT_DOPRI:
        assert _rel(gdA, rdA) < EOM_RTOL


def test_rkqs_rejected_step(core_cls):
    """A rejected first trial shrinks dt by errmax ** -0.25; with errmax ~ 30 the
    DeltaPsi cancellation leaves ~1e-5 relative noise, so the retried step
    agrees with the oracle to that level."""
    model = small_lvc()
    A, psi = random_state(model, seed=6, spread=1.0)
    o = Oracle(model)
    dA, dpsi = o.calc_derivs(A, psi, 0.0)
    rA, rp, _, _, rhdid, _, ratt = o.rkqs(A, psi, dA, dpsi, 0.0, 2.0, INT_RK45)
    assert ratt > 1
    gA, gp, _, _, ghdid, _ = core_cls(model).rkqs(A, psi, dA, dpsi, 0.0, 2.0, INT_RK45)
    assert abs(ghdid - rhdid) <= 1e-4 * rhdid
    assert np.abs(gA - rA).max() < 1e-4 * np.abs(dA).max() * rhdid + 1e-12


def _replay(core, model, A0, psi0, steps, attempt):
    """Replay the oracle's accepted step lengths through the C-ABI and collect the
    observables at the output times, following propagate_wf (propagator.f90:110-146)."""
    A, psi = A0.copy(), psi0.copy()
    core.set_state(A0, psi0, as_start=True)
    t = model.tinit
    maxtime = model.tfinal + 0.1 * model.tout
    outs = [core.observables(t)]
    tnext = t + model.tout
    errs = []
    for (_, _, hdid, _, _) in steps:
        A, psi, err = attempt(A, psi, t, hdid)
        errs.append(err)
        t += hdid
        if t >= tnext - model.min_stepsize:
            if t < maxtime:
                core.set_state(A, psi, as_start=False)
                outs.append(core.observables(t))
            tnext = t + model.tout
    return outs, errs


def _compare(outs, ref, atol):
    assert len(outs) == len(ref)
    for g, r in zip(outs, ref):
        assert abs(g["t"] - r["t"]) < 1e-9
        assert abs(g["auto"] - r["auto"]) < atol, (g["t"], g["auto"], r["auto"])
        assert np.abs(g["pop"] - r["pop"]).max() < atol
        assert abs(g["norm"] - r["norm"]) < atol
        assert abs(g["energy"] - r["energy"]) < atol


def test_rk45_replay_observables(core_cls):
    """C(t), populations, norm and energy within 1e-10 on the oracle's step sequence."""
    model = small_lvc(tfinal_fs=2.0)
    A, psi = initial_wavefunction(model)
    ref, steps, _ = Oracle(model).propagate(A, psi, record_steps=True)
    gpu = core_cls(model)

    def attempt(A, psi, t, h):
        dA, dpsi = gpu.calc_derivs(A, psi, t)
        A, psi, _, _, err = gpu.rk_attempt(A, psi, dA, dpsi, t, h, INT_RK45)
        return A, psi, err

    outs, errs = _replay(gpu, model, A, psi, steps, attempt)
    assert max(errs) < 1.5
    _compare(outs, ref, OBS_ATOL)


def test_rk45_free_running(core_cls):
    """Free-running step control: step sequences differ by the rounding noise of
    DeltaPsi, so observables agree to the integrator tolerance, not to rounding."""
    model = small_lvc(tfinal_fs=2.0)
    A, psi = initial_wavefunction(model)
    ref, _, _ = Oracle(model).propagate(A, psi)
    outs = core_cls(model).propagate(A, psi)
    _compare(outs, ref, 10 * model.eps_int)


@pytest.mark.parametrize("int_type_psi", [1, 2])
def test_cmf2_step(core_cls, int_type_psi):
    """One CMF2 step; the SPFs integrated with Cash-Karp (1) or Dormand-Prince (2)."""
    model = small_qvc()
    model.int_type_psi = int_type_psi
    A, psi = initial_wavefunction(model)
    o = Oracle(model)
    rA, rp, rh, rn, tries = o.cmf2(A, psi, 0.0, 1.0)
    assert tries == 1
    gA, gp, gh, gn = core_cls(model).cmf2(A, psi, 0.0, 1.0)
    assert gh == rh == 1.0
    assert abs(gn - rn) <= 1e-4 * rn   # hnext uses err_psi = DeltaPsi (rounding-floor noise)
    assert np.abs(gA - rA).max() < 1e-10
    assert np.abs(gp - rp).max() < 1e-10


def test_cmf2_step_with_rejected_attempts(core_cls):
    """A trial step far above the tolerated one: the step control rejects it and
    retries from the same state, where the device restores the step-start
    operators saved after their evaluation instead of evaluating them again;
    the accepted step equals the oracle's (cmf2_base.f90:176-201)."""
    model = small_qvc()
    A, psi = initial_wavefunction(model)
    o = Oracle(model)
    rA, rp, rh, rn, tries = o.cmf2(A, psi, 0.0, 40.0)
    assert tries >= 2
    gA, gp, gh, gn = core_cls(model).cmf2(A, psi, 0.0, 40.0)
    assert abs(gh - rh) <= 1e-6 * rh
    assert np.abs(gA - rA).max() < 1e-10
    assert np.abs(gp - rp).max() < 1e-10


def test_cmf2_replay_observables(core_cls):
    model = small_qvc(tfinal_fs=1.0)
    A, psi = initial_wavefunction(model)
    ref, steps, _ = Oracle(model).propagate(A, psi, record_steps=True)
    gpu = core_cls(model)
    outs, errs = _replay(gpu, model, A, psi, steps, lambda A, psi, t, h: gpu.cmf2_attempt(A, psi, t, h))
    assert max(errs) <= 1.0 + 1e-6
    _compare(outs, ref, OBS_ATOL)


def test_cmf2_free_running(core_cls):
    model = small_qvc(tfinal_fs=1.0)
    A, psi = initial_wavefunction(model)
    ref, _, _ = Oracle(model).propagate(A, psi)
    outs = core_cls(model).propagate(A, psi)
    _compare(outs, ref, 10 * model.eps_int)


@pytest.mark.parametrize("prec,tol", [(1, 1e-6), (2, 1e-10), (3, 1e-5), (4, 1e-6), (5, 1e-10), (6, 1e-5)])
def test_split_precision_eom(core_cls, prec, tol):
    """Split-FP32 mode products (1: FP32 sums, 2: compensated FP32 sums; mean
    fields compensated) against the FP64 oracle; 3 and 6 sum the contractions
    (all of them, or the mean fields') in FP32; 4 and 5 differ from 1 and 2 only
    in the Lanczos H_B products, which the EOM does not use."""
    for builder, seed in ((lambda: small_lvc(), 21), (lambda: small_qvc(), 22)):
        model = builder()
        A, psi = random_state(model, seed=seed)
        ref_dA, ref_dpsi = Oracle(model).calc_derivs(A, psi, 0.0)
        dA, dpsi = core_cls(model, precision=prec).calc_derivs(A, psi, 0.0)
        assert _rel(dA, ref_dA) < tol
        assert _rel(dpsi, ref_dpsi) < tol


@pytest.mark.parametrize("prec", [1, 5])
def test_split_precision_cmf2_replay(core_cls, prec):
    """The split-FP32 CMF2 path on the oracle's step sequence stays within 1e-7 of
    C(t) (FP32 Lanczos products in both modes)."""
    model = small_qvc(tfinal_fs=1.0)
    A, psi = initial_wavefunction(model)
    ref, steps, _ = Oracle(model).propagate(A, psi, record_steps=True)
    gpu = core_cls(model, precision=prec)
    outs, _ = _replay(gpu, model, A, psi, steps, lambda A, psi, t, h: gpu.cmf2_attempt(A, psi, t, h))
    _compare(outs, ref, 1e-7)


def test_gpu_stays_usable_after_error(core_cls):
    """A rejected call (bad method) returns a status and the context keeps working."""
    from macaw_gb300.capi import MctdhError
    model = small_lvc()
    A, psi = initial_wavefunction(model)
    gpu = core_cls(model)
    with pytest.raises(MctdhError):
        gpu.rkqs(A, psi, A * 0, psi * 0, 0.0, 1.0, method=7)
    dA, _ = gpu.calc_derivs(A, psi)
    assert np.all(np.isfinite(dA))


@pytest.mark.parametrize("order,par1", [(4, 0), (3, 1)])
def test_adams_free_running(core_cls, order, par1):
    """Adams PECE ('abm<order><par1>', integrator.f90:244-380) after the Cash-Karp
    bootstrap of propagate_wf (propagator.f90:156-181), free running against the
    oracle's restatement: the step control sees DeltaPsi's rounding noise, so the
    bound is the integrator tolerance."""
    from macaw_gb300.model import INT_ABM
    model = small_lvc(tfinal_fs=1.0)
    model.int_type = INT_ABM
    model.int_order = order
    model.int_par1 = par1
    A, psi = initial_wavefunction(model)
    ref, _, _ = Oracle(model).propagate(A, psi)
    outs = core_cls(model).propagate(A, psi)
    _compare(outs, ref, 10 * model.eps_int)


def test_bulirsch_stoer_free_running(core_cls):
    """Bulirsch-Stoer ('bs', integrator.f90:384-608; propagate_wf :210-248) free
    running against the oracle's restatement, bounded by the integrator tolerance."""
    from macaw_gb300.model import INT_BS
    model = small_lvc(tfinal_fs=1.0)
    model.int_type = INT_BS
    A, psi = initial_wavefunction(model)
    ref, _, _ = Oracle(model).propagate(A, psi)
    outs = core_cls(model).propagate(A, psi)
    _compare(outs, ref, 10 * model.eps_int)
