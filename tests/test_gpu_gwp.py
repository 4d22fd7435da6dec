"""GPU parity of the G-MCTDH (Gaussian SPF) path against the oracle.

The device solves the regularised parameter equations by QR of [C; eps I]
instead of the reference's eigen-decomposition of C; both give the minimiser of
|C x - Y|^2 + eps^2 |x|^2, and on these models (C well conditioned) they agree
to 1e-14.  EOM evaluations agree to 1e-10 relative; propagated observables on
the oracle's step sequence to 1e-10 absolute.
"""
import numpy as np
import pytest

from macaw_gb300.model import initial_wavefunction, INT_RK45, INT_CMF2
from oracle.mctdh import Oracle
from tests.helpers import small_gmctdh, random_state
from tests.test_gpu_parity import _replay, _compare, _rel

pytestmark = pytest.mark.gpu

GWP_RTOL = 1e-10


@pytest.fixture(scope="module")
def core_cls():
    from macaw_gb300.capi import GpuCore
    return GpuCore


def _check_eom(core_cls, model, A, psi):
    o = Oracle(model)
    ref_dA, ref_dpsi = o.calc_derivs(A, psi, 0.0)
    dA, dpsi = core_cls(model).calc_derivs(A, psi, 0.0)
    assert _rel(dA, ref_dA) < GWP_RTOL
    assert _rel(dpsi, ref_dpsi) < GWP_RTOL
    for m in model.modes_gwp:
        for s in range(model.nstates):
            o_ = int(model.ipsispf[m, s])
            n = int(model.nspf[m, s]) * len(model.mode_dofs[m])
            blk, ref = dpsi[o_:o_ + n], ref_dpsi[o_:o_ + n]
            assert np.linalg.norm(blk - ref) <= GWP_RTOL * max(np.linalg.norm(ref), 1e-12)


@pytest.mark.parametrize("seed", [3, 4])
def test_gwp_eom_random_state(core_cls, seed):
    model = small_gmctdh()
    A, psi = random_state(model, seed=seed)
    _check_eom(core_cls, model, A, psi)


def test_gwp_eom_initial_state(core_cls):
    """Single-configuration start on state 2: rho of state 1 and with it C are
    zero, so the Tikhonov solution for that state's Gaussians is zero."""
    model = small_gmctdh()
    A, psi = initial_wavefunction(model)
    _check_eom(core_cls, model, A, psi)


def test_gwp_norm_and_overlap(core_cls):
    model = small_gmctdh()
    A1, p1 = random_state(model, seed=5)
    A2, p2 = random_state(model, seed=6)
    o = Oracle(model)
    gpu = core_cls(model)
    assert abs(gpu.norm_wf(A1, p1) - o.norm_wf(A1, p1)) < 1e-13
    assert abs(gpu.wf_ovl(A1, p1, A2, p2) - o.wf_ovl(A1, p1, A2, p2)) < 1e-13


def test_gwp_rk45_replay_observables(core_cls):
    """C(t), populations, norm and energy of the RK propagation on the oracle's
    step sequence, within 1e-10."""
    model = small_gmctdh(tfinal_fs=1.0)
    A, psi = initial_wavefunction(model)
    ref, steps, _ = Oracle(model).propagate(A, psi, record_steps=True)
    gpu = core_cls(model)

    def attempt(A, psi, t, h):
        dA, dpsi = gpu.calc_derivs(A, psi, t)
        A, psi, _, _, err = gpu.rk_attempt(A, psi, dA, dpsi, t, h, INT_RK45)
        return A, psi, err

    outs, errs = _replay(gpu, model, A, psi, steps, attempt)
    assert max(errs) < 1.5
    _compare(outs, ref, 1e-10)


def test_gwp_rk45_free_running(core_cls):
    model = small_gmctdh(tfinal_fs=1.0)
    A, psi = initial_wavefunction(model)
    ref, _, _ = Oracle(model).propagate(A, psi)
    outs = core_cls(model).propagate(A, psi)
    _compare(outs, ref, 10 * model.eps_int)


def _cmf2_model(tfinal_fs=1.0):
    model = small_gmctdh(tfinal_fs=tfinal_fs)
    model.int_type = INT_CMF2
    return model


@pytest.mark.parametrize("int_type_psi", [1, 2])
def test_gwp_cmf2_step(core_cls, int_type_psi):
    """One CMF2 step of the Gaussian model (cmf2_base.f90:47-206): D = S^-1/2 by
    Cholesky, B = D^H S A, Lanczos with D^H h D, the Gaussian parameters and D
    integrated with Cash-Karp (1) or Dormand-Prince (2), A = D B at the end."""
    model = _cmf2_model()
    model.int_type_psi = int_type_psi
    A, psi = random_state(model, seed=7, gwp_shift=0.05)
    rA, rp, rh, rn, tries = Oracle(model).cmf2(A, psi, 0.0, 0.2)
    gA, gp, gh, gn = core_cls(model).cmf2(A, psi, 0.0, 0.2)
    assert gh == rh
    assert abs(gn - rn) <= 1e-4 * rn   # hnext uses err_psi = DeltaPsi (rounding-floor noise)
    assert np.abs(gA - rA).max() < 1e-10
    assert np.abs(gp - rp).max() < 1e-10


def test_gwp_cmf2_propagation(core_cls):
    """CMF2 over 0.5 fs from the single-configuration start: on the oracle's step
    sequence within 1e-10, free running within 10 eps_int."""
    model = _cmf2_model(tfinal_fs=0.5)
    A, psi = initial_wavefunction(model)
    ref, steps, _ = Oracle(model).propagate(A, psi, record_steps=True)
    gpu = core_cls(model)
    outs, errs = _replay(gpu, model, A, psi, steps, lambda A, psi, t, h: gpu.cmf2_attempt(A, psi, t, h))
    # err_psi = sqrt(2 (1 - Re<1|2>/..)) with 1 - Re<1|2> ~ eps_int^2: FP64 rounding
    # of the overlaps (1e-16) moves the accepted steps' error by up to ~1e-4 relative
    assert max(errs) <= 1.0 + 1e-3
    _compare(outs, ref, 1e-10)
    outs = core_cls(model).propagate(A, psi)
    _compare(outs, ref, 10 * model.eps_int)
