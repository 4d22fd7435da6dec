"""GPU parity at the full sizes of the benchmark configurations.

The small-model tests (test_gpu_parity.py, test_gpu_gwp.py) pin every code path;
these repeat the decisive comparisons at the sizes the throughput numbers are
quoted on, where the batched launches split into many blocks, the contractions
reduce over tens of thousands of fibres and the Gaussian parameter system is
384 x 384:

* lvc5 (2 states, 5 HO modes of 24-40 points, 6 SPFs): the oracle's adaptive
  Cash-Karp step sequence over 5 fs (tolerance 1e-8, output every 0.5 fs)
  replayed through the C-ABI; C(t), populations, norm and energy within 1e-10
  (propagate_wf, propagator.f90:110-146).
* qvc12 (3 states, 6 two-DOF modes of 20x20 grids, 8 SPFs, 262,144
  coefficients per state): three CMF2 steps of the benchmark's step length from
  the state the benchmark starts from (1 fs of FP64 CMF2), against the oracle's
  cmf2 (cmf2_base.f90:47-206) on the same steps; A and the observables within
  1e-10, the SPF values within 1e-9 (see the test).
* gmctdh16 (2 states, 4 HO modes of 32 points with 6 SPFs plus one 12-DOF mode
  of 32 Gaussians per state): one EOM evaluation on a displaced random state
  (1e-10 relative) and one Cash-Karp attempt from it (1e-10 absolute).
"""
import numpy as np
import pytest

from macaw_gb300.generate import gmctdh16, lvc5, qvc12
from macaw_gb300.model import AU2FS, INT_CMF2, INT_RK45, initial_wavefunction
from oracle.mctdh import Oracle
from tests.helpers import random_state
from tests.test_gpu_parity import _compare, _rel, _replay

pytestmark = pytest.mark.gpu

OBS_ATOL = 1e-10
EOM_RTOL = 1e-10


@pytest.fixture(scope="module")
def core_cls():
    from macaw_gb300.capi import GpuCore
    return GpuCore


def test_lvc5_full_rk45_replay(core_cls):
    model = lvc5(tfinal_fs=5.0)
    assert model.naconftot == 2 * 6 ** 5
    A, psi = initial_wavefunction(model)
    ref, steps, _ = Oracle(model).propagate(A, psi, record_steps=True)
    gpu = core_cls(model)

    def attempt(A, psi, t, h):
        dA, dpsi = gpu.calc_derivs(A, psi, t)
        A, psi, _, _, err = gpu.rk_attempt(A, psi, dA, dpsi, t, h, INT_RK45)
        return A, psi, err

    outs, errs = _replay(gpu, model, A, psi, steps, attempt)
    assert len(outs) == 11 and len(steps) > 50
    # at eps_int = 1e-8 the error norm sqrt|2(1 - Re<1|2>/...)| / eps_int of an
    # accepted step is rounding noise of order one (a few ulps under the root),
    # in the oracle as on the device: only its finiteness is checked
    assert np.all(np.isfinite(errs))
    _compare(outs, ref, OBS_ATOL)


def test_qvc12_full_cmf2_steps(core_cls):
    """Three CMF2 steps at the benchmark's operating point.  The start state is
    the FP64 device propagation to 1 fs (as in the benchmark); from it the oracle
    and the device take the same three steps of the device's own proposed length."""
    model = qvc12(eps_int=1e-5, eps_lanczos=1e-8, eps_spf=1e-7)
    A0, psi0 = initial_wavefunction(model)
    gpu = core_cls(model)
    gpu.set_state(A0, psi0, as_start=True)
    t, h, _, _, _ = gpu.propagate_interval(INT_CMF2, 1.0 / AU2FS, 0.0, model.tout * model.eps_int)
    assert 0.005 < h * AU2FS < 0.1
    A1, psi1 = gpu.get_state()
    o = Oracle(model)
    rA, rp = A1.copy(), psi1.copy()
    gA, gp = A1.copy(), psi1.copy()
    for k in range(3):
        rA, rp, rerr = o.cmf2_fixed(rA, rp, t + k * h, h)
        gA, gp, gerr = gpu.cmf2_attempt(gA, gp, t + k * h, h)
        # the step error is max(err_A, err_psi) / eps_int; err_psi is DeltaPsi,
        # at its rounding floor for such steps, so only its scale is compared
        assert abs(gerr - rerr) <= 0.02 * max(rerr, 1.0)
    assert np.abs(gA - rA).max() < OBS_ATOL
    # The SPF derivative applies the regularised inverse of rho, which scales the
    # weakly occupied directions by up to 1 / eps_rho = 1e8: ulp-level differences
    # between two FP64 eigen-decompositions (Jacobi on the device, LAPACK in the
    # oracle) reach ~1e-10 in the SPF values there after three steps.  Those
    # directions carry almost no weight, and the observables below hold the
    # 1e-10 bar.
    assert np.abs(gp - rp).max() < 10 * OBS_ATOL
    gpu.set_state(gA, gp, as_start=False)
    g = gpu.observables(t + 3 * h)
    r = o.observables(rA, rp, A0, psi0, t + 3 * h)
    _compare([g], [r], OBS_ATOL)


def test_gmctdh16_full_eom_and_rk_attempt(core_cls):
    model = gmctdh16()
    assert model.naconftot == 2 * 6 ** 4 * 32 and model.nspf[4, 0] == 32
    A, psi = random_state(model, seed=31, gwp_shift=0.05)
    o = Oracle(model)
    ref_dA, ref_dpsi = o.calc_derivs(A, psi, 0.0)
    gpu = core_cls(model)
    dA, dpsi = gpu.calc_derivs(A, psi, 0.0)
    assert _rel(dA, ref_dA) < EOM_RTOL
    assert _rel(dpsi, ref_dpsi) < EOM_RTOL
    dt = 0.01 / AU2FS
    rA, rp, _, _, rerr = o.rk_fixed(A, psi, ref_dA, ref_dpsi, 0.0, dt, INT_RK45)
    gA, gp, _, _, gerr = gpu.rk_attempt(A, psi, ref_dA, ref_dpsi, 0.0, dt, INT_RK45)
    assert np.abs(gA - rA).max() < OBS_ATOL
    assert np.abs(gp - rp).max() < OBS_ATOL
    assert abs(gerr - rerr) <= 0.02 * max(rerr, 1.0)
