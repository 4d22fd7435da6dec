"""GPU parity on the reference's own example inputs and on the parametrised
operators and the Legendre DVR.

* The two butadiene inputs the reference ships (5 DOFs in 3 modes: a 56 x 25
  sine x HO grid mode with spline-interpolated potentials, a one-DOF and a
  two-DOF Gaussian mode, multi- and single-set SPFs), stored as fixtures by
  tests/golden/make_butadiene.py.  Dormand-Prince (eps_int 1e-6) and CMF2
  (eps_int 1e-3) runs of 2 fs are replayed on the oracle's step sequence through
  the C-ABI; C(t), populations, norm and energy agree within 1e-10.
* A synthetic model with every parametrised operator (gau, interp, square,
  hermite, sin and cos powers, the eig_proj projector) and two Legendre DOFs
  (M = 0 and M = 1, with L0^2 and sin^-2): one EOM evaluation at 1e-10 and a
  replayed Cash-Karp run.
"""
import os
import pickle

import numpy as np
import pytest

from macaw_gb300.model import AU2FS, INT_CMF2, INT_DOPRI, INT_RK45, initial_wavefunction, model_from_fields
from oracle.mctdh import Oracle
from tests.helpers import parametrised_model, random_state
from tests.test_gpu_parity import _compare, _rel, _replay

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
OBS_ATOL = 1e-10
EOM_RTOL = 1e-10


@pytest.fixture(scope="module")
def core_cls():
    from macaw_gb300.capi import GpuCore
    return GpuCore


def butadiene(name, tfinal_fs=2.0):
    with open(os.path.join(GOLDEN, name + ".pkl"), "rb") as fh:
        model = model_from_fields(pickle.load(fh))
    model.tfinal = tfinal_fs / AU2FS
    return model


def test_butadiene_eom(core_cls):
    model = butadiene("butadiene_dopri")
    for seed in (41, 42):
        A, psi = random_state(model, seed=seed, gwp_shift=0.05)
        ref_dA, ref_dpsi = Oracle(model).calc_derivs(A, psi, 0.0)
        dA, dpsi = core_cls(model).calc_derivs(A, psi, 0.0)
        assert _rel(dA, ref_dA) < EOM_RTOL
        assert _rel(dpsi, ref_dpsi) < EOM_RTOL


def test_butadiene_dopri_replay(core_cls):
    """Examples/Butadiene_5modes (integration = DOPRI): the derivative of the
    last stage is carried into the next step (FSAL), as the reference's rkqs
    does (integrator.f90:82-85)."""
    model = butadiene("butadiene_dopri")
    assert model.int_type == INT_DOPRI
    A, psi = initial_wavefunction(model)
    ref, steps, _ = Oracle(model).propagate(A, psi, record_steps=True)
    gpu = core_cls(model)
    carry = {}

    def attempt(A, psi, t, h):
        if not carry:
            carry["d"] = gpu.calc_derivs(A, psi, t)
        dA, dpsi = carry["d"]
        A, psi, dA, dpsi, err = gpu.rk_attempt(A, psi, dA, dpsi, t, h, INT_DOPRI)
        carry["d"] = (dA, dpsi)
        return A, psi, err

    outs, errs = _replay(gpu, model, A, psi, steps, attempt)
    assert len(outs) == 5 and np.all(np.isfinite(errs))
    _compare(outs, ref, OBS_ATOL)


def test_butadiene_cmf2_replay(core_cls):
    """Examples/Butadiene_5modes_CMF (integration = CMF2, Lanczos and rk45 at
    8e-7): Gaussian modes propagate through B = D^H S A."""
    model = butadiene("butadiene_cmf2")
    assert model.int_type == INT_CMF2
    A, psi = initial_wavefunction(model)
    ref, steps, _ = Oracle(model).propagate(A, psi, record_steps=True)
    gpu = core_cls(model)
    outs, errs = _replay(gpu, model, A, psi, steps, lambda A, psi, t, h: gpu.cmf2_attempt(A, psi, t, h))
    assert len(outs) == 5
    _compare(outs, ref, OBS_ATOL)


def test_parametrised_and_legendre_eom(core_cls):
    model = parametrised_model()
    for seed in (51, 52):
        A, psi = random_state(model, seed=seed)
        ref_dA, ref_dpsi = Oracle(model).calc_derivs(A, psi, 0.0)
        dA, dpsi = core_cls(model).calc_derivs(A, psi, 0.0)
        assert _rel(dA, ref_dA) < EOM_RTOL
        assert _rel(dpsi, ref_dpsi) < EOM_RTOL


def test_parametrised_and_legendre_rk45_replay(core_cls):
    model = parametrised_model()
    A, psi = initial_wavefunction(model)
    ref, steps, _ = Oracle(model).propagate(A, psi, record_steps=True)
    gpu = core_cls(model)

    def attempt(A, psi, t, h):
        dA, dpsi = gpu.calc_derivs(A, psi, t)
        A, psi, _, _, err = gpu.rk_attempt(A, psi, dA, dpsi, t, h, INT_RK45)
        return A, psi, err

    outs, _ = _replay(gpu, model, A, psi, steps, attempt)
    _compare(outs, ref, OBS_ATOL)
