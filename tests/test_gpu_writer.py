"""GPU parity of the writer quantities computed on the device for the resident
state (output.f90:88-140 natural populations, gross Gaussian populations and
population errors; :276-300 density matrices; :449-500 expectation values)
against the oracle.  FP64 throughout: 1e-12 absolute on O(1) quantities."""
import numpy as np
import pytest

from macaw_gb300.model import initial_wavefunction
from oracle.mctdh import Oracle, herm_from_upper
from tests.helpers import small_lvc, small_qvc, small_gmctdh, random_state, with_expect

pytestmark = pytest.mark.gpu

TOL = 1e-12


@pytest.fixture(scope="module")
def core_cls():
    from macaw_gb300.capi import GpuCore
    return GpuCore


def _model(name):
    if name == "lvc":
        return with_expect(small_lvc())
    if name == "qvc":
        return with_expect(small_qvc())
    m = small_gmctdh()
    initial_wavefunction(m)
    return with_expect(m)


@pytest.mark.parametrize("name,seed", [("lvc", 31), ("qvc", 32), ("gmctdh", 33)])
def test_writer_quantities(core_cls, name, seed):
    model = _model(name)
    A, psi = random_state(model, seed=seed)
    o = Oracle(model)
    core = core_cls(model)
    core.set_state(A, psi, as_start=True)
    ev = core.expect()
    ref = o.expectation(A, psi)
    assert np.abs(ev - ref).max() < TOL * max(1.0, np.abs(ref).max())
    nat, ggp, perr = core.natpop()
    rnat, rggp, rperr = o.natpop(A, psi)
    for (mode, s), w in rnat.items():
        assert np.abs(nat[:len(w), mode, s] - w).max() < TOL
    for i, mode in enumerate(model.modes_gwp):
        for s in range(model.nstates):
            n = int(model.nspf[mode, s])
            assert np.abs(ggp[:n, i, s] - rggp[(mode, s)]).max() < TOL
            assert np.abs(perr[:n, i, s] - rperr[(mode, s)]).max() < TOL
    o._prepare(A, psi)
    for mode in range(model.nmodes):
        for s in range(model.nstates):
            r = herm_from_upper(np.triu(o.rho[(mode, s)]))
            assert np.abs(core.densmat(mode, s) - r).max() < TOL


def test_expectation_operators_leave_the_eom_unchanged(core_cls):
    """Operators only expectation operators use stay out of the EOM (their mean
    fields are zero in the reference): the derivatives still match the oracle."""
    model = _model("gmctdh")
    A, psi = random_state(model, seed=34)
    ref_dA, ref_dpsi = Oracle(model).calc_derivs(A, psi, 0.0)
    dA, dpsi = core_cls(model).calc_derivs(A, psi, 0.0)
    assert np.linalg.norm(dA - ref_dA) < 1e-10 * np.linalg.norm(ref_dA)
    assert np.linalg.norm(dpsi - ref_dpsi) < 1e-10 * np.linalg.norm(ref_dpsi)


@pytest.mark.parametrize("name,seed", [("qvc", 35), ("gmctdh", 36)])
def test_density(core_cls, name, seed):
    """Calc_Density along every DOF: grid DOFs (inner and outer DOF of two-DOF
    modes) with the basis populations, and Gaussian DOFs."""
    model = _model(name)
    A, psi = random_state(model, seed=seed)
    o = Oracle(model)
    core = core_cls(model)
    core.set_state(A, psi, as_start=True)
    for dof in range(model.ndof):
        dens, pop = core.density(dof)
        if model.dvr_type[dof] == "gwp":
            rd, _ = o.density(A, psi, dof, xrange=model.dvrpar[dof])
        else:
            rd, rp = o.density(A, psi, dof, trafo=model.trafo[dof])
            assert np.abs(pop - rp).max() < TOL
        assert np.abs(dens - rd).max() < TOL
