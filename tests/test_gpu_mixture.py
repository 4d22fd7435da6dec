"""GPU parity of statistical mixtures and dissipation: the CUDA path through the
C-ABI against the oracle (gmctdh_objects.f90:481-1141, derivatives.f90:70-83,
238-242, DeltaPsi :206-248, WriteOutput output.f90:44-60, 143-149).

Tolerances as for a single packet: one EOM evaluation agrees to 1e-11 relative in
FP64 (1e-6 / 1e-10 in the split modes), one fixed RK attempt to 1e-11, and a
free-running propagation to 10 eps_int in the observables (step sequences differ
by the rounding noise of DeltaPsi).
"""
import numpy as np
import pytest

from macaw_gb300.model import initial_wavefunction, AU2FS, INT_RK45, INT_DOPRI, INT_CMF2
from oracle.mctdh import Oracle
from tests.helpers import small_lvc, with_mixture, random_mixture

pytestmark = pytest.mark.gpu

EOM_RTOL = 1e-11


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _model(P=3, which="both", **kw):
    m = with_mixture(small_lvc(nspf=3, grid=(8, 7, 6, 6, 7), **kw), npackets=P, diss=(which != "none"))
    if which in ("type1", "type2"):
        m.dissipation = [d for d in m.dissipation if d[0] == (1 if which == "type1" else 2)]
        m.finalize()
    return m


@pytest.fixture(scope="module")
def core_cls():
    from macaw_gb300.capi import GpuCore
    return GpuCore


@pytest.mark.parametrize("P,which", [(3, "both"), (3, "type1"), (3, "type2"), (1, "both"), (2, "none"),
                                     (5, "both")])
def test_mixture_derivs(core_cls, P, which):
    model = _model(P, which)
    A, psi = random_mixture(model, seed=P + 7)
    rA, rp = Oracle(model).calc_derivs(A, psi, 0.3)
    dA, dpsi = core_cls(model).calc_derivs(A, psi, 0.3)
    assert _rel(dA, rA) < EOM_RTOL
    assert _rel(dpsi, rp) < EOM_RTOL


def test_mixture_derivs_nonorthonormal_spfs(core_cls):
    """Intermediate states of a step have non-orthonormal SPFs: the packet
    populations WPpop are norm_wf values with the SPF overlaps (derivatives.f90:74)."""
    model = _model(3, "both")
    model.eps_pop = 1e-3
    model.finalize()
    A, psi = initial_wavefunction(model)
    orc = Oracle(model)
    dA, dpsi = orc.calc_derivs(A, psi, 0.0)
    A2, p2 = A + 0.04 * dA, psi + 0.04 * dpsi
    rA, rp = orc.calc_derivs(A2, p2, 0.0)
    gA, gp = core_cls(model).calc_derivs(A2, p2, 0.0)
    assert _rel(gA, rA) < EOM_RTOL
    assert _rel(gp, rp) < EOM_RTOL


@pytest.mark.parametrize("prec,tol", [(1, 1e-6), (2, 1e-10)])
def test_mixture_split_precision(core_cls, prec, tol):
    model = _model(3, "both")
    A, psi = random_mixture(model, seed=11)
    rA, rp = Oracle(model).calc_derivs(A, psi, 0.0)
    dA, dpsi = core_cls(model, precision=prec).calc_derivs(A, psi, 0.0)
    assert _rel(dA, rA) < tol
    assert _rel(dpsi, rp) < tol


@pytest.mark.parametrize("method", [INT_RK45, INT_DOPRI])
def test_mixture_rk_attempt(core_cls, method):
    """One fixed attempt with the packet DeltaPsi error."""
    model = _model(3, "both")
    A, psi = initial_wavefunction(model)
    orc = Oracle(model)
    dA, dpsi = orc.calc_derivs(A, psi, 0.0)
    h = 2.0
    rA, rp, rdA, rdp, rerr = orc.rk_fixed(A, psi, dA, dpsi, 0.0, h, method)
    gA, gp, _, _, gerr = core_cls(model).rk_attempt(A, psi, dA, dpsi, 0.0, h, method)
    assert _rel(gA, rA) < EOM_RTOL
    assert _rel(gp, rp) < EOM_RTOL
    assert abs(gerr - rerr) < 1e-6 * max(rerr, 1.0)


def test_mixture_propagation(core_cls):
    """Free-running RK45 of a mixture with both dissipation types: observables,
    packet populations and entropy against the oracle; the total population stays 1."""
    model = _model(3, "both", tfinal_fs=0.5, eps_int=1e-7)
    model.tout = 0.25 / AU2FS
    model.eps_pop = 1e-3
    model.finalize()
    A, psi = initial_wavefunction(model)
    orc = Oracle(model)
    ref, _, _ = orc.propagate(A, psi)
    gpu = core_cls(model)
    outs = gpu.propagate(A, psi)
    assert len(outs) == len(ref)
    for g, r in zip(outs, ref):
        assert abs(g["auto"] - r["auto"]) < 10 * model.eps_int
        assert np.abs(g["pop"] - r["pop"]).max() < 10 * model.eps_int
        assert abs(g["norm"] - 1.0) < 1e-6
        assert abs(g["energy"] - r["energy"]) < 10 * model.eps_int
    assert gpu.device_bytes() > 0
    Af, pf = gpu.get_state()
    w, ent = gpu.packets()
    ro = orc.observables(Af, pf, A, psi, model.tfinal)
    assert np.abs(w - ro["wppop"]).max() < 1e-12
    assert abs(ent - ro["entropy"]) < 1e-12


def test_cmf2_rejects_mixtures(core_cls):
    from macaw_gb300.capi import MctdhError
    model = _model(2, "none")
    A, psi = initial_wavefunction(model)
    gpu = core_cls(model)
    with pytest.raises(MctdhError) as e:
        gpu.propagate(A, psi, tfinal=model.tout, int_type=INT_CMF2)
    assert e.value.code == -1
    # the context stays usable
    dA, _ = gpu.calc_derivs(A, psi, 0.0)
    assert np.isfinite(dA).all()


def _free_running(core_cls, model, atol_scale=10.0):
    A, psi = initial_wavefunction(model)
    ref, _, _ = Oracle(model).propagate(A, psi)
    outs = core_cls(model).propagate(A, psi)
    assert len(outs) == len(ref)
    for g, r in zip(outs, ref):
        assert abs(g["auto"] - r["auto"]) < atol_scale * model.eps_int
        assert np.abs(g["pop"] - r["pop"]).max() < atol_scale * model.eps_int
        assert abs(g["energy"] - r["energy"]) < atol_scale * model.eps_int
    return outs


@pytest.mark.parametrize("integrator", ["abm40", "bs"])
def test_mixture_adams_and_bulirsch_stoer(core_cls, integrator):
    """Adams PECE and Bulirsch-Stoer on a dissipative mixture: both error norms are
    the packet DeltaPsi (integrator.f90:360-371, 540-548)."""
    from macaw_gb300.model import INT_ABM, INT_BS
    model = _model(3, "both", tfinal_fs=0.5, eps_int=1e-7)
    model.tout = 0.25 / AU2FS
    model.eps_pop = 1e-3
    if integrator == "bs":
        model.int_type = INT_BS
    else:
        model.int_type, model.int_order, model.int_par1 = INT_ABM, 4, 0
    model.finalize()
    _free_running(core_cls, model)


def test_mixture_relaxation_and_packets_block(core_cls):
    """Relaxation (der_factor = -1) of a dissipative mixture started from an explicit
    'packets' block (init_calc.f90:527-540): the dissipative terms carry der_factor
    exactly as the reference's (gmctdh_objects.f90:805)."""
    model = _model(2, "both", tfinal_fs=0.5, eps_int=1e-7)
    model.tout = 0.25 / AU2FS
    model.relaxation = True
    model.init_packets = [(1, (0, 0, 0, 0, 0), 0.8 + 0.0j), (0, (1, 0, 0, 0, 0), 0.6j)]
    model.finalize()
    _free_running(core_cls, model)


def _gmodel(P=3, **kw):
    from tests.helpers import small_gmctdh
    return with_mixture(small_gmctdh(**kw), npackets=P, eps_pop=1e-3)


def test_gaussian_mixture_derivs(core_cls):
    """A dissipative mixture over grid modes and a Gaussian mode: S^-1 and tau act on
    every packet (derivatives.f90:177-235), WPpop carries the Gaussian overlaps."""
    model = _gmodel(3)
    A, psi = initial_wavefunction(model)
    orc = Oracle(model)
    gpu = core_cls(model)
    for scale in (0.0, 0.04):
        if scale:
            dA, dpsi = orc.calc_derivs(A, psi, 0.0)
            A2, p2 = A + scale * dA, psi + scale * dpsi
        else:
            A2, p2 = A, psi
        rA, rp = orc.calc_derivs(A2, p2, 0.0)
        gA, gp = gpu.calc_derivs(A2, p2, 0.0)
        assert _rel(gA, rA) < 1e-10
        assert _rel(gp, rp) < 1e-10


def test_gaussian_mixture_propagation(core_cls):
    model = _gmodel(3, tfinal_fs=0.5, eps_int=1e-6)
    model.tout = 0.25 / AU2FS
    model.finalize()
    _free_running(core_cls, model)


def test_mixture_setup_errors(core_cls):
    """Bad mixture set-up fields are refused at mctdh_create with a status, and the
    device stays usable: a term kind outside 0..2 (-7), a type-1 term without its
    operator (-7), more than 4 type-1 operators (-1), more than 16 packets (-1); a
    type-1 term between two states with equal SPF counts is admitted."""
    import ctypes as C
    from macaw_gb300.capi import build_setup, load_library
    lib = load_library()
    model = _model(2, "both")

    def create(mutate):
        s, keep = build_setup(model, 0)
        keep.append(mutate(s))
        h = C.c_void_p()
        rc = lib.mctdh_create(C.byref(s), C.byref(h))
        if rc == 0:
            lib.mctdh_destroy(h)
        return rc

    def kinds(s, values):
        arr = np.array(values, dtype=np.int64)
        s.term_kind = arr.ctypes.data_as(C.POINTER(C.c_int64))
        return arr

    assert create(lambda s: None) == 0
    s0, _ = build_setup(model, 0)
    n = s0.nham
    base = [s0.term_kind[i] for i in range(n)]
    assert create(lambda s: kinds(s, [5] + base[1:])) == -7
    k1 = base.index(1)
    assert create(lambda s: setattr(s, "ndiss1", 0)) == -7

    def cross_state(s):
        lhs = np.array([s.lhs_el[i] for i in range(n)], dtype=np.int64)
        lhs[k1] = 1 - lhs[k1]
        s.lhs_el = lhs.ctypes.data_as(C.POINTER(C.c_int64))
        return lhs
    assert create(cross_state) == 0          # equal SPF counts: admitted (a decay channel)
    assert create(lambda s: setattr(s, "ndiss1", 5)) == -1
    assert create(lambda s: setattr(s, "npackets", 17)) == -1
    # still usable
    A, psi = initial_wavefunction(model)
    dA, _ = core_cls(model).calc_derivs(A, psi, 0.0)
    assert np.isfinite(dA).all()


@pytest.mark.parametrize("P,prec,tol", [(3, 0, EOM_RTOL), (1, 0, EOM_RTOL), (3, 1, 1e-6)])
def test_decay_channel_derivs(core_cls, P, prec, tol):
    """Electronic decay L = sqrt(gamma)|1><2|: a type-1 term between the states
    (mean field <V^(not m) A_rhs | AuxA_lhs> added into the operator's slot,
    gmctdh_objects.f90:696-741) and the type-2 anticommutator."""
    from tests.helpers import with_decay
    model = with_decay(small_lvc(nspf=3, grid=(8, 7, 6, 6, 7)), npackets=P, gamma=0.05)
    A, psi = random_mixture(model, seed=21)
    rA, rp = Oracle(model).calc_derivs(A, psi, 0.1)
    dA, dpsi = core_cls(model, precision=prec).calc_derivs(A, psi, 0.1)
    assert _rel(dA, rA) < tol
    assert _rel(dpsi, rp) < tol
