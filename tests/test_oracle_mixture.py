"""Statistical mixtures and dissipation in the CPU oracle (no GPU).

The reference ships no example with npackets > 1 or a dissipation file, so these
pins are properties the equations must have:
  * the Lagrange multipliers conserve the total population and keep orthogonal
    packets orthogonal (gmctdh_objects.f90:612-676, 805-818, 1128-1137);
  * one packet with a type-2 operator is the Hamiltonian with the terms
    i aeD2 aeExtra added (gmctdh_objects.f90:747-845 reuse the Hamiltonian code);
  * an empty packet leaves the other packets' equations unchanged;
  * the parser and the initial mixture (init_calc.f90:490-540, 1093-1126).
"""
import numpy as np
import pytest

from macaw_gb300.model import Term, initial_wavefunction, parse_input, ModelError
from oracle.mctdh import Oracle
from tests.helpers import small_lvc, with_mixture, random_mixture


def _lvc():
    return small_lvc(nspf=3, grid=(8, 7, 6, 6, 7))


@pytest.mark.parametrize("which", ["type1", "type2", "both"])
def test_multipliers_conserve_trace_and_orthogonality(which):
    model = with_mixture(_lvc(), npackets=3)
    if which != "both":
        model.dissipation = [d for d in model.dissipation if d[0] == (1 if which == "type1" else 2)]
        model.finalize()
    A, psi = random_mixture(model, seed=3)
    orc = Oracle(model)
    dA, dpsi = orc.calc_derivs(A, psi, 0.0)
    n, P = model.naconftot, model.npackets
    Am, dAm = A.reshape((n, P), order="F"), dA.reshape((n, P), order="F")
    dS = dAm.conj().T @ Am + Am.conj().T @ dAm        # d/dt <A_i|A_j> (orthonormal SPFs)
    scale = np.abs(dAm).max()
    assert abs(np.trace(dS).real) < 1e-12 * scale
    off = dS - np.diag(np.diag(dS))
    assert np.abs(off).max() < 1e-12 * scale
    # the dissipation moves population between packets (it is not a no-op)
    assert np.abs(np.diag(dS).real).max() > 1e-6 * scale
    # SPF derivatives stay orthogonal to the SPFs (projector)
    for m in model.modes_dvr:
        for s in range(model.nstates):
            phi = model.spf_block(psi, m, s)
            d = dpsi[int(model.ipsispf[m, s]):int(model.ipsispf[m, s]) + phi.size].reshape(phi.shape, order="F")
            assert np.abs(phi.conj().T @ d).max() < 1e-10 * max(1e-30, np.abs(d).max())


def test_single_packet_type2_is_a_hamiltonian_term():
    base = _lvc()
    model = with_mixture(small_lvc(nspf=3, grid=(8, 7, 6, 6, 7)), npackets=1)
    model.dissipation = [d for d in model.dissipation if d[0] == 2]
    model.finalize()
    aeD2 = model.dissipation[0][1]
    base.terms = base.terms + [Term(1j * aeD2 * t.coeff, t.lhs, t.rhs, dict(t.dof_ops))
                               for t in model.dissipation[0][2]]
    base.finalize()
    A, psi = random_mixture(model, seed=1)
    dA1, dp1 = Oracle(model).calc_derivs(A, psi, 0.0)
    dA2, dp2 = Oracle(base).calc_derivs(A, psi, 0.0)
    assert np.allclose(dA1, dA2, rtol=0, atol=1e-13 * np.abs(dA2).max())
    assert np.allclose(dp1, dp2, rtol=0, atol=1e-11 * np.abs(dp2).max())


def test_empty_packet_leaves_the_others_unchanged():
    one = _lvc()
    two = with_mixture(small_lvc(nspf=3, grid=(8, 7, 6, 6, 7)), npackets=2, diss=False)
    A1, psi = random_mixture(one, seed=5)
    A2 = np.concatenate([A1, np.zeros_like(A1)])
    dA1, dp1 = Oracle(one).calc_derivs(A1, psi, 0.0)
    dA2, dp2 = Oracle(two).calc_derivs(A2, psi, 0.0)
    n = one.naconftot
    assert np.allclose(dA2[:n], dA1, rtol=0, atol=1e-13 * np.abs(dA1).max())
    assert np.abs(dA2[n:]).max() == 0.0
    assert np.allclose(dp2, dp1, rtol=0, atol=1e-12 * np.abs(dp1).max())


def test_initial_mixture_from_el_line():
    model = with_mixture(_lvc(), npackets=4, diss=False, eps_pop=1e-3)
    A, psi = initial_wavefunction(model)
    n, P = model.naconftot, model.npackets
    Am = A.reshape((n, P), order="F")
    S = Am.conj().T @ Am
    pops = np.diag(S).real
    # natural states: orthogonal, ascending populations eps*2, eps*3, eps*4, 1, unit trace
    assert np.abs(S - np.diag(pops)).max() < 1e-15
    expect = np.array([2e-3, 3e-3, 4e-3, 1.0])
    assert np.allclose(pops, expect / expect.sum(), rtol=1e-13)
    # the RK interval of a mixture: the packet DeltaPsi of identical states is 0
    assert Oracle(model).delta_psi(A, psi, A, psi) < 1e-7


def test_mixture_input_is_parsed(tmp_path):
    from macaw_gb300.generate import write_inputs
    model = _lvc()
    inp = write_inputs(model, str(tmp_path), "mix")
    txt = open(inp).read()
    txt = "npackets = 2\neps_pop = 1d-4\ndissipation = d1.op\ndissipation = d2.op\n" + txt
    lines = txt.splitlines()
    k = lines.index([l for l in lines if l.strip().startswith("el ")][0])
    lines[k:k + 1] = ["packets", "2 1 1 1 1 1 0.8 0.0", "1 2 1 1 1 1 0.0 0.6"]
    open(inp, "w").write("\n".join(lines) + "\n")
    (tmp_path / "d1.op").write_text("1  0.02\n0.4 | S1&1 | 1 q\n0.4 | S2&2 | 1 q\n")
    (tmp_path / "d2.op").write_text("# comment\n2, 0.03\n-0.5 | 1 | 1 q^2\n")
    m = parse_input(inp)
    assert m.npackets == 2 and m.eps_pop == 1e-4
    assert [d[0] for d in m.dissipation] == [1, 2]
    assert m.aeD1 == [0.01] and m.aeD2 == [0.03]
    assert len(m.dissipation[0][2]) == 2 and m.dissipation[1][2][0].coeff == -0.5
    assert len(m.dissipation[1][2]) == m.nstates
    assert m.init_packets[0][0] == 1 and m.init_packets[1][1] == (1, 0, 0, 0, 0)
    A, psi = initial_wavefunction(m)
    n = m.naconftot
    assert abs(np.vdot(A, A).real - 1.0) < 1e-14
    assert abs(np.vdot(A[:n], A[n:])) < 1e-15
    bad = with_mixture(_lvc(), npackets=1, diss=False)
    bad.dissipation = [(3, 0.1, [Term(1.0, 0, 0, {0: 1})])]
    with pytest.raises(ModelError):
        bad.finalize()


def test_decay_channel_between_states():
    """Electronic decay as a type-1 term between the states (L = sqrt(gamma)|1><2|)
    plus its type-2 anticommutator on a 3-packet mixture: the multipliers keep the
    trace, and state 1 gains population (gamma sum_W WPpopm1_W |<A_W|V A_j>|^2 (1 - p_1)
    + gamma p_1 p_2 > 0 after the diagonal multiplier).  A single packet has no
    multipliers in the reference (derivatives.f90:238), and its type-1 term is the
    projection |<Psi|V|Psi>|^2, so decay needs a mixture."""
    from tests.helpers import with_decay
    P = 3
    model = with_decay(_lvc(), npackets=P, gamma=0.05)
    A, psi = random_mixture(model, seed=9)
    dA, _ = Oracle(model).calc_derivs(A, psi, 0.0)
    n = model.naconftot
    Am, dAm = A.reshape((n, P), order="F"), dA.reshape((n, P), order="F")
    dtrace = float(np.real(np.trace(dAm.conj().T @ Am + Am.conj().T @ dAm)))
    assert abs(dtrace) < 1e-12 * np.abs(dAm).max()
    ref = _lvc()
    ref.npackets = P
    ref.finalize()
    dA0, _ = Oracle(ref).calc_derivs(A, psi, 0.0)
    d0 = (dA - dA0).reshape((n, P), order="F")
    o0, n0 = int(model.astate_offset[0]), int(model.naconf[0])
    gain0 = 2.0 * float(np.real(np.sum(Am[o0:o0 + n0].conj() * d0[o0:o0 + n0])))
    assert gain0 > 0.0


def test_gaussian_overlap_matches_oracle():
    """The set-up code's Gaussian overlap (natural-state start of a Gaussian-mode
    mixture) is the oracle's GauOvlMultiD on random widths and complex centres."""
    from macaw_gb300.model import gaussian_overlap
    from oracle.mctdh import gau_ovl_multid
    rng = np.random.default_rng(4)
    for _ in range(20):
        d = int(rng.integers(1, 5))
        a1, a2 = -rng.uniform(0.1, 2.0, d), -rng.uniform(0.1, 2.0, d)
        x1 = rng.normal(size=d) + 1j * rng.normal(size=d)
        x2 = rng.normal(size=d) + 1j * rng.normal(size=d)
        assert abs(gaussian_overlap(a1, a2, x1, x2) - gau_ovl_multid(a1, a2, x1, x2)) < 1e-14


def test_gaussian_mixture_start_is_orthogonal():
    """OrthoWP with Gaussian SPFs: the packets of the 'el' start are orthogonal in
    the full SPF metric (WF_Ovl with the Gaussian overlaps) and the trace is 1."""
    from tests.helpers import small_gmctdh
    model = with_mixture(small_gmctdh(), npackets=3, diss=False, eps_pop=1e-3)
    A, psi = initial_wavefunction(model)
    orc = Oracle(model)
    pk = orc.packets(A)
    S = np.array([[orc.wf_ovl(pi, psi, pj, psi) for pj in pk] for pi in pk])
    assert abs(np.trace(S).real - 1.0) < 1e-12
    assert np.abs(S - np.diag(np.diag(S))).max() < 1e-12
