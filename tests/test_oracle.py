"""Pins for the CPU oracle (no GPU).

The reference ships no tests or golden outputs and cannot be compiled here (no
Fortran compiler), so the oracle is pinned by physics known-answer tests:
  * analytic autocorrelation of uncoupled displaced harmonic oscillators;
  * the exact limit n_SPF = n_grid against direct propagation with expm;
  * conservation of norm and energy, Hermiticity of rho and h1mode;
  * the committed golden fixtures (tests/golden/make_golden.py).
"""
import os

import numpy as np
import pytest
import scipy.linalg

from macaw_gb300.model import (Model, Term, AU2FS, AU2EV, AU2CMM1, OP_DQ2, INT_RK45, initial_wavefunction,
                               harm_dvr, parse_input)
from macaw_gb300.generate import lvc5, write_inputs
from oracle.mctdh import Oracle, std_reg_inv, herm_from_upper
from tests.helpers import small_lvc, small_qvc, random_state

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _displaced_ho(omegas, kappas, nspf=4, grid=28, eps_int=1e-10, tfinal_fs=6.0):
    terms = []
    for k, (w, kap) in enumerate(zip(omegas, kappas)):
        terms.append(Term(-0.5 * w + 0j, 0, 0, {k: OP_DQ2}))
        terms.append(Term(0.5 * w + 0j, 0, 0, {k: 2}))
        terms.append(Term(kap + 0j, 0, 0, {k: 1}))
    f = len(omegas)
    m = Model(nstates=1, mode_dofs=[[k] for k in range(f)], multiset=[True] * f,
              nspf=np.full((f, 1), nspf), dvr_type=["HO"] * f, ngp=[grid] * f,
              dvrpar=[(0.0, 1.0)] * f, terms=terms, tfinal=tfinal_fs / AU2FS, tout=1.0 / AU2FS,
              eps_int=eps_int, int_type=INT_RK45, init_state=0, label="dho")
    return m.finalize()


def test_harmonic_dvr_spectrum():
    g, w, d1, d2, xd1 = harm_dvr(30, 0.0, 1.0)
    assert np.allclose(d2, d2.T) and np.allclose(d1, -d1.T)
    ev = np.linalg.eigvalsh(-0.5 * d2 + np.diag(0.5 * g ** 2))
    assert np.allclose(ev[:10], np.arange(10) + 0.5, atol=1e-10)
    assert abs(np.sum(w * np.exp(-g ** 2)) - np.sqrt(np.pi)) < 1e-10


def test_displaced_oscillators_analytic_autocorrelation():
    omegas = np.array([1200.0, 2300.0]) / AU2CMM1
    kappas = np.array([0.05, -0.08]) / AU2EV
    model = _displaced_ho(omegas, kappas)
    A, psi = initial_wavefunction(model)
    outs, _, _ = Oracle(model).propagate(A, psi)
    for o in outs:
        t = o["t"]
        c = 1.0 + 0j
        for w, k in zip(omegas, kappas):
            S = 0.5 * (k / w) ** 2
            c *= np.exp(-1j * (0.5 * w - k * k / (2 * w)) * t) * np.exp(-S * (1 - np.exp(-1j * w * t)))
        assert abs(o["auto"] - c) < 2e-7, (t * AU2FS, o["auto"], c)
        assert abs(o["norm"] - 1.0) < 1e-8


def _full_hamiltonian(model):
    dims = [model.ngp[d] for d in range(model.ndof)]
    nprim = int(np.prod(dims))
    H = np.zeros((model.nstates * nprim, model.nstates * nprim), dtype=np.complex128)
    for term in model.terms:
        op = np.eye(1, dtype=np.complex128)
        for d in reversed(range(model.ndof)):
            code = term.dof_ops.get(d, 0)
            if code == 0:
                M = np.eye(dims[d])
            else:
                kind, mat = model.dof_op_matrix(d, code)
                M = mat.T if kind == "dense" else np.diag(mat)
            op = np.kron(op, M)
        E = np.zeros((model.nstates, model.nstates))
        E[term.lhs, term.rhs] = 1.0
        H += term.coeff * np.kron(E, op)
    return H


def test_exact_limit_full_spf_basis():
    """n_SPF = n_grid makes MCTDH exact: C(t) and populations match expm."""
    from tests.helpers import small_qvc  # noqa
    from macaw_gb300.generate import qvc
    model = qvc(2, 2, 6, 6, 1, 11, (800.0, 2500.0), (0.1, 0.2), (0.0, 0.3), "exact", integrator=INT_RK45,
                eps_int=1e-10, tfinal_fs=3.0)
    # 1 DOF per mode: rebuild as two single-DOF modes with a full SPF basis
    model = Model(nstates=2, mode_dofs=[[0], [1]], multiset=[True, True], nspf=np.full((2, 2), 6),
                  dvr_type=["HO", "HO"], ngp=[6, 6], dvrpar=[(0.0, 1.0)] * 2, terms=model.terms,
                  tfinal=3.0 / AU2FS, tout=0.5 / AU2FS, eps_int=1e-10, int_type=INT_RK45,
                  init_state=1, label="exact").finalize()
    A, psi = initial_wavefunction(model)
    outs, _, _ = Oracle(model).propagate(A, psi)
    H = _full_hamiltonian(model)
    # the initial state on the primitive grid: A_{11} phi_1(q1) phi_1(q2) on state 2
    phi1 = model.spf_block(psi, 0, 1)[:, 0]
    phi2 = model.spf_block(psi, 1, 1)[:, 0]
    nprim = 36
    v0 = np.zeros(2 * nprim, dtype=np.complex128)
    v0[nprim:] = np.kron(phi2, phi1)
    for o in outs:
        v = scipy.linalg.expm(-1j * H * o["t"]) @ v0
        c = np.vdot(v0, v)
        assert abs(o["auto"] - c) < 1e-7
        pops = [np.linalg.norm(v[:nprim]) ** 2, np.linalg.norm(v[nprim:]) ** 2]
        assert np.abs(o["pop"] - pops).max() < 1e-7


def test_conservation_and_hermiticity():
    model = small_lvc(eps_int=1e-9, tfinal_fs=2.0)
    A, psi = initial_wavefunction(model)
    o = Oracle(model)
    outs, _, _ = o.propagate(A, psi)
    e0 = outs[0]["energy"]
    for r in outs:
        assert abs(r["norm"] - 1.0) < 1e-7
        assert abs(r["energy"] - e0) < 1e-8
    A, psi = random_state(model, seed=3)
    o.calc_derivs(A, psi, 0.0)
    for (m, s), rho in o.rho.items():
        assert np.allclose(rho, rho.conj().T, atol=1e-15)
    for m, hm in o.h1mode.items():
        for k, h in hm.items():
            l, r, _ = model.oper[m][k]
            if l == r:
                assert np.allclose(h, h.conj().T, atol=1e-14)


def test_regularised_inverse_poly():
    rng = np.random.default_rng(1)
    X = rng.normal(size=(5, 5)) + 1j * rng.normal(size=(5, 5))
    rho = X @ X.conj().T
    rho[:, -1] = 0
    rho[-1, :] = 0
    eps = 1e-8
    inv = std_reg_inv(rho, eps, "poly")
    w, U = np.linalg.eigh(rho)
    assert np.allclose(inv @ U[:, 0], U[:, 0] / (0.5 * (eps + w[0] ** 2 / eps)), rtol=1e-6)
    assert np.allclose(herm_from_upper(np.triu(rho)), rho)


def test_parser_round_trip(tmp_path):
    model = lvc5(grid=[12, 10, 11, 9, 10], nspf=3, eps_int=1e-7)
    path = write_inputs(model, str(tmp_path), "lvc")
    m2 = parse_input(path)
    assert m2.nham == model.nham
    assert np.array_equal(m2.nspf, model.nspf)
    assert np.allclose(m2.ae, model.ae, rtol=1e-13)
    A, psi = initial_wavefunction(model)
    A2, psi2 = initial_wavefunction(m2)
    assert np.allclose(A, A2) and np.allclose(psi, psi2)
    d1 = Oracle(model).calc_derivs(A, psi, 0.0)
    d2 = Oracle(m2).calc_derivs(A2, psi2, 0.0)
    assert np.allclose(d1[0], d2[0], rtol=1e-12, atol=1e-15)


def _reference_example(name):
    from tests.golden.make_butadiene import example_input
    ex = example_input(name)
    if not os.path.exists(ex):
        pytest.skip("the reference's examples are not present (MACAW_REFERENCE_DIR)")
    return ex


@pytest.mark.parametrize("name", ["butadiene_dopri", "butadiene_cmf2"])
def test_reference_examples_parse_like_their_fixtures(name):
    """Both example inputs of the reference parse (interp spline operators,
    sine/HO grids, Gaussian modes, S/M sets, DOPRI and CMF2), and the committed
    fixture the GPU tests run is what they declare."""
    import pickle
    from macaw_gb300.model import model_fields
    model = parse_input(_reference_example(name))
    with open(os.path.join(GOLDEN, name + ".pkl"), "rb") as fh:
        assert pickle.load(fh) == model_fields(model)


def test_butadiene_fixture_model():
    """The fixture rebuilds the example model: the spline operators on the sine
    grid of dof 1 (the q^2 data file is a parabola, which the spline reproduces
    exactly, extrapolation included), a finite start energy, unit norm."""
    import pickle
    from macaw_gb300.model import model_from_fields, INT_DOPRI, OP_PARAM
    with open(os.path.join(GOLDEN, "butadiene_dopri.pkl"), "rb") as fh:
        model = model_from_fields(pickle.load(fh))
    assert model.int_type == INT_DOPRI and model.nmodes == 3 and list(model.nspf[:, 0]) == [6, 6, 7]
    assert len(model.op_params) == 2
    q2 = model.grid_oper[(0, 1)]
    assert np.allclose(q2, model.grid[0] ** 2, rtol=0, atol=1e-10)
    assert any(c > OP_PARAM for t in model.terms for c in t.dof_ops.values())
    A, psi = initial_wavefunction(model)
    ob = Oracle(model).observables(A, psi, A, psi, 0.0)
    assert abs(ob["norm"] - 1.0) < 1e-12 and np.isfinite(ob["energy"])


def test_spline_known_answers():
    """Spline (maths.f90:651-728): quadratic data are reproduced exactly, outside
    the data range too (zero third derivative in the end intervals); the
    interpolant passes through the data and is C2 at the inner knots."""
    from macaw_gb300.model import spline
    x = np.array([-3.0, -2.2, -1.0, 0.0, 0.7, 1.5, 3.0])
    xx = np.linspace(-4.0, 4.0, 41)
    assert np.allclose(spline(x, 2.0 * x ** 2 - x + 0.5, xx), 2.0 * xx ** 2 - xx + 0.5, rtol=0, atol=1e-12)
    y = np.sin(x)
    assert np.allclose(spline(x, y, x), y, rtol=0, atol=1e-13)
    h = 1e-4
    for xk in x[1:-1]:
        left = spline(x, y, np.array([xk - 2 * h, xk - h, xk]))
        right = spline(x, y, np.array([xk, xk + h, xk + 2 * h]))
        d1l, d1r = (left[2] - left[1]) / h, (right[1] - right[0]) / h
        assert abs(d1l - d1r) < 1e-3
        d2l = (left[2] - 2 * left[1] + left[0]) / h ** 2
        d2r = (right[2] - 2 * right[1] + right[0]) / h ** 2
        assert abs(d2l - d2r) < 1e-2


@pytest.mark.parametrize("MM", [0, 1, 2])
def test_legendre_dvr_known_answers(MM):
    """Leg_DVR (dvr.f90:361-530): the grid is symmetric about pi/2; the FBR of
    L0^2 + M^2 sin^-2 is diag(l(l+1)), l = M .. M + n - 1; for M > 0 the FBR of
    sin^-2 has the closed form <P_M^M|sin^-2|P_M^M> = (2M+1)/(2M); for M = 0 the
    quadrature-built sin^-2 is symmetric positive definite; the M = 0 weights sum
    to 2; d1 is antisymmetric."""
    from macaw_gb300.model import leg_dvr
    n = 12
    g, w, d1, d2, xd1, tr, sm2 = leg_dvr(n, MM, True)
    assert np.allclose(g + g[::-1], np.pi, atol=1e-13)
    L2 = tr @ (d2 + MM ** 2 * sm2) @ tr.T
    ll = MM + np.arange(n)
    assert np.allclose(L2, np.diag(ll * (ll + 1.0)), atol=1e-9)
    assert np.allclose(d1, -d1.T, atol=1e-14)
    if MM > 0:
        fbr = tr @ sm2 @ tr.T
        assert abs(fbr[0, 0] - (2 * MM + 1) / (2.0 * MM)) < 1e-12
    else:
        assert abs(w.sum() - 2.0) < 1e-12
        assert np.allclose(sm2, sm2.T) and np.linalg.eigvalsh(sm2).min() > 0.0


def test_parametrised_operator_values():
    """gridOper of every parametrised function (hamilton.f90:210-290) on the
    grids of the synthetic model the GPU tests use; the eig_proj vector is the
    normalised eigenvector of -p2 d2 + V (Eigenf1DPot_real)."""
    from macaw_gb300.model import OP_PARAM
    from tests.helpers import parametrised_model
    m = parametrised_model()
    x = m.grid[3]
    assert np.allclose(m.grid_oper[(3, 1)], np.exp(-0.1 * x - 0.05 * x ** 2))
    assert np.allclose(m.grid_oper[(1, 3)], (np.abs(m.grid[1] - 0.5) < 1.5).astype(float))
    assert np.allclose(m.grid_oper[(3, 4)], x ** 2 * np.exp(0.2 * x - 0.1 * x ** 2))
    assert np.allclose(m.grid_oper[(0, 5)], np.sin(m.grid[0]) ** 2)
    v = m.grid_oper[(3, 7)]
    H = -0.5 * m.d2[3] + np.diag(0.5 * x ** 2)
    assert abs(np.linalg.norm(v) - 1.0) < 1e-12
    assert np.linalg.norm(H @ v - (v @ H @ v) * v) < 1e-10
    kind, P = m.dof_op_matrix(3, -OP_PARAM - 7)
    assert kind == "dense" and np.allclose(P @ P, P)


def test_model_fields_round_trip():
    from macaw_gb300.model import model_fields, model_from_fields
    from tests.helpers import parametrised_model
    m = parametrised_model()
    m2 = model_from_fields(model_fields(m))
    assert np.array_equal(m.ae, m2.ae) and m.ioper.tolist() == m2.ioper.tolist()
    for k, v in m.grid_oper.items():
        assert np.array_equal(v, m2.grid_oper[k])


@pytest.mark.parametrize("name", ["lvc_small", "qvc_small"])
def test_golden_fixtures(name):
    from tests.golden.make_golden import compute
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    cur = compute(name)
    for key in g.files:
        assert np.allclose(cur[key], g[key], rtol=1e-11, atol=1e-13), key


@pytest.mark.parametrize("builder", ["lvc", "gmctdh"])
def test_writer_quantities_oracle(builder):
    """Natural populations of every mode sum to the state population (the trace of
    rho, of rho S for Gaussian modes), population errors are sorted and
    non-negative, and <1> equals the norm (output.f90:88-140, 449-500)."""
    from tests.helpers import small_lvc, small_gmctdh, random_state, with_expect
    model = small_lvc() if builder == "lvc" else small_gmctdh()
    if builder == "gmctdh":
        initial_wavefunction(model)
    model = with_expect(model)
    A, psi = random_state(model, seed=11)
    o = Oracle(model)
    ev = o.expectation(A, psi)
    obs = o.observables(A, psi, A, psi, 0.0)
    assert abs(ev[0] - obs["norm"]) < 1e-12
    assert abs(ev[1] - obs["pop"][0]) < 1e-12
    assert abs(ev[2].imag) < 1e-12          # q is Hermitian
    nat, ggp, perr = o.natpop(A, psi)
    for (mode, s), w in nat.items():
        assert np.all(np.diff(w) <= 1e-14)
        assert abs(w.sum() - obs["pop"][s]) < 1e-10
    for key, e in perr.items():
        assert np.all(e >= 0) and np.all(np.diff(e) <= 0)
        assert abs(ggp[key].sum() - obs["pop"][key[1]]) < 1e-10


def test_expect_keyword_is_parsed(tmp_path):
    model = lvc5(grid=[12, 10, 11, 9, 10], nspf=3, eps_int=1e-7)
    path = write_inputs(model, str(tmp_path), "lvc")
    with open(os.path.join(str(tmp_path), "q1.op"), "w") as fh:
        fh.write("# position of dof 1\n1.0 | 1 | 1 q\n")
    with open(path) as fh:
        text = fh.read()
    with open(path, "w") as fh:
        fh.write("expect = q1.op\n" + text)
    m2 = parse_input(path)
    assert len(m2.expect) == 1 and len(m2.expect[0]) == m2.nstates
    assert all(t.dof_ops == {0: 1} and t.lhs == t.rhs for t in m2.expect[0])
    # the expectation operator's mode operators follow the Hamiltonian's
    assert m2.nham == model.nham
    assert np.array_equal(m2.ioper, model.ioper)


@pytest.mark.parametrize("builder", ["qvc", "gmctdh"])
def test_density_oracle(builder):
    """Calc_Density: on a grid DOF the density and the basis populations both sum to
    the state population; on a Gaussian DOF the Riemann sum of the density over the
    plotting range approaches it."""
    from tests.helpers import small_qvc, small_gmctdh, random_state
    model = small_qvc() if builder == "qvc" else small_gmctdh()
    if builder == "gmctdh":
        initial_wavefunction(model)
    A, psi = random_state(model, seed=12)
    o = Oracle(model)
    pop = o.observables(A, psi, A, psi, 0.0)["pop"]
    for dof in range(model.ndof):
        if model.dvr_type[dof] == "gwp":
            dens, _ = o.density(A, psi, dof, xrange=model.dvrpar[dof])
            assert np.abs(dens.sum(axis=0) - pop).max() < 1e-3
        else:
            dens, bpop = o.density(A, psi, dof, trafo=model.trafo[dof])
            assert np.abs(dens.sum(axis=0) - pop).max() < 1e-10
            assert np.abs(bpop.sum(axis=0) - pop).max() < 1e-10
