"""Seeded synthetic vibronic-coupling models in the reference's input formats.

Each workload is drawn with ``numpy.random.default_rng(20261203 + index)``
(dimensionless normal modes, coefficients in Hartree).  Kinetic and potential
terms follow the butadiene example's convention (``-w/2 |1| k dq^2``,
``w/2 |1| k q^2``); linear intrastate couplings use ``| Sa&a | k q``,
diagonal quadratic ones ``| Sa&a | k q^2``, interstate couplings
``| Sa&b | k q`` and vertical energies ``| Sa&a``.  The initial state is the
ground-state Gaussian ``k gauss 0.0 0.0 0.707107`` on one electronic state.

Workloads (sizes as named by their builders):
  lvc5      2-state LVC, 5 HO modes (24-40 points), 6 SPFs per mode, RK45 1e-8
  qvc12     3-state QVC, 12 DOFs paired into 6 modes of 20x20 grids, 8 SPFs, CMF2
  ensemble  ragged LVC instances (2-4 states, 4-10 modes, 4-10 SPFs, 16-48 points)
  gmctdh16  2-state LVC: 4 HO DVR modes + one 12-DOF Gaussian mode (32 GWPs)
  qvc24     4-state QVC, 24 DOFs in 8 three-DOF modes of 12^3 grids, 8 SPFs, CMF2
"""
from __future__ import annotations

import math
import os
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from .model import (Model, Term, AU2EV, AU2FS, AU2CMM1, INT_RK45, INT_CMF2, OP_DQ2,
                    initial_wavefunction)

SEED0 = 20261203


def _vibronic_terms(nstates: int, omegas: Sequence[float], kappa: np.ndarray,
                    gamma: Optional[np.ndarray], lambdas: Sequence[Tuple[int, int, int, float]],
                    energies: Sequence[float]) -> List[Term]:
    """LVC/QVC Hamiltonian terms, in the term order read_declare_ham produces."""
    terms: List[Term] = []
    for k, w in enumerate(omegas):
        for s in range(nstates):
            terms.append(Term(-0.5 * w + 0j, s, s, {k: OP_DQ2}))
        for s in range(nstates):
            terms.append(Term(0.5 * w + 0j, s, s, {k: 2}))
    for s, e in enumerate(energies):
        terms.append(Term(complex(e), s, s, {}))
    for s in range(nstates):
        for k in range(len(omegas)):
            if kappa[s, k] != 0.0:
                terms.append(Term(complex(kappa[s, k]), s, s, {k: 1}))
    if gamma is not None:
        for s in range(nstates):
            for k in range(len(omegas)):
                if gamma[s, k] != 0.0:
                    terms.append(Term(complex(gamma[s, k]), s, s, {k: 2}))
    for (a, b, k, lam) in lambdas:
        terms.append(Term(complex(lam), a, b, {k: 1}))
        terms.append(Term(complex(lam), b, a, {k: 1}))
    return terms


def lvc5(seed: int = SEED0 + 0, grid: Optional[Sequence[int]] = None, nspf: int = 6,
         eps_int: float = 1e-8, tfinal_fs: float = 100.0) -> Model:
    """2-state LVC over 5 HO modes (24-40 points), 6 SPFs per mode and state."""
    rng = np.random.default_rng(seed)
    f = 5
    omegas = rng.uniform(300.0, 3200.0, f) / AU2CMM1
    kappa = rng.normal(0.0, 0.08, (2, f)) / AU2EV
    lam_mode = int(rng.integers(0, f))
    ngp = [int(x) for x in rng.integers(24, 41, f)] if grid is None else list(grid)
    terms = _vibronic_terms(2, omegas, kappa, None, [(0, 1, lam_mode, 0.15 / AU2EV)],
                            [-0.25 / AU2EV, 0.25 / AU2EV])
    model = Model(nstates=2, mode_dofs=[[k] for k in range(f)], multiset=[True] * f,
                  nspf=np.full((f, 2), nspf), dvr_type=["HO"] * f, ngp=ngp,
                  dvrpar=[(0.0, 1.0)] * f, terms=terms, tfinal=tfinal_fs / AU2FS,
                  tout=0.5 / AU2FS, eps_int=eps_int, int_type=INT_RK45, init_state=1,
                  label="lvc5")
    return model.finalize()


def qvc(nstates: int, ndof: int, grid: int, nspf: int, ncoup: int, seed: int,
        wrange: Tuple[float, float], lam_range: Tuple[float, float], energies_ev: Sequence[float],
        label: str, integrator: int = INT_CMF2, eps_int: float = 1e-5,
        eps_lanczos: float = 1e-8, eps_spf: float = 1e-8, tfinal_fs: float = 200.0,
        init_state: Optional[int] = None, tout_fs: float = 0.5, dofs_per_mode: int = 2) -> Model:
    """QVC model with `dofs_per_mode` DOFs combined into each logical mode
    (grid^dofs_per_mode points)."""
    rng = np.random.default_rng(seed)
    omegas = rng.uniform(wrange[0], wrange[1], ndof) / AU2CMM1
    kappa = rng.normal(0.0, 0.1, (nstates, ndof)) / AU2EV
    gamma = rng.normal(0.0, 0.01, (nstates, ndof)) / AU2EV
    cdofs = rng.choice(ndof, size=ncoup, replace=False)
    pairs = [(a, b) for a in range(nstates) for b in range(a + 1, nstates)]
    lambdas = []
    for k in cdofs:
        a, b = pairs[int(rng.integers(0, len(pairs)))]
        lambdas.append((a, b, int(k), float(rng.uniform(*lam_range)) / AU2EV))
    terms = _vibronic_terms(nstates, omegas, kappa, gamma, lambdas,
                            [e / AU2EV for e in energies_ev])
    k = dofs_per_mode
    nmodes = ndof // k
    model = Model(nstates=nstates, mode_dofs=[[k * m + i for i in range(k)] for m in range(nmodes)],
                  multiset=[True] * nmodes, nspf=np.full((nmodes, nstates), nspf),
                  dvr_type=["HO"] * ndof, ngp=[grid] * ndof, dvrpar=[(0.0, 1.0)] * ndof,
                  terms=terms, tfinal=tfinal_fs / AU2FS, tout=tout_fs / AU2FS, eps_int=eps_int,
                  int_type=integrator, init_state=nstates - 1 if init_state is None else init_state,
                  eps_A=eps_lanczos, eps_psi=eps_spf, label=label)
    model.coupling_pairs = lambdas
    return model.finalize()


def qvc12(seed: int = SEED0 + 1, grid: int = 20, nspf: int = 8, **kw) -> Model:
    """3-state QVC, 12 DOFs -> 6 modes of 20x20 HO grids, 8 SPFs, CMF2 + Lanczos."""
    return qvc(3, 12, grid, nspf, 4, seed, (200.0, 3500.0), (0.05, 0.2), (0.0, 0.3, 0.7),
               "qvc12", **kw)


def qvc24(seed: int = SEED0 + 4, grid: int = 12, nspf: int = 8, dofs_per_mode: int = 3, **kw) -> Model:
    """4-state QVC over 24 DOFs combined into 8 logical modes of three DOFs (12^3-point
    HO product grids), 8 SPFs per mode and state: 8^8 = 16,777,216 configurations per
    state, 1.07 GB of FP64 coefficients for the four states."""
    return qvc(4, 24, grid, nspf, 8, seed, (150.0, 3500.0), (0.02, 0.2), (0.0, 0.3, 0.7, 1.0),
               "qvc24", tfinal_fs=300.0, dofs_per_mode=dofs_per_mode, **kw)


def ensemble_member(rng: np.random.Generator, idx: int, max_conf: int = 1 << 20) -> Model:
    """One ragged LVC instance: 2-4 states, 4-10 modes, 4-10 SPFs, 16-48 points,
    re-drawn until prod(nSPF) <= max_conf."""
    while True:
        S = int(rng.integers(2, 5))
        f = int(rng.integers(4, 11))
        n = int(rng.integers(4, 11))
        if n ** f <= max_conf:
            break
    ngp = [int(x) for x in rng.integers(16, 49, f)]
    omegas = rng.uniform(300.0, 3200.0, f) / AU2CMM1
    kappa = rng.normal(0.0, 0.08, (S, f)) / AU2EV
    lam_mode = int(rng.integers(0, f))
    a, b = 0, int(rng.integers(1, S))
    energies = list(np.linspace(-0.25, 0.25, S) / AU2EV)
    terms = _vibronic_terms(S, omegas, kappa, None, [(a, b, lam_mode, 0.15 / AU2EV)], energies)
    model = Model(nstates=S, mode_dofs=[[k] for k in range(f)], multiset=[True] * f,
                  nspf=np.full((f, S), n), dvr_type=["HO"] * f, ngp=ngp,
                  dvrpar=[(0.0, 1.0)] * f, terms=terms, tfinal=100.0 / AU2FS,
                  tout=0.5 / AU2FS, eps_int=1e-6, int_type=INT_RK45,
                  init_state=int(rng.integers(1, S)), label=f"ensemble[{idx}]")
    return model.finalize()


def ensemble(count: int = 512, seed: int = SEED0 + 2, max_conf: int = 1 << 20) -> List[Model]:
    rng = np.random.default_rng(seed)
    return [ensemble_member(rng, i, max_conf) for i in range(count)]


def gmctdh16(seed: int = SEED0 + 3, ngwp: int = 32, gwp_dofs: int = 12, dvr_grid: int = 32,
             dvr_nspf: int = 6, tfinal_fs: float = 100.0, eps_int: float = 1e-6) -> Model:
    """2-state LVC over 16 DOFs: 4 HO DVR modes + one Gaussian mode of 12 DOFs."""
    rng = np.random.default_rng(seed)
    ndof = 4 + gwp_dofs
    omegas = rng.uniform(300.0, 3200.0, ndof) / AU2CMM1
    kappa = rng.normal(0.0, 0.08, (2, ndof)) / AU2EV
    lam_mode = int(rng.integers(0, 4))
    terms = _vibronic_terms(2, omegas, kappa, None, [(0, 1, lam_mode, 0.15 / AU2EV)],
                            [-0.25 / AU2EV, 0.25 / AU2EV])
    mode_dofs = [[k] for k in range(4)] + [list(range(4, ndof))]
    nspf = np.array([[dvr_nspf, dvr_nspf]] * 4 + [[ngwp, ngwp]])
    model = Model(nstates=2, mode_dofs=mode_dofs, multiset=[True] * 5, nspf=nspf,
                  dvr_type=["HO"] * 4 + ["gwp"] * gwp_dofs, ngp=[dvr_grid] * 4 + [101] * gwp_dofs,
                  dvrpar=[(0.0, 1.0)] * 4 + [(-10.0, 10.0)] * gwp_dofs, terms=terms,
                  tfinal=tfinal_fs / AU2FS, tout=0.5 / AU2FS, eps_int=eps_int, eps_ovl=1e-8, eps_C=1e-8,
                  int_type=INT_RK45, init_state=1, label="gmctdh16")
    for d in range(4, ndof):
        model.init_spf[d] = ("gwp", (0, 0.0, 0.0, 0.707107, 0.8, 0.9))
    return model.finalize()


# ----------------------------------------------------------------------------
# Writers for the reference's formats (input.f90 keyword grammar, operator file)
# ----------------------------------------------------------------------------

def _opname(code: int) -> str:
    return {-1: "p", -2: "dq^2", -3: "qp", 1: "q"}.get(code, f"q^{code}")


def write_inputs(model: Model, directory: str, name: str = "model") -> str:
    """Write ``<name>.inp`` and ``<name>.op`` that the reference reads unchanged."""
    os.makedirs(directory, exist_ok=True)
    ops = []
    for t in model.terms:
        el = f"S{t.lhs + 1}&{t.rhs + 1}"
        seg = "".join(f" |{d + 1:2d}  {_opname(c)}" for d, c in sorted(t.dof_ops.items()))
        ops.append(f"{t.coeff.real: .14e}  | {el}{seg}")
    # Hermitian pairs Sa&b / Sb&a are written once (the reader expands them)
    out, seen = [], set()
    for t, line in zip(model.terms, ops):
        key = (min(t.lhs, t.rhs), max(t.lhs, t.rhs), tuple(sorted(t.dof_ops.items())), t.coeff)
        if t.lhs != t.rhs:
            if key in seen:
                continue
            seen.add(key)
        out.append(line)
    with open(os.path.join(directory, name + ".op"), "w") as fh:
        fh.write("# generated vibronic-coupling Hamiltonian\n" + "\n".join(out) + "\n")
    L = []
    L.append(f"tfinal = {model.tfinal * AU2FS:.6f}")
    L.append(f"tout = {model.tout * AU2FS:.6f}")
    L.append(f"nstates = {model.nstates}")
    L.append(f"ndof = {model.ndof}")
    L.append(f"nmodes = {model.nmodes}")
    L.append("SPF")
    for m in range(model.nmodes):
        dofs = ",".join(str(d + 1) for d in model.mode_dofs[m])
        spf = ",".join(str(int(x)) for x in model.nspf[m])
        L.append(f" {'M' if model.multiset[m] else 'S'},  {dofs} = {spf}")
    L.append("GRID")
    for d in range(model.ndof):
        if model.dvr_type[d] == "gwp":
            L.append(f" {d + 1:3d}  gwp")
        else:
            L.append(f" {d + 1:3d}  {model.dvr_type[d]}  {model.ngp[d]}  {model.dvrpar[d][0]}  {model.dvrpar[d][1]}")
    L.append(f"Hamiltonian = {name}.op")
    L.append("INIT-WF")
    L.append("   single-conf")
    L.append(f"   el  {model.init_state + 1}")
    for d in range(model.ndof):
        kind, par = model.init_spf.get(d, ("gauss", (0.0, 0.0, 0.707107)))
        if kind == "gauss":
            L.append(f"   {d + 1}  gauss  {par[0]}  {par[1]}  {par[2]}")
        else:
            L.append(f"   {d + 1}  gwp {par[0]}  {par[1]}  {par[2]}  {par[3]}  ovl = {par[4]}  scw = {par[5]}")
    L.append("END-INIT-WF")
    L.append(f"eps_int = {model.eps_int:.3e}")
    L.append(f"eps_rho = {model.eps_rho:.3e}")
    L.append(f"eps_C = {model.eps_C:.3e}")
    L.append(f"eps_S = {model.eps_ovl:.3e}")
    L.append(f"minstep = {model.min_stepsize * AU2FS:.3e}")
    if model.int_type == INT_CMF2:
        L.append("integration = CMF2")
        L.append(f"Lanczos  {model.eps_A:.3e}")
        L.append(f"rk45     {model.eps_psi:.3e}")
    else:
        L.append("integration = " + ("rk45" if model.int_type == INT_RK45 else "dopri"))
    path = os.path.join(directory, name + ".inp")
    with open(path, "w") as fh:
        fh.write("\n".join(L) + "\n")
    return path


BUILDERS = {"lvc5": lvc5, "qvc12": qvc12, "gmctdh16": gmctdh16, "qvc24": qvc24}


def lvc5_mixture(npackets: int = 4, gamma: float = 2e-3, eps_int: float = 1e-8, tfinal_fs: float = 100.0,
                 eps_pop: float = 1e-6) -> Model:
    """lvc5 as a statistical mixture of `npackets` packets (initialised from the
    'el' line) under Lindblad dephasing of mode 1 with L = sqrt(gamma) q:
    D[L] rho = gamma (q rho q - 1/2 {q^2, rho}), i.e. a type-1 operator V = q with
    alpha = gamma and a type-2 operator W = q^2 with beta = -gamma / 2, on every
    electronic state (input.f90:216-229, 596-616)."""
    model = lvc5(eps_int=eps_int, tfinal_fs=tfinal_fs)
    ns = model.nstates
    model.npackets = npackets
    model.eps_pop = eps_pop
    model.dissipation = [(1, gamma, [Term(1.0, s, s, {0: 1}) for s in range(ns)]),
                         (2, -0.5 * gamma, [Term(1.0, s, s, {0: 2}) for s in range(ns)])]
    model.label = "lvc5-mixture"
    return model.finalize()
