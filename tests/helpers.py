"""Shared test helpers: small seeded models and random MCTDH states."""
import numpy as np

from macaw_gb300.generate import gmctdh16, lvc5, qvc
from macaw_gb300.model import (AU2FS, INT_CMF2, INT_RK45, Model, OP_DQ2, OP_PARAM, OP_SINM2, PAR_COS,
                               PAR_EIGPROJ, PAR_GAU, PAR_HERMITE, PAR_INTERP, PAR_SIN, PAR_SQUARE, Term,
                               initial_wavefunction)


def small_lvc(nspf=3, grid=(12, 10, 11, 9, 10), eps_int=1e-7, tfinal_fs=2.0):
    return lvc5(grid=list(grid), nspf=nspf, eps_int=eps_int, tfinal_fs=tfinal_fs)


def small_qvc(nstates=3, ndof=4, grid=6, nspf=4, integrator=INT_CMF2, eps_int=1e-5, tfinal_fs=1.0, seed=7):
    return qvc(nstates, ndof, grid, nspf, 2, seed, (200.0, 3500.0), (0.05, 0.2),
               tuple(np.linspace(0.0, 0.7, nstates)), "qvc-small", integrator=integrator,
               eps_int=eps_int, eps_lanczos=1e-8, eps_spf=1e-7, tfinal_fs=tfinal_fs)


def small_gmctdh(tfinal_fs=1.0, eps_int=1e-6):
    """2-state LVC: 4 HO DVR modes (6 points, 3 SPFs) + one Gaussian mode of 2 DOFs
    with 4 Gaussians per state (the G-MCTDH model at small size)."""
    return gmctdh16(ngwp=4, gwp_dofs=2, dvr_grid=6, dvr_nspf=3, tfinal_fs=tfinal_fs, eps_int=eps_int)


def random_state(model, seed=0, spread=1.0, gwp_shift=0.1):
    """Random normalised A and SPF blocks with orthonormal columns (per mode and state)."""
    rng = np.random.default_rng(seed)
    A = rng.normal(size=model.naconftot) + 1j * rng.normal(size=model.naconftot)
    A *= spread
    psi = np.zeros(model.dimpsi, dtype=np.complex128)
    if model.modes_gwp:
        # Gaussian parameters: the initial ones, displaced at random
        _, psi0 = initial_wavefunction(model)
        for m in model.modes_gwp:
            for s in range(model.nstates):
                o = int(model.ipsispf[m, s])
                n = int(model.nspf[m, s]) * len(model.mode_dofs[m])
                psi[o:o + n] = psi0[o:o + n] + gwp_shift * (rng.normal(size=n) + 1j * rng.normal(size=n))
    for m in range(model.nmodes):
        if model.is_gwp_mode[m]:
            continue
        for s in range(model.nstates):
            if (not model.multiset[m]) and s > 0:
                continue
            G = model.ngpm[m]
            n = int(model.nspf[m, s])
            X = rng.normal(size=(G, n)) + 1j * rng.normal(size=(G, n))
            q, _ = np.linalg.qr(X)
            o = int(model.ipsispf[m, s])
            psi[o:o + G * n] = q.reshape(-1, order="F")
    from oracle.mctdh import Oracle
    nrm = Oracle(model).norm_wf(A, psi)
    return A / np.sqrt(nrm), psi


def with_expect(model):
    """The model with expectation operators (the 'expect' keyword): the identity
    (= the norm), the projector on state 1, q of dof 1 on every state, and the
    one-sided coherence |1><2| q of dof 2 (complex in general)."""
    from macaw_gb300.model import Term
    ns = model.nstates
    model.expect = [
        [Term(1.0, s, s, {}) for s in range(ns)],
        [Term(1.0, 0, 0, {})],
        [Term(1.0, s, s, {0: 1}) for s in range(ns)],
        [Term(0.5, 0, 1, {1: 1})],
    ]
    gwpa = getattr(model, "gwpa", None)
    model.finalize()
    if gwpa is not None:
        model.gwpa = gwpa
    return model


def with_mixture(model, npackets=3, diss=True, eps_pop=1e-6):
    """The model as a statistical mixture of `npackets` packets, with (diss=True)
    a type-1 operator V = 0.4 q_1 on every state plus 0.3 q_2^2 on state 1 and
    coefficient 0.02 (aeD1 = 0.01), and a type-2 operator W = -0.5 q_1^2 on
    every state plus the coupling 0.2 (|1><2| + |2><1|) q_3 with coefficient 0.03."""
    from macaw_gb300.model import Term
    ns = model.nstates
    model.npackets = npackets
    model.eps_pop = eps_pop
    model.dissipation = []
    if diss:
        v = [Term(0.4, s, s, {0: 1}) for s in range(ns)] + [Term(0.3, 0, 0, {1: 2})]
        w = [Term(-0.5, s, s, {0: 2}) for s in range(ns)]
        if ns > 1:
            w += [Term(0.2, 0, 1, {2: 1}), Term(0.2, 1, 0, {2: 1})]
        model.dissipation = [(1, 0.02, v), (2, 0.03, w)]
    return model.finalize()


def random_mixture(model, seed=0, pops=None):
    """Random SPFs and P mutually orthogonal packets with distinct populations
    (default 0.6, 0.3, 0.1, ... normalised to unit trace), packet-major."""
    rng = np.random.default_rng(seed)
    P = model.npackets
    A1, psi = random_state(model, seed=seed)
    n = model.naconftot
    X = rng.normal(size=(n, P)) + 1j * rng.normal(size=(n, P))
    q, _ = np.linalg.qr(X)
    if pops is None:
        pops = np.array([0.6 / 2 ** k for k in range(P)])
    pops = np.asarray(pops, dtype=float)
    pops = pops / pops.sum()
    A = (q * np.sqrt(pops)[None, :]).reshape(-1, order="F")
    return A, psi


def with_decay(model, npackets=2, gamma=0.05, eps_pop=1e-6):
    """The model as a mixture under electronic decay L = sqrt(gamma) |1><2|:
    gamma L rho L^+ as a type-1 term between the states and -gamma/2 {|2><2|, rho}
    as a type-2 term (state indices 0-based: |0><1| and |1><1|)."""
    from macaw_gb300.model import Term
    model.npackets = npackets
    model.eps_pop = eps_pop
    model.dissipation = [(1, gamma, [Term(1.0, 0, 1, {})]), (2, -0.5 * gamma, [Term(1.0, 1, 1, {})])]
    return model.finalize()


def parametrised_model(tfinal_fs=0.5):
    """2 states; mode 1 = Legendre DOF (M = 0, 14 points) x sine DOF (9 points),
    mode 2 = Legendre DOF (M = 1, 10 points), mode 3 = HO DOF (16 points).  The
    Hamiltonian uses L0^2 and sin^-2 on the angles and every parametrised
    operator; the spline data are a double well sampled on 13 points."""
    x = np.linspace(-6.0, 6.0, 13)
    interp = {"dw.dat": (x, 0.02 * (x ** 2 - 4.0) ** 2 / 16.0), "harm.dat": (x, 0.5 * x ** 2)}
    ops = [(PAR_GAU, -0.1, -0.05, 0.0, ""), (PAR_INTERP, 0.0, 0.0, 0.0, "dw.dat"),
           (PAR_SQUARE, 0.5, 3.0, 0.0, ""), (PAR_HERMITE, 0.2, -0.1, 2.0, ""),
           (PAR_SIN, 1.0, 2.0, 0.0, ""), (PAR_COS, 1.0, 1.0, 0.0, ""),
           (PAR_EIGPROJ, 0.0, 0.5, 1.0, "harm.dat")]
    P = [OP_PARAM + j for j in range(1, 8)]
    terms = []
    for s in range(2):
        terms += [Term(0.004 + 0j, s, s, {0: OP_DQ2}), Term(0.001 + 0j, s, s, {0: 2}),
                  Term(-0.003 + 0j, s, s, {1: OP_DQ2}), Term(0.002 + 0j, s, s, {1: 2}),
                  Term(0.005 + 0j, s, s, {2: OP_DQ2}), Term(0.001 + 0j, s, s, {2: OP_SINM2}),
                  Term(-0.004 + 0j, s, s, {3: OP_DQ2}), Term(0.004 + 0j, s, s, {3: P[1]})]
    terms += [Term(0.01 + 0j, 0, 0, {}), Term(-0.01 + 0j, 1, 1, {}),
              Term(0.003 + 0j, 0, 0, {3: P[0]}), Term(0.002 + 0j, 1, 1, {1: P[2], 3: 1}),
              Term(0.001 + 0j, 0, 0, {3: P[3]}), Term(0.002 + 0j, 1, 1, {0: P[4]}),
              Term(0.003 + 0j, 0, 0, {2: P[5]}), Term(0.004 + 0j, 1, 1, {3: -P[6]}),
              Term(0.006 + 0j, 0, 1, {3: 1}), Term(0.006 + 0j, 1, 0, {3: 1}),
              Term(0.002 + 0j, 0, 1, {0: P[5]}), Term(0.002 + 0j, 1, 0, {0: P[5]})]
    m = Model(nstates=2, mode_dofs=[[0, 1], [2], [3]], multiset=[True, True, True],
              nspf=np.array([[4, 3], [3, 3], [4, 4]]), dvr_type=["Leg", "sin", "Leg", "HO"],
              ngp=[14, 9, 10, 16], dvrpar=[(0.0, 0.0), (-4.0, 4.0), (1.0, 0.0), (0.0, 1.0)],
              terms=terms, tfinal=tfinal_fs / AU2FS, tout=0.25 / AU2FS, eps_int=1e-7,
              int_type=INT_RK45, init_state=1, label="parametrised",
              op_params=ops, interp_data=interp)
    m.init_spf[0] = ("Leg", (0, 0))
    m.init_spf[2] = ("Leg", (1, 1))
    return m.finalize()
