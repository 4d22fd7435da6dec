"""Host-side model set-up for the G-MCTDH propagation core.

This module stands in for the reference's one-off host work that precedes the
time loop: reading the keyword input and the operator file
(input.f90:30-426, :812-1144), building the primitive DVR grids and matrices
(dvr.f90:107-357), deduplicating the per-mode operators
(hamilton.f90:91-167, :353-399), laying out the coefficient and SPF vectors
(init_calc.f90:22-53, :160-181) and building the initial wavefunction
(init_calc.f90:230-761 single-conf, :763-1068 SetSPF).

Everything here is FP64 NumPy and runs once per model.  The arrays produced
are exactly what the reference keeps in its global modules (psidef, storage,
hamilton, dvr); they are handed to the GPU core through the C-ABI
(``include/macaw_gb300.h``) and to the CPU oracle.

Indexing is 0-based throughout (the reference is 1-based); tensors keep the
reference's column-major order with mode 1 fastest (init_calc.f90:531-536).
"""
from __future__ import annotations

import dataclasses
import functools
import math
import os
import re
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

AU2EV = 27.2113961          # globals.f90:17
AU2FS = 0.02418884326505    # globals.f90:17
AU2CMM1 = 219474.63         # globals.f90:18

# Primitive DOF operator codes (input.f90:1098-1137, hamilton.f90:27-30)
OP_ID = 0
OP_P = -1        # p = -i d/dq
OP_DQ2 = -2      # d^2/dq^2
OP_QP = -3       # qp + pq
OP_SINM2 = -4    # sin^-2 (Legendre DVR only)
# Parametrised DOF operators (input.f90:950-1072): code 200 + j applies the
# diagonal gridOper(:, j, dof); code -200 - j the projector v v^T with
# v = gridOper(:, j, dof) (MultTensProj, hamilton.f90:632-661); j is 1-based
# in the order the operator files declare them.
OP_PARAM = 200
PAR_GAU = 0        # exp(p1 x + p2 x^2)
PAR_INTERP = 1     # cubic spline through the points of a data file
PAR_SQUARE = 2     # indicator of |x - p1| < p2 / 2
PAR_HERMITE = 3    # x^r exp(p1 x + p2 x^2), r = p3
PAR_SIN = 4        # sin(p1 x)^p2
PAR_COS = 5        # cos(p1 x)^p2
PAR_EIGPROJ = 6    # eigenfunction p3 of -p2 d^2/dx^2 + V(x), V splined from a data file

INT_RK45 = 1     # Cash-Karp (input.f90:280-282)
INT_DOPRI = 2    # Dormand-Prince (input.f90:283-285)
INT_ABM = 3      # Adams PECE, 'abm<order><par1>' (input.f90:286-292)
INT_BS = 4       # Bulirsch-Stoer, 'bs' (input.f90:293-294)
INT_CMF2 = 10    # constant mean field (input.f90:295-331)


class ModelError(ValueError):
    """Raised for input the reference would reject with ``stop``."""


# ----------------------------------------------------------------------------
# Primitive DVRs
# ----------------------------------------------------------------------------

def harm_dvr(n: int, x0: float, mw: float, with_trafo: bool = False):
    """Harmonic-oscillator DVR (dvr.f90:263-357).

    Returns grid, weights, d1 (d/dq), d2 (d^2/dq^2), xd1 (x d/dx + d/dx x)
    as float64 arrays, and with_trafo the DVR-to-FBR transformation trafoDVR
    (basis x grid).  Eigenvector signs are fixed by making the first row of the
    transformation non-negative, as the reference does (dvr.f90:287).
    """
    if n < 2:
        raise ModelError("too few grid points selected for a DVR")
    xmat = np.zeros((n, n))
    for i in range(1, n):
        xmat[i - 1, i] = math.sqrt(0.5 * i / mw)
        xmat[i, i - 1] = xmat[i - 1, i]
    grid, trafo = np.linalg.eigh(xmat)
    grid = grid.copy()
    for i in range(1, n // 2 + 1):
        d = 0.5 * (-grid[i - 1] + grid[n - i])
        grid[i - 1] = -d
        grid[n - i] = d
    if n % 2 == 1:
        grid[n // 2] = 0.0
    grid = grid + x0
    for i in range(n):
        if trafo[0, i] < 0.0:
            trafo[:, i] = -trafo[:, i]
    w = trafo[0, :] ** 2 * np.exp(mw * (grid - x0) ** 2) * math.sqrt(math.pi / mw)
    aux = np.zeros((n, n))
    for i in range(1, n):
        aux[i - 1, i] = math.sqrt(i)
        aux[i, i - 1] = -math.sqrt(i)
    aux *= math.sqrt(0.5 * mw)
    d1 = trafo.T @ (aux @ trafo)
    aux = np.zeros((n, n))
    for i in range(1, n - 1):
        aux[i - 1, i + 1] = math.sqrt(i * (i + 1))
        aux[i + 1, i - 1] = -math.sqrt(i * (i + 1))
    xd1 = trafo.T @ (aux @ trafo)
    d1 = 0.5 * (d1 - d1.T)
    xd1 = 0.5 * (xd1 - xd1.T)
    np.fill_diagonal(d1, 0.0)
    np.fill_diagonal(xd1, 0.0)
    aux = np.zeros((n, n))
    for i in range(1, n + 1):
        aux[i - 1, i - 1] = -(2 * i - 1)
    for i in range(1, n - 1):
        aux[i - 1, i + 1] = math.sqrt(i * (i + 1))
        aux[i + 1, i - 1] = aux[i - 1, i + 1]
    d2 = 0.5 * mw * (trafo.T @ (aux @ trafo))
    d2 = np.triu(d2) + np.triu(d2, 1).T
    if with_trafo:
        return grid, w, d1, d2, xd1, trafo
    return grid, w, d1, d2, xd1


@functools.lru_cache(maxsize=256)
def _dvr_cached(kind: str, n: int, a: float, b: float):
    """One DVR per (kind, size, parameters): models and ensemble members that share
    a grid share its construction (callers get copies)."""
    if kind == "Leg":
        return tuple(np.asarray(x) for x in leg_dvr(n, int(a), True))
    f = harm_dvr if kind == "HO" else sin_dvr
    return tuple(np.asarray(x) for x in f(n, a, b, True))


def sin_dvr(n: int, xi: float, xf: float, with_trafo: bool = False):
    """Sine (particle-in-a-box) DVR (dvr.f90:107-186); with_trafo also trafoDVR."""
    if n < 2:
        raise ModelError("too few grid points selected for a DVR")
    dx = (xf - xi) / (n - 1)
    grid = xi + dx * np.arange(n, dtype=np.float64)
    w = np.full(n, dx)
    if abs(abs(xf) - abs(xi)) < np.finfo(float).eps:
        for i in range(1, n // 2 + 1):
            d = 0.5 * (-grid[i - 1] + grid[n - i])
            grid[i - 1] = -d
            grid[n - i] = d
        if n % 2 == 1:
            grid[n // 2] = 0.0
    np1 = float(n + 1)
    ii = np.arange(1, n + 1)
    trafo = np.sin(np.outer(ii, ii) * math.pi / np1) * math.sqrt(2.0 / np1)
    aux = np.zeros((n, n))
    for i in range(1, n + 1):
        for j in range(1, n + 1):
            if i != j:
                aux[i - 1, j - 1] = (abs(i - j) % 2) * i * j / float(i * i - j * j)
    aux1 = (4.0 / (xf - xi)) * (aux @ trafo)
    d1 = trafo @ aux1
    xd1 = d1 * (grid[:, None] + grid[None, :])
    d2 = np.zeros((n, n))
    for i in range(1, n + 1):
        d2[i - 1, i - 1] = (2 * n * n + 4 * n + 3) / 3.0 - 1.0 / math.sin(math.pi * i / np1) ** 2
    ph = 0.5 * math.pi
    for i in range(1, n):
        s = -1.0
        for j in range(i + 1, n + 1):
            d2[i - 1, j - 1] = (1.0 / math.sin(ph * (i - j) / np1) ** 2
                                - 1.0 / math.sin(ph * (i + j) / np1) ** 2) * s
            s = -s
    fac = 0.5 * (math.pi / (xf - xi + 2 * dx)) ** 2
    d2 = -np.triu(d2) * fac
    d2 = d2 + np.triu(d2, 1).T
    if with_trafo:
        return grid, w, d1, d2, xd1, trafo
    return grid, w, d1, d2, xd1


def spline(x: np.ndarray, y: np.ndarray, xx: np.ndarray) -> np.ndarray:
    """Cubic spline of (x, y) evaluated at xx (Spline, maths.f90:651-728).

    On [x_i, x_(i+1)] f(t) = y_i + a_i (t - x_i) + b_i (t - x_i)^2 + c_i (t - x_i)^3;
    the 3(n-1) coefficients solve one dense system (dgesv in the reference,
    LU with partial pivoting here too) made of the passage through y_(i+1), the
    continuity of f' and f'' at the inner points, and c = 0 in the first and
    last interval.  Points left of x_1 use the first interval's (quadratic)
    polynomial, points right of x_(n-1) the last one's.
    """
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    n = len(x)
    if n < 2:
        raise ModelError("an interpolation file needs at least two points")
    N = 3 * n - 3
    M = np.zeros((N, N))
    rhs = np.zeros(N)
    M[0, 2] = 1.0
    ieq, iabc = 1, 0          # 1-based equation counter of the reference, 0-based column offset
    for i in range(n - 2):
        dx = x[i + 1] - x[i]
        M[ieq, iabc:iabc + 3] = (dx, dx ** 2, dx ** 3)
        rhs[ieq] = y[i + 1] - y[i]
        M[ieq + 1, iabc:iabc + 4] = (1.0, 2 * dx, 3 * dx ** 2, -1.0)
        M[ieq + 2, iabc + 1] = 1.0
        M[ieq + 2, iabc + 2] = 3 * dx
        M[ieq + 2, iabc + 4] = -1.0
        ieq += 3
        iabc += 3
    dx = x[n - 1] - x[n - 2]
    M[ieq, iabc:iabc + 3] = (dx, dx ** 2, dx ** 3)
    rhs[ieq] = y[n - 1] - y[n - 2]
    M[ieq + 1, iabc + 2] = 1.0
    coef = np.linalg.solve(M, rhs)
    out = np.empty(len(xx))
    for i, xt in enumerate(np.asarray(xx, dtype=np.float64)):
        j = n - 1                       # 0-based interval; the reference's loop leaves j = n
        for jj in range(n - 1):
            if xt < x[jj + 1]:
                j = jj
                break
        if xt > x[n - 2]:
            j = n - 2
        d = xt - x[j]
        a, b, c = coef[3 * j:3 * j + 3]
        out[i] = y[j] + a * d + b * d ** 2 + c * d ** 3
    return out


def read_xy(path: str) -> Tuple[np.ndarray, np.ndarray]:
    """Two columns (x, f(x)) of a data file, read up to the first line that does
    not hold two numbers (list-directed reads until an error, hamilton.f90:234-246)."""
    xs, ys = [], []
    with open(path) as fh:
        for line in fh:
            toks = line.replace(",", " ").split()
            try:
                xv, yv = _read_float(toks[0]), _read_float(toks[1])
            except (IndexError, ValueError):
                break
            xs.append(xv)
            ys.append(yv)
    return np.array(xs), np.array(ys)


_LEG_WEIGHT = (2.0, 4.0 / 3.0, 16.0 / 15.0, 32.0 / 35.0, 256.0 / 315.0, 512.0 / 693.0, 2048.0 / 3003.0,
               4096.0 / 6435.0, 65536.0 / 109395.0, 131072.0 / 230945.0, 524288.0 / 969969.0)
_LEG_NXL = 3001   # grid of the 1/sin(theta) quadrature for M = 0 (dvr.f90:371)


def _sym_grid(g: np.ndarray) -> np.ndarray:
    """Symmetrise an angular grid about pi/2 (dvr.f90:389-395)."""
    g = g.copy()
    n = len(g)
    for i in range(n // 2):
        d = 0.5 * (g[i] + math.pi - g[n - 1 - i])
        g[i] = d
        g[n - 1 - i] = math.pi - d
    if n % 2 == 1:
        g[n // 2] = 0.5 * math.pi
    return g


@functools.lru_cache(maxsize=8)
def _leg_sinm1_xl():
    """1/sin(theta) of the 3001-point Legendre grid with its eigenvectors (M = 0)."""
    n = _LEG_NXL
    T = np.zeros((n, n))
    i = np.arange(1, n)
    T[i - 1, i] = i / np.sqrt(4.0 * i ** 2 - 1.0)
    w, U = np.linalg.eigh(T + T.T)
    g = _sym_grid(np.arccos(np.clip(w, -1.0, 1.0)))
    return 1.0 / np.sin(g), U


def leg_dvr(nP: int, MM: int, with_trafo: bool = False):
    """Legendre DVR in theta for the associated Legendre functions of order MM
    (Leg_DVR, dvr.f90:361-530): grid, weights, d1 (d/dtheta sin theta),
    d2 (the L0^2 operator, L^2 - M^2 sin^-2), the sin^-2 matrix and trafoDVR."""
    if MM > 10:
        raise ModelError("Leg DVR implemented only for M <= 10")
    if nP < 2:
        raise ModelError("too few grid points selected for a DVR")
    i = np.arange(1, nP)
    T = np.zeros((nP, nP))
    T[i - 1, i] = np.sqrt(((MM + i) ** 2 - MM ** 2) / (4.0 * (MM + i) ** 2 - 1.0))
    w, trafo = np.linalg.eigh(T + T.T)
    grid = _sym_grid(np.arccos(np.clip(w, -1.0, 1.0)))
    trafo = trafo * np.where(trafo[0, :] < 0.0, -1.0, 1.0)[None, :]
    wts = (trafo[0, :] / np.sin(grid) ** MM) ** 2 * _LEG_WEIGHT[MM]
    aux = np.zeros((nP, nP))
    v = np.sqrt(((MM + i) ** 4 - (MM + i) ** 2 * MM ** 2) / (4.0 * (MM + i) ** 2 - 1.0))
    aux[i - 1, i] = v
    aux[i, i - 1] = -v
    d1 = trafo.T @ (aux @ trafo)
    d1 = 0.5 * (d1 - d1.T)
    np.fill_diagonal(d1, 0.0)
    if MM == 0:
        sinv, U = _leg_sinm1_xl()
        Uk = U[:nP, :]
        s1 = (Uk * sinv[None, :]) @ Uk.T
        s1 = np.triu(s1) + np.triu(s1, 1).T
        aux1 = s1 @ trafo
        s1 = 0.5 * (trafo.T @ aux1 + aux1.T @ trafo)
        s1 = np.triu(s1) + np.triu(s1, 1).T
        sinm2 = s1 @ s1.T
        sinm2 = np.triu(sinm2) + np.triu(sinm2, 1).T
    else:
        aux = np.zeros((nP, nP))
        for a in range(1, nP + 1):
            li = a - 1 + MM
            idm = 1
            for k in range(2 * MM):
                idm *= (li + MM - k)
            for b in range(a, nP + 1, 2):
                lj = b - 1 + MM
                jdm = 1
                for k in range(2 * MM):
                    jdm *= (lj + MM - k)
                aux[a - 1, b - 1] = math.sqrt((2 * li + 1) * (2 * lj + 1)) / (2 * MM) * math.sqrt(idm / jdm)
        aux = np.triu(aux) + np.triu(aux, 1).T
        aux1 = aux @ trafo
        sinm2 = 0.5 * (trafo.T @ aux1 + aux1.T @ trafo)
        sinm2 = np.triu(sinm2) + np.triu(sinm2, 1).T
    ll = (MM + np.arange(1, nP + 1)) ** 2 - (MM + np.arange(1, nP + 1))
    aux1 = ll[:, None] * trafo
    d2 = 0.5 * (trafo.T @ aux1 + aux1.T @ trafo) - float(MM) ** 2 * sinm2
    d2 = np.triu(d2) + np.triu(d2, 1).T
    xd1 = np.zeros((nP, nP))
    if with_trafo:
        return grid, wts, d1, d2, xd1, trafo, sinm2
    return grid, wts, d1, d2, xd1, sinm2


def associated_legendre(L: int, M: int, theta: np.ndarray) -> np.ndarray:
    """Normalised associated Legendre functions for L <= 2 (AssociatedLegendreP,
    maths.f90:734-775)."""
    if abs(M) > L:
        raise ModelError("requested a Legendre function with M > L")
    th = np.asarray(theta, dtype=np.float64)
    if L == 0:
        return np.full_like(th, math.sqrt(0.5))
    if L == 1:
        if M == 0:
            return math.sqrt(1.5) * np.cos(th)
        return -math.copysign(1.0, M) * math.sqrt(0.75) * np.sin(th)
    if L == 2:
        if M == 0:
            return math.sqrt(0.15625) * (1.0 + 3.0 * np.cos(2.0 * th))
        if abs(M) == 1:
            return -math.copysign(1.0, M) * math.sqrt(0.9375) * np.sin(2.0 * th)
        return math.sqrt(0.9375) * np.sin(th) ** 2
    raise ModelError(f"Associated Legendre function not implemented for L,M = {L} {M}")


# ----------------------------------------------------------------------------
# Model description
# ----------------------------------------------------------------------------

@dataclasses.dataclass
class Term:
    """One Hamiltonian term ae * |lhs><rhs| * prod_k op_k (input.f90:812-1144)."""
    coeff: complex
    lhs: int                   # 0-based electronic state
    rhs: int
    dof_ops: Dict[int, int]    # 0-based dof -> primitive operator code


@dataclasses.dataclass
class Model:
    """The state of the reference's global modules after set-up."""
    nstates: int
    mode_dofs: List[List[int]]              # iDOF (0-based dofs per mode)
    multiset: List[bool]                    # MultiSet
    nspf: np.ndarray                        # (nmodes, nstates) int64
    dvr_type: List[str]                     # per dof: 'HO', 'sin', 'Leg', 'gwp'
    ngp: List[int]                          # per dof
    dvrpar: List[Tuple[float, float]]       # per dof
    terms: List[Term]
    # propagation parameters (globals.f90)
    tinit: float = 0.0                      # a.u.
    tfinal: float = 100.0 / AU2FS
    tout: float = 1.0 / AU2FS               # writetime
    eps_int: float = 1e-8
    eps_rho: float = 1e-8
    eps_ovl: float = 1e-8                   # eps_S
    eps_C: float = 1e-8
    eps_A: float = 1e-8
    eps_psi: float = 1e-8
    min_stepsize: float = 1e-9 / AU2FS
    int_type: int = INT_RK45
    int_order: int = 4                      # Adams PECE order (input.f90:75, 299)
    int_par1: int = 0                       # extra EC iterations of Adams (input.f90:300-304)
    int_type_A: int = 5                     # Lanczos
    int_type_psi: int = 1                   # rk45 (Cash-Karp) for the SPFs
    relaxation: bool = False
    inorm_psi: int = 0
    init_state: int = 0                     # populated electronic state (0-based)
    init_spf: Dict[int, Tuple[str, tuple]] = dataclasses.field(default_factory=dict)
    label: str = "model"
    # operators whose expectation values are written (the 'expect' keyword, input.f90:196-216)
    expect: List[List[Term]] = dataclasses.field(default_factory=list)
    # statistical mixtures (the 'npackets' and 'eps_pop' keywords, input.f90:156, 262)
    npackets: int = 1
    eps_pop: float = 1e-6
    # dissipative operators (the 'dissipation' keyword, input.f90:216-229, 596-616):
    # (type 1 or 2, global coefficient as read, terms); type 1 is alpha V rho V^+
    # with aeD1 = alpha / 2, type 2 is beta (W rho + rho W^+) with aeD2 = beta
    dissipation: List[Tuple[int, float, List[Term]]] = dataclasses.field(default_factory=list)
    # explicit mixture states of the INIT-WF 'packets' block (init_calc.f90:527-540):
    # (state, 0-based SPF index per mode, coefficient) per packet
    init_packets: Optional[List[Tuple[int, Tuple[int, ...], complex]]] = None
    # parametrised operators (OpParam, OpParamFunc; input.f90:950-1072): (function,
    # p1, p2, p3, data file) for operator j = index + 1 of the codes 200 + j / -200 - j
    op_params: List[Tuple[int, float, float, float, str]] = dataclasses.field(default_factory=list)
    # contents (x, f(x)) of the data files the parametrised operators name
    interp_data: Dict[str, Tuple[np.ndarray, np.ndarray]] = dataclasses.field(default_factory=dict)
    # Gaussian lattice indices read from gwpgrid_<mode> (distribution 1,
    # init_calc.f90:1048-1060): 0-based mode -> (ndof of the mode, nS) int array
    gwp_grid: Dict[int, np.ndarray] = dataclasses.field(default_factory=dict)

    # ---- derived (filled by finalize) ----
    def finalize(self) -> "Model":
        self.nmodes = len(self.mode_dofs)
        self.ndof = len(self.dvr_type)
        self.nspf = np.asarray(self.nspf, dtype=np.int64).reshape(self.nmodes, self.nstates)
        for m in range(self.nmodes):
            if not self.multiset[m]:
                self.nspf[m, :] = self.nspf[m, 0]
        self.is_gwp_mode = [self.dvr_type[self.mode_dofs[m][0]] == "gwp" for m in range(self.nmodes)]
        for m in range(self.nmodes):
            kinds = {self.dvr_type[d] == "gwp" for d in self.mode_dofs[m]}
            if len(kinds) != 1:
                raise ModelError(f"mode {m + 1} mixes dvr and gwp representations")
        self.modes_dvr = [m for m in range(self.nmodes) if not self.is_gwp_mode[m]]
        self.modes_gwp = [m for m in range(self.nmodes) if self.is_gwp_mode[m]]
        self.der_factor = complex(-1.0, 0.0) if self.relaxation else complex(0.0, -1.0)
        self._build_dvr()
        self._build_param_ops()
        self._build_operators()
        self._build_layout()
        return self

    # init_calc.f90:97-123 (DVR matrices), :126-133 (ngpm)
    def _build_dvr(self):
        self.grid: Dict[int, np.ndarray] = {}
        self.wgrid: Dict[int, np.ndarray] = {}
        self.d1: Dict[int, np.ndarray] = {}
        self.d2: Dict[int, np.ndarray] = {}
        self.xd1: Dict[int, np.ndarray] = {}
        self.trafo: Dict[int, np.ndarray] = {}     # trafoDVR (basis x grid)
        self.oper_dvr: Dict[int, np.ndarray] = {}  # operDVR (sin^-2 of Legendre DVRs)
        for d in range(self.ndof):
            t = self.dvr_type[d]
            if t in ("HO", "sin"):
                g, w, d1, d2, xd1, tr = (np.array(x) for x in _dvr_cached(t, self.ngp[d], float(self.dvrpar[d][0]),
                                                                            float(self.dvrpar[d][1])))
            elif t == "Leg":
                g, w, d1, d2, xd1, tr, sm2 = (np.array(x) for x in _dvr_cached(t, self.ngp[d],
                                                                                 float(self.dvrpar[d][0]), 0.0))
                self.oper_dvr[d] = sm2
            elif t == "gwp":
                continue
            else:
                raise ModelError(f"DVR type {t!r} is not supported by this core")
            self.grid[d], self.wgrid[d], self.d1[d], self.d2[d], self.xd1[d] = g, w, d1, d2, xd1
            self.trafo[d] = tr
        self.ngpm = {}
        for m in self.modes_dvr:
            self.ngpm[m] = int(np.prod([self.ngp[d] for d in self.mode_dofs[m]]))

    # hamilton.f90:210-290: values of the parametrised operators on the grids of
    # the DVR dofs that use them
    def _build_param_ops(self):
        self.grid_oper: Dict[Tuple[int, int], np.ndarray] = {}
        used = set()
        for op in [self.terms] + self.expect + [d[2] for d in self.dissipation]:
            for term in op:
                for d, c in term.dof_ops.items():
                    if c > OP_PARAM or c <= -OP_PARAM:
                        used.add((d, abs(c) - OP_PARAM))
        for (d, j) in sorted(used):
            if j < 1 or j > len(self.op_params):
                raise ModelError(f"parametrised operator {j} on dof {d + 1} is not declared")
            if self.dvr_type[d] == "gwp":
                raise ModelError(f"parametrised operators act on DVR dofs only (dof {d + 1})")
            func, p1, p2, p3, fname = self.op_params[j - 1]
            x = self.grid[d]
            if func == PAR_GAU:
                v = np.exp(p1 * x + p2 * x ** 2)
            elif func == PAR_INTERP:
                v = spline(*self.interp_data[fname], x)
            elif func == PAR_SQUARE:
                v = np.where(np.abs(x - p1) < 0.5 * p2, 1.0, 0.0)
            elif func == PAR_HERMITE:
                v = x ** int(p3) * np.exp(p1 * x + p2 * x ** 2)
            elif func == PAR_SIN:
                v = np.sin(p1 * x) ** p2
            elif func == PAR_COS:
                v = np.cos(p1 * x) ** p2
            elif func == PAR_EIGPROJ:
                # Eigenf1DPot_real (dvr.f90:600-650): eigenvector p3 of -p2 d2DVR + V
                V = spline(*self.interp_data[fname], x)
                H = -p2 * self.d2[d] + np.diag(V)
                _, U = np.linalg.eigh(H)
                v = U[:, int(p3)].copy()
            else:
                raise ModelError(f"unknown parametrised operator function {func}")
            self.grid_oper[(d, j)] = np.asarray(v, dtype=np.float64)

    # hamilton.f90:91-167 (operator dedup, the extra operators after the
    # Hamiltonian's), :353-374 (IsIdentity), :377-399 (SkipTerm)
    def _build_operators(self):
        nham = len(self.terms)
        self.nham = nham
        self.iopdof = np.zeros((self.ndof, nham), dtype=np.int64)
        for t, term in enumerate(self.terms):
            for d, op in term.dof_ops.items():
                self.iopdof[d, t] = op
        self.oper: List[List[Tuple[int, int, Tuple[int, ...]]]] = []
        self.ioper = np.zeros((self.nmodes, nham), dtype=np.int64)
        # iOperExtra: (nmodes, nterms) per expectation operator
        self.ioper_expect = [np.zeros((self.nmodes, len(op)), dtype=np.int64) for op in self.expect]
        self.ioper_diss = [np.zeros((self.nmodes, len(d[2])), dtype=np.int64) for d in self.dissipation]

        def vec_of(m, term):
            el = (term.lhs, term.rhs) if self.multiset[m] else (0, 0)
            return (el[0], el[1], tuple(int(term.dof_ops.get(d, 0)) for d in self.mode_dofs[m]))

        for m in range(self.nmodes):
            ops: List[Tuple[int, int, Tuple[int, ...]]] = []

            def index_of(vec):
                try:
                    return ops.index(vec)
                except ValueError:
                    ops.append(vec)
                    return len(ops) - 1

            for t, term in enumerate(self.terms):
                self.ioper[m, t] = index_of(vec_of(m, term))
            for i, op in enumerate(self.expect):
                for t, term in enumerate(op):
                    self.ioper_expect[i][m, t] = index_of(vec_of(m, term))
            for i, (_, _, dterms) in enumerate(self.dissipation):
                for t, term in enumerate(dterms):
                    self.ioper_diss[i][m, t] = index_of(vec_of(m, term))
            self.oper.append(ops)
        self.nopermax = max(len(o) for o in self.oper)
        self.is_identity = np.zeros((self.nmodes, self.nopermax), dtype=bool)
        for m in range(self.nmodes):
            for k, (l, r, dops) in enumerate(self.oper[m]):
                if l == r and all(o == 0 for o in dops):
                    self.is_identity[m, k] = True
        self.skip_term = np.zeros((self.nmodes, nham), dtype=bool)
        for t in range(nham):
            for m in range(self.nmodes):
                if (not self.is_gwp_mode[m]) and self.is_identity[m, self.ioper[m, t]]:
                    self.skip_term[m, t] = True
        # SkipTerm of the dissipative terms: the identity on a DVR mode is not applied
        # (gmctdh_objects.f90:632, 773)
        self.skip_diss = []
        for i, (_, _, dterms) in enumerate(self.dissipation):
            sk = np.zeros((self.nmodes, len(dterms)), dtype=bool)
            for t in range(len(dterms)):
                for m in range(self.nmodes):
                    sk[m, t] = (not self.is_gwp_mode[m]) and self.is_identity[m, self.ioper_diss[i][m, t]]
            self.skip_diss.append(sk)
        self.aeD1 = [0.5 * c for (ty, c, _) in self.dissipation if ty == 1]   # input.f90:607
        self.aeD2 = [c for (ty, c, _) in self.dissipation if ty == 2]         # input.f90:612
        self.diss1 = [i for i, d in enumerate(self.dissipation) if d[0] == 1]
        self.diss2 = [i for i, d in enumerate(self.dissipation) if d[0] == 2]
        for ty, _, dterms in self.dissipation:
            if ty not in (1, 2):
                raise ModelError(f"dissipation type {ty} is not supported (1: V rho V^+, 2: W rho + rho W^+)")
            for term in dterms:
                # between two states the reference adds the (nSPF(rhs) x nSPF(lhs)) contraction
                # into the operator's (lhs x rhs) mean field (gmctdh_objects.f90:726-741):
                # defined for equal SPF counts on the multi-set modes
                if ty == 1 and term.lhs != term.rhs and any(
                        self.multiset[m] and self.nspf[m, term.lhs] != self.nspf[m, term.rhs]
                        for m in range(self.nmodes)):
                    raise ModelError("type-1 terms between states need equal SPF counts in both states")
        if self.npackets < 1:
            raise ModelError("npackets must be at least 1")
        self.ae = np.array([term.coeff for term in self.terms], dtype=np.complex128)
        self.lhs_el = np.array([term.lhs for term in self.terms], dtype=np.int64)
        self.rhs_el = np.array([term.rhs for term in self.terms], dtype=np.int64)
        codes = {d: set(int(c) for c in self.iopdof[d]) for d in range(self.ndof)}
        for op in self.expect + [d[2] for d in self.dissipation]:
            for term in op:
                for d, c in term.dof_ops.items():
                    codes[d].add(int(c))
        for d in range(self.ndof):
            if self.dvr_type[d] == "gwp":
                continue
            for code in codes[d]:
                if code in (OP_ID, OP_P, OP_DQ2, OP_QP) or 1 <= code <= 20:
                    continue
                if code > OP_PARAM or code <= -OP_PARAM:
                    continue
                if code == OP_SINM2 and self.dvr_type[d] == "Leg":
                    continue
                raise ModelError(f"primitive operator code {code} on dof {d + 1} is not supported")

    # init_calc.f90:22-53 (nAConf, AStateOffset), :160-181 (ipsiSPF, dimPsi)
    def _build_layout(self):
        self.naconf = np.array([int(np.prod(self.nspf[:, s])) for s in range(self.nstates)], dtype=np.int64)
        self.astate_offset = np.zeros(self.nstates, dtype=np.int64)
        off = 0
        for s in range(self.nstates):
            self.astate_offset[s] = off
            off += int(self.naconf[s])
        self.naconftot = off
        self.ipsispf = np.zeros((self.nmodes, self.nstates), dtype=np.int64)
        dim = 0
        for s in range(self.nstates):
            for m in range(self.nmodes):
                if (not self.multiset[m]) and s > 0:
                    self.ipsispf[m, s] = self.ipsispf[m, 0]
                    continue
                self.ipsispf[m, s] = dim
                if self.is_gwp_mode[m]:
                    dim += len(self.mode_dofs[m]) * int(self.nspf[m, s])
                else:
                    dim += self.ngpm[m] * int(self.nspf[m, s])
        self.dimpsi = dim
        self.nspfmax = int(self.nspf.max())
        self.ns00max = int(max([self.nspf[m, :].max() for m in self.modes_gwp], default=0))

    # ---- helpers ----
    def a_state(self, A: np.ndarray, s: int) -> np.ndarray:
        """View of state s's coefficient tensor, shape nspf[:, s], Fortran order."""
        o = int(self.astate_offset[s])
        return A[o:o + int(self.naconf[s])].reshape(tuple(int(x) for x in self.nspf[:, s]), order="F")

    def spf_block(self, psi: np.ndarray, m: int, s: int) -> np.ndarray:
        """SPF block of DVR mode m, state s: (G, n) Fortran-ordered view."""
        o = int(self.ipsispf[m, s])
        n = int(self.nspf[m, s])
        if self.is_gwp_mode[m]:
            nd = len(self.mode_dofs[m])
            return psi[o:o + nd * n].reshape((nd, n), order="F")
        G = self.ngpm[m]
        return psi[o:o + G * n].reshape((G, n), order="F")

    def dof_op_matrix(self, d: int, code: int) -> Tuple[str, np.ndarray]:
        """('dense', M) or ('diag', v) for primitive operator ``code`` on DVR dof d.

        Dense matrices are applied from the right by MultTens (hamilton.f90:577-602)
        as psi(.., g, ..) <- sum_g' psi(.., g', ..) M(g', g); p and qp carry the
        +i factor of hamilton.f90:455-461.
        """
        if code == OP_P:
            return "dense", 1j * self.d1[d]
        if code == OP_DQ2:
            return "dense", self.d2[d].astype(np.complex128)
        if code == OP_QP:
            return "dense", 1j * self.xd1[d]
        if 1 <= code <= 20:
            return "diag", self.grid[d] ** code
        if code > OP_PARAM:
            return "diag", self.grid_oper[(d, code - OP_PARAM)]
        if code <= -OP_PARAM:
            # MultTensProj builds AM = v v^T (dger) and applies it like MultTens
            v = self.grid_oper[(d, -code - OP_PARAM)]
            return "dense", np.outer(v, v).astype(np.complex128)
        if code == OP_SINM2 and d in self.oper_dvr:
            return "dense", self.oper_dvr[d].astype(np.complex128)
        raise ModelError(f"operator code {code} not supported on a DVR dof")


def _plain(v):
    """v with NumPy arrays and scalars replaced by Python lists and numbers."""
    if isinstance(v, np.ndarray):
        return _plain(v.tolist())
    if isinstance(v, np.generic):
        return v.item()
    if isinstance(v, dict):
        return {_plain(k): _plain(x) for k, x in v.items()}
    if isinstance(v, (list, tuple)):
        return type(v)(_plain(x) for x in v)
    return v


def model_fields(model: Model) -> Dict:
    """The constructor fields of a model (what an input file declares), as plain
    Python values (no NumPy objects, so any NumPy version reads them back):
    ``model_from_fields`` rebuilds the same model."""
    out = {}
    for f in dataclasses.fields(Model):
        v = getattr(model, f.name)
        if f.name in ("terms",):
            v = [(complex(t.coeff), int(t.lhs), int(t.rhs), dict(t.dof_ops)) for t in v]
        elif f.name == "expect":
            v = [[(complex(t.coeff), int(t.lhs), int(t.rhs), dict(t.dof_ops)) for t in op] for op in v]
        elif f.name == "dissipation":
            v = [(ty, c, [(complex(t.coeff), int(t.lhs), int(t.rhs), dict(t.dof_ops)) for t in op])
                 for (ty, c, op) in v]
        out[f.name] = _plain(v)
    return out


def model_from_fields(d: Dict) -> Model:
    """Inverse of ``model_fields``: a finalised model."""
    d = dict(d)
    d["terms"] = [Term(*t) for t in d["terms"]]
    d["expect"] = [[Term(*t) for t in op] for op in d.get("expect", [])]
    d["dissipation"] = [(ty, c, [Term(*t) for t in op]) for (ty, c, op) in d.get("dissipation", [])]
    return Model(**d).finalize()


# ----------------------------------------------------------------------------
# Initial wavefunction (init_calc.f90:230-761 single-conf, SetSPF :763-1068)
# ----------------------------------------------------------------------------

def initial_wavefunction(model: Model) -> Tuple[np.ndarray, np.ndarray]:
    """Single-configuration initial state: A = e_1 on ``init_state`` and SPFs
    built by SetSPF (DVR: product Gaussian, then q-multiplied virtual SPFs,
    Gram-Schmidt + QR; GWP: lattice of Gaussians).  Returns (A, psi) with the
    normalisation of init_calc.f90:208-221 applied."""
    psi = np.zeros(model.dimpsi, dtype=np.complex128)
    phi: Dict[int, np.ndarray] = {}
    gwp_par: Dict[int, tuple] = {}
    for d in range(model.ndof):
        kind, par = model.init_spf.get(d, ("gauss", (0.0, 0.0, 0.707107)))
        if kind == "gauss":
            if model.dvr_type[d] == "gwp":
                raise ModelError('Input Error: use "gwp" instead of "gauss"')
            x0, p0, dx = par
            g, w = model.grid[d], model.wgrid[d]
            n = len(g)
            f = np.zeros(n, dtype=np.complex128)
            eps = np.finfo(float).eps
            if abs(x0) < eps and abs(p0) < eps:
                for j in range(n // 2 + 1):
                    f[j] = math.exp(-(0.5 * g[j] / dx) ** 2) * math.sqrt(w[j])
                    f[n - j - 1] = f[j]
            else:
                xx = g - x0
                f = np.exp(-(0.5 * xx / dx) ** 2 + 1j * p0 * xx) * np.sqrt(w)
            phi[d] = f
        elif kind == "gwp":
            if model.dvr_type[d] != "gwp":
                raise ModelError('gwp initial SPFs are allowed only for "gwp representation"')
            dist, x0, p0, dx, ovl, scw = par
            gwp_par[d] = (dist, dx, ovl, scw)
            eps = np.finfo(float).eps
            phi[d] = np.array([0.0 if max(abs(x0), abs(p0)) < eps else complex(0.5 * x0 / dx ** 2, p0)],
                              dtype=np.complex128)
        elif kind == "Leg":
            # associated Legendre function times the square root of the weights
            # (init_calc.f90:578-592)
            if model.dvr_type[d] != "Leg":
                raise ModelError("Input Error: Legendre functions available only for Leg-DVR")
            LL, MM = par
            phi[d] = (associated_legendre(int(LL), int(MM), model.grid[d])
                      * np.sqrt(model.wgrid[d])).astype(np.complex128)
        else:
            raise ModelError(f"initial SPF kind {kind!r} not supported")
    # DVR modes
    for m in model.modes_dvr:
        dofs = model.mode_dofs[m]
        nmd = len(dofs)
        G = model.ngpm[m]
        ns = int(model.nspf[m, :].max())
        shape = tuple(model.ngp[d] for d in dofs)
        prod = np.ones(shape, dtype=np.complex128)
        for k, d in enumerate(dofs):
            sh = [1] * nmd
            sh[k] = model.ngp[d]
            prod = prod * phi[d].reshape(sh)
        psi_t = np.zeros((G, ns), dtype=np.complex128)
        psi_t[:, 0] = prod.reshape(-1, order="F")
        psi_t[:, 0] /= np.linalg.norm(psi_t[:, 0])
        kg = 0
        jj = 1
        for j in range(2, ns + 1):
            jj += 1
            kg = kg % nmd + 1
            l = (jj - 2) // nmd + 1
            col = psi_t[:, l - 1].reshape(shape, order="F").copy()
            d = dofs[kg - 1]
            sh = [1] * nmd
            sh[kg - 1] = model.ngp[d]
            col = col * model.grid[d].reshape(sh)
            psi_t[:, j - 1] = col.reshape(-1, order="F")
        for j in range(1, ns):
            c = -np.vdot(psi_t[:, 0], psi_t[:, j])
            psi_t[:, j] += c * psi_t[:, 0]
        if ns > 1:
            q, _ = np.linalg.qr(psi_t[:, 1:ns], mode="reduced")
            psi_t[:, 1:ns] = q
        for s in range(model.nstates):
            if (not model.multiset[m]) and s > 0:
                continue
            o = int(model.ipsispf[m, s])
            n = int(model.nspf[m, s])
            psi[o:o + G * n] = psi_t[:, :n].reshape(-1, order="F")
    # GWP modes
    model.gwpa = np.zeros((max([len(model.mode_dofs[m]) for m in model.modes_gwp], default=0),
                           max(model.ns00max, 1), len(model.modes_gwp)))
    for i, m in enumerate(model.modes_gwp):
        dofs = model.mode_dofs[m]
        nmd = len(dofs)
        nsm = model.nspfmax
        xi_values = np.zeros((2 * nsm + 1, nmd), dtype=np.complex128)
        w_values = np.zeros((2 * nsm + 1, nmd))
        for j, d in enumerate(dofs):
            dist, dx, ovl, scw = gwp_par[d]
            for l in range(-nsm, nsm + 1):
                w_values[l + nsm, j] = dx * scw ** abs(l)
            xi_values[nsm, j] = 0.0
            for l in range(1, nsm + 1):
                dd = -math.log(ovl) + 0.5 * math.log(2 * scw / (1.0 + scw ** 2))
                dd = dd * (1.0 + scw ** 2) / w_values[l - 1 + nsm, j] ** 2
                dd = (xi_values[l - 1 + nsm, j].real + math.sqrt(dd)) / scw ** 2
                xi_values[l + nsm, j] = dd
                xi_values[-l + nsm, j] = -dd
            if abs(phi[d][0]) > np.finfo(float).eps:
                xi_values[:, j] += phi[d][0]
        dists = {gwp_par[d][0] for d in dofs}
        if len(dists) != 1:
            raise ModelError("the same GWP distribution must be used for all dofs of a mode")
        ns = int(model.nspf[m, :].max())
        index_lat = np.zeros((nmd, ns), dtype=np.int64)
        dist = dists.pop()
        if ns > 1 and dist == 1:
            # distribution read from gwpgrid_<mode> (init_calc.f90:1048-1060)
            if m not in model.gwp_grid:
                raise ModelError(f"INPUT ERROR: Gaussian grid file gwpgrid_{m + 1} not found")
            index_lat[:, :] = np.asarray(model.gwp_grid[m], dtype=np.int64)[:nmd, :ns]
        elif ns > 1:
            if dist != 0:
                raise ModelError(f"Unknown distribution type: {dist}")
            i1, i2, l = 1, 1, 2
            done = False
            while not done:
                for i3 in range(i1, i2 + 1):
                    for j in range(nmd):
                        for i4 in (-1, 1):
                            cand = index_lat[:, i3 - 1].copy()
                            cand[j] += i4
                            if any(np.array_equal(cand, index_lat[:, j1]) for j1 in range(l - 1)):
                                continue
                            index_lat[:, l - 1] = cand
                            l += 1
                            if l > ns:
                                done = True
                                break
                        if done:
                            break
                    if done:
                        break
                i1 = i2 + 1
                i2 = l - 1
        psi_t = np.zeros((nmd, ns), dtype=np.complex128)
        for l in range(ns):
            for j in range(nmd):
                psi_t[j, l] = xi_values[index_lat[j, l] + nsm, j]
                model.gwpa[j, l, i] = -(0.5 / w_values[index_lat[j, l] + nsm, j]) ** 2
        for s in range(model.nstates):
            if (not model.multiset[m]) and s > 0:
                continue
            o = int(model.ipsispf[m, s])
            n = int(model.nspf[m, s])
            psi[o:o + nmd * n] = psi_t[:, :n].reshape(-1, order="F")
    return initial_coefficients(model, psi), psi


def gaussian_overlap(a1: np.ndarray, a2: np.ndarray, xi1: np.ndarray, xi2: np.ndarray) -> complex:
    """<g1|g2> of normalised multi-dimensional Gaussians g = N exp(sum_k a_k x_k^2 + xi_k x_k)
    with real widths a < 0 (GauOvlMultiD, gmctdh_objects.f90:1497-1519): per dimension
    the Gaussian integral exp((conj(xi1) + xi2)^2 / (-4 (a1 + a2))) times the norms."""
    c = np.sum(xi1.real ** 2 / a1 + xi2.real ** 2 / a2 - (np.conj(xi1) + xi2) ** 2 / (a1 + a2))
    d = math.sqrt(float(np.prod(4.0 * a1 * a2 / (a1 + a2) ** 2)))
    return complex(np.exp(0.25 * c) * math.sqrt(d))


def spf_overlap(model: Model, psi: np.ndarray, m: int, s: int) -> np.ndarray:
    """phi^H phi of the SPFs of mode m, state s: grid SPFs by their columns,
    Gaussian SPFs by gaussian_overlap of their parameters (widths model.gwpa)."""
    blk = model.spf_block(psi, m, s)
    if not model.is_gwp_mode[m]:
        return blk.conj().T @ blk
    i = model.modes_gwp.index(m)
    nmd, ns = blk.shape
    a = model.gwpa[:nmd, :ns, i]
    S = np.eye(ns, dtype=np.complex128)
    for j1 in range(ns):
        for j2 in range(ns):
            if j1 != j2:
                S[j1, j2] = gaussian_overlap(a[:, j1], a[:, j2], blk[:, j1], blk[:, j2])
    return S


def initial_coefficients(model: Model, psi: np.ndarray) -> np.ndarray:
    """Coefficients of the initial mixture, packet-major (APacketOffset(W) =
    W * nAConftot).  'el' line (init_calc.f90:490-500): packet W (0-based) has the
    single coefficient 1 (W = 0) or sqrt(eps_pop (W + 1)) on configuration W of the
    initial state; 'packets' block (:527-540): one given coefficient per packet.
    With more than one packet the packets are then rotated into the eigenvectors of
    their overlap matrix (OrthoWP, init_calc.f90:1093-1126, eigenvalues ascending)
    and the mixture is normalised to unit trace (trace_wf, init_calc.f90:212-219)."""
    P = model.npackets
    n = model.naconftot
    A = np.zeros(n * P, dtype=np.complex128)
    if model.init_packets is None:
        s = model.init_state
        o = int(model.astate_offset[s])
        if P > int(model.naconf[s]):
            raise ModelError("the number of wave packets is larger than the configurations of the initial state")
        for W in range(P):
            A[W * n + o + W] = 1.0 if W == 0 else math.sqrt(model.eps_pop * (W + 1))
    else:
        if len(model.init_packets) != P:
            raise ModelError("the 'packets' block needs one line per wave packet")
        for W, (s, jspf, coef) in enumerate(model.init_packets):
            idx, stride = 0, 1
            for m in range(model.nmodes):
                if not 0 <= jspf[m] < int(model.nspf[m, s]):
                    raise ModelError("SPF index of a 'packets' line out of range")
                idx += jspf[m] * stride
                stride *= int(model.nspf[m, s])
            A[W * n + int(model.astate_offset[s]) + idx] = coef
    if P == 1:
        return A
    # <A_i|A_j> = sum_s A_i,s^H (x_m S_m) A_j,s with the SPF overlap matrices S_m
    # (WF_Ovl, gmctdh_objects.f90:101-180)
    Amat = A.reshape((n, P), order="F")
    ovl = np.zeros((P, P), dtype=np.complex128)
    for s in range(model.nstates):
        o, ns = int(model.astate_offset[s]), int(model.naconf[s])
        shape = tuple(int(x) for x in model.nspf[:, s])
        for j in range(P):
            Y = Amat[o:o + ns, j].reshape(shape, order="F")
            for m in range(model.nmodes):
                Y = np.moveaxis(np.tensordot(spf_overlap(model, psi, m, s), Y, axes=([1], [m])), 0, m)
            y = Y.reshape(-1, order="F")
            for i in range(P):
                ovl[i, j] += np.vdot(Amat[o:o + ns, i], y)
    _, V = np.linalg.eigh(ovl, UPLO="U")
    Amat = Amat @ V
    trace = float(np.real(np.trace(V.conj().T @ ovl @ V)))
    return (Amat / math.sqrt(trace)).reshape(-1, order="F")


# ----------------------------------------------------------------------------
# Reader for the reference's keyword input and operator file
# ----------------------------------------------------------------------------

_OPNAMES = {"p": OP_P, "dq^2": OP_DQ2, "qp": OP_QP, "q": 1}


def _first_floats(text: str, count: int, defaults=None) -> List[float]:
    toks = text.replace(",", " ").split()
    if not toks and defaults is not None:
        return list(defaults)
    try:
        return [_read_float(t) for t in toks[:count]] + [0.0] * max(0, count - len(toks))
    except ValueError as exc:
        raise ModelError(f"cannot read the parameters of operator {text!r}") from exc


class OperatorDeclarations:
    """The declaration state shared by every operator file of one input
    (read_declare_ham, input.f90:812-1144, and read_declare_op, :1149-1443):
    the parametrised operators (OpParam, OpParamFunc, nOpParam) and the data
    files they read (strings, nStrings).  Data files are read relative to
    ``base`` and kept in ``interp_data``."""

    def __init__(self, base: str = ".", dvr_type: Optional[Sequence[str]] = None):
        self.base = base
        self.dvr_type = dvr_type
        self.op_params: List[Tuple[int, float, float, float, str]] = []
        self.interp_data: Dict[str, Tuple[np.ndarray, np.ndarray]] = {}

    def _load(self, fname: str):
        if fname not in self.interp_data:
            path = os.path.join(self.base, fname)
            if not os.path.exists(path):
                raise ModelError(f"data file {fname} not found")
            self.interp_data[fname] = read_xy(path)

    def _add(self, func, p1=0.0, p2=0.0, p3=0.0, fname="") -> int:
        self.op_params.append((func, float(p1), float(p2), float(p3), fname))
        return len(self.op_params)

    def _need_leg(self, k: int, what: str):
        if self.dvr_type is not None and self.dvr_type[k] != "Leg":
            raise ModelError(f"ERROR: {what} operator allowed only for Leg-DVR")

    def parse(self, name: str, k: int) -> int:
        """Code of the primitive operator text ``name`` on dof k (0-based).  The
        keyword checks run in the reference's order (input.f90:953-1092)."""
        name = name.strip()
        i = name.find("gau")
        if i >= 0:
            p1, p2 = _first_floats(name[i + 3:], 2)
            return OP_PARAM + self._add(PAR_GAU, p1, p2)
        i = name.find("interp")
        if i >= 0:
            fname = name[i + 6:].strip().split()[0].strip("'\"")
            for j, (func, _, _, _, fn) in enumerate(self.op_params):
                if func == PAR_INTERP and fn == fname:   # the same file is one operator
                    return OP_PARAM + j + 1
            self._load(fname)
            return OP_PARAM + self._add(PAR_INTERP, fname=fname)
        i = name.find("square")
        if i >= 0:
            p1, p2 = _first_floats(name[i + 6:], 2)
            return OP_PARAM + self._add(PAR_SQUARE, p1, p2)
        i = name.find("hermite")
        if i >= 0:
            r, p1, p2 = _first_floats(name[i + 7:], 3)
            return OP_PARAM + self._add(PAR_HERMITE, p1, p2, int(r))
        if "sin^-2" in name:
            self._need_leg(k, "sin^-2")
            return OP_SINM2
        i = name.find("sin")
        if i >= 0:
            p1, p2 = _first_floats(name[i + 3:], 2, defaults=(1.0, 1.0))
            return OP_PARAM + self._add(PAR_SIN, p1, p2)
        i = name.find("cos")
        if i >= 0:
            p1, p2 = _first_floats(name[i + 3:], 2, defaults=(1.0, 1.0))
            return OP_PARAM + self._add(PAR_COS, p1, p2)
        i = name.find("eig_proj")
        if i >= 0:
            toks = name[i + 8:].replace(",", " ").split()
            if len(toks) < 3:
                raise ModelError(f"eig_proj needs a potential file, a kinetic prefactor and a level: {name!r}")
            fname = toks[0].strip("'\"")
            self._load(fname)
            j = self._add(PAR_EIGPROJ, 0.0, _read_float(toks[1]), int(toks[2]), fname)
            return -OP_PARAM - j
        if name == "L0^2":
            self._need_leg(k, "L0^2")
            return OP_DQ2
        if name in _OPNAMES:
            return _OPNAMES[name]
        mm = re.fullmatch(r"q\^(\d+)", name)
        if mm and 1 <= int(mm.group(1)) <= 10:
            return int(mm.group(1))
        raise ModelError(f"Operator {name} not implemented")


def parse_operator_file(text: str, nstates: int, decl: Optional["OperatorDeclarations"] = None) -> List[Term]:
    """Operator grammar of input.f90:812-1144: ``coeff | el-op | k op | k op ...``.

    Supported el-ops: none or ``1`` (one term per state), ``Sa&b`` (one term, or
    two Hermitian-conjugate terms for a != b), ``Za&b``.  Parametrised operators
    are declared in ``decl`` (one per input, shared by all its operator files)."""
    if decl is None:
        decl = OperatorDeclarations()
    terms: List[Term] = []
    for raw in text.splitlines():
        if raw.startswith("----"):
            break
        line = raw.split("#", 1)[0]
        if not line.strip():
            continue
        parts = line.split("|")
        cstr = parts[0].strip()
        cstr_num = cstr.replace("d", "e").replace("D", "e")
        imag = "i" in cstr_num
        coeff = float(cstr_num.replace("i", "")) * (1j if imag else 1.0)
        pairs: List[Tuple[int, int]]
        if len(parts) == 1 or parts[1].strip() == "1":
            pairs = [(s, s) for s in range(nstates)]
        else:
            el = parts[1].strip()
            mm = re.fullmatch(r"([SZ])\s*(\d+)\s*&\s*(\d+)", el)
            if not mm:
                raise ModelError('Only operator labels "1", "Sa&b" or "Za&b" are allowed')
            a, b = int(mm.group(2)) - 1, int(mm.group(3)) - 1
            if mm.group(1) == "S":
                pairs = [(a, b)] if a == b else [(a, b), (b, a)]
            else:
                if a == b:
                    raise ModelError('Electronic operators "Za&b" are allowed only between different states')
                pairs = [(a, b)]
        dof_ops: Dict[int, int] = {}
        for seg in parts[2:]:
            toks = seg.split(None, 1)
            if not toks:
                continue
            k = int(toks[0]) - 1
            opname = toks[1].strip() if len(toks) > 1 else "1"
            if opname == "1":
                continue
            dof_ops[k] = decl.parse(opname, k)
        for (a, b) in pairs:
            terms.append(Term(coeff, a, b, dict(dof_ops)))
    return terms


def _read_float(v: str) -> float:
    return float(v.lower().replace("d", "e"))


def parse_input(path: str) -> Model:
    """Read a reference ``.inp`` file (input.f90:30-426) and its operator file."""
    base = os.path.dirname(os.path.abspath(path))
    with open(path) as fh:
        lines = fh.read().splitlines()
    kw: Dict[str, str] = {}
    spf_lines: List[str] = []
    grid_lines: List[str] = []
    init_lines: List[str] = []
    cmf_lines: List[str] = []
    nstates, ndof, nmodes = 1, -1, 0
    i = 0
    flags = set()
    expect_files: List[str] = []
    diss_files: List[str] = []
    while i < len(lines):
        line = lines[i].split("#", 1)[0]
        i += 1
        s = line.strip()
        if not s:
            continue
        if s == "INIT-WF":
            while i < len(lines):
                l2 = lines[i].split("#", 1)[0]
                i += 1
                if l2.strip() == "END-INIT-WF":
                    break
                if l2.strip():
                    init_lines.append(l2.strip())
            continue
        if "=" in s:
            name, val = s.split("=", 1)
            name, val = name.strip().lower(), val.strip().lower()
        else:
            name, val = s.lower(), "blank"
        if name == "nstates":
            nstates = int(val)
        elif name == "ndof":
            ndof = int(val)
            if ndof > 99:
                raise ModelError("Error: the maximum number of degrees of freedom is 99")
        elif name == "nmodes":
            nmodes = int(val)
        elif name == "spf":
            spf_lines = [lines[i + k].split("#", 1)[0] for k in range(nmodes)]
            i += nmodes
        elif name == "grid":
            grid_lines = [lines[i + k].split("#", 1)[0] for k in range(ndof)]
            i += ndof
        elif name == "integration":
            kw[name] = val
            if val.startswith("cmf2"):
                cmf_lines = [lines[i].split("#", 1)[0], lines[i + 1].split("#", 1)[0]]
                i += 2
        elif name in ("steps", "density", "wp_ovl", "relaxation"):
            flags.add(name)
        elif name in ("hamiltonian", "tinit", "tfinal", "tout", "eps_rho", "eps_c", "eps_int",
                      "eps_s", "eps_pop", "minstep", "normalize", "psi", "npackets"):
            kw[name] = val
        elif name == "expect":
            expect_files.append(val)
        elif name == "dissipation":
            diss_files.append(val)
        elif name == "lcharmbathpt":
            raise ModelError("the perturbative harmonic bath (lcharmbathpt) is not supported by this core")
        elif name == "densmat":
            continue
        else:
            raise ModelError(f"Input instruction: {s} cannot be understood")
    mode_dofs: List[List[int]] = []
    multiset: List[bool] = []
    nspf = np.zeros((nmodes, nstates), dtype=np.int64)
    for m, ln in enumerate(spf_lines):
        lhs, rhs = ln.split("=", 1)
        fields = [f.strip() for f in lhs.split(",")]
        multiset.append(fields[0] != "S")
        mode_dofs.append([int(f) - 1 for f in fields[1:]])
        vals = [int(v) for v in rhs.split(",")]
        for s in range(nstates):
            nspf[m, s] = vals[s] if s < len(vals) else vals[0]
    dvr_type = [""] * ndof
    ngp = [0] * ndof
    dvrpar = [(0.0, 0.0)] * ndof
    for ln in grid_lines:
        toks = ln.split()
        d = int(toks[0]) - 1
        t = toks[1]
        dvr_type[d] = t
        if t == "gwp" and len(toks) == 2:
            ngp[d], dvrpar[d] = 101, (-10.0, 10.0)
        elif t == "Leg":
            # 'k Leg M nP': |M| of the associated Legendre functions, grid points
            # (read_declare_dvr, dvr.f90:58-64)
            dvrpar[d] = (float(abs(int(toks[2]))), 0.0)
            ngp[d] = int(toks[3])
        else:
            ngp[d] = int(toks[2])
            dvrpar[d] = (_read_float(toks[3]), _read_float(toks[4]))
    hfile = kw.get("hamiltonian")
    if not hfile:
        raise ModelError("Input error: Hamiltonian file not given")
    hpath = os.path.join(base, hfile)
    if not os.path.exists(hpath):
        # the reference lower-cases input values (input.f90:145-147)
        raise ModelError(f"Operator file, {hfile} not found")
    decl = OperatorDeclarations(base, dvr_type)
    with open(hpath) as fh:
        terms = parse_operator_file(fh.read(), nstates, decl)
    expect: List[List[Term]] = []
    for ef in expect_files:
        epath = os.path.join(base, ef)
        if not os.path.exists(epath):
            raise ModelError(f"Operator file, {ef} not found")
        with open(epath) as fh:
            expect.append(parse_operator_file(fh.read(), nstates, decl))
    dissipation: List[Tuple[int, float, List[Term]]] = []
    for df in diss_files:
        dpath = os.path.join(base, df)
        if not os.path.exists(dpath):
            raise ModelError(f"Operator file, {df} not found")
        with open(dpath) as fh:
            dtext = fh.read().splitlines()
        # the first line holds the type and the global coefficient (input.f90:221, 602)
        first = 0
        while first < len(dtext) and not dtext[first].split("#", 1)[0].strip():
            first += 1
        if first == len(dtext):
            raise ModelError(f"dissipation file {df} is empty")
        head = dtext[first].split("#", 1)[0].replace(",", " ").split()
        dissipation.append((int(head[0]), _read_float(head[1]),
                            parse_operator_file("\n".join(dtext[first + 1:]), nstates, decl)))
    model = Model(nstates=nstates, mode_dofs=mode_dofs, multiset=multiset, nspf=nspf,
                  dvr_type=dvr_type, ngp=ngp, dvrpar=dvrpar, terms=terms,
                  label=os.path.basename(path), expect=expect, dissipation=dissipation,
                  npackets=int(kw.get("npackets", "1")), op_params=decl.op_params,
                  interp_data=decl.interp_data)
    if "eps_pop" in kw:
        model.eps_pop = _read_float(kw["eps_pop"])
    if "tinit" in kw:
        model.tinit = _read_float(kw["tinit"]) / AU2FS
    if "tfinal" in kw:
        model.tfinal = _read_float(kw["tfinal"]) / AU2FS
    if "tout" in kw:
        model.tout = _read_float(kw["tout"]) / AU2FS
    for k_in, attr in (("eps_rho", "eps_rho"), ("eps_c", "eps_C"), ("eps_int", "eps_int"),
                       ("eps_s", "eps_ovl")):
        if k_in in kw:
            setattr(model, attr, _read_float(kw[k_in]))
    if "minstep" in kw:
        model.min_stepsize = _read_float(kw["minstep"]) / AU2FS
    if "relaxation" in flags:
        model.relaxation = True
        model.inorm_psi = 2
    if "normalize" in kw:
        model.inorm_psi = int(kw["normalize"])
    integ = kw.get("integration", "rk45")
    if integ == "rk45":
        model.int_type = INT_RK45
    elif integ == "dopri":
        model.int_type = INT_DOPRI
    elif integ.startswith("bs"):
        model.int_type = INT_BS
    elif integ.startswith("abm"):
        model.int_type = INT_ABM
        model.int_order = int(integ[3:5])
        model.int_par1 = int(integ[5:]) if integ[5:].strip() else 0
    elif integ.startswith("cmf2"):
        model.int_type = INT_CMF2
        a_name, a_eps = cmf_lines[0].split()[:2]
        p_name, p_eps = cmf_lines[1].split()[:2]
        if a_name.lower() != "lanczos":
            raise ModelError("only Lanczos is supported for the A coefficients in CMF2")
        model.eps_A = _read_float(a_eps)
        model.int_type_psi = {"rk45": 1, "dopri": 2}[p_name.lower()]
        model.eps_psi = _read_float(p_eps)
    else:
        raise ModelError(f"unknown integrator: {integ}")
    # INIT-WF single-conf
    if not init_lines or init_lines[0] != "single-conf":
        raise ModelError("only the single-conf INIT-WF block is supported")
    spf_start = 2
    if init_lines[1].strip().lower() == "packets":
        # one line per packet: state, SPF index per mode, Re, Im (init_calc.f90:527-540)
        packets = []
        for W in range(model.npackets):
            toks = init_lines[2 + W].replace(",", " ").split()
            st = int(toks[0]) - 1
            jspf = tuple(int(v) - 1 for v in toks[1:1 + nmodes])
            cr, ci = _read_float(toks[1 + nmodes]), _read_float(toks[2 + nmodes])
            packets.append((st, jspf, complex(cr, ci)))
        model.init_packets = packets
        model.init_state = packets[0][0]
        spf_start = 2 + model.npackets
    else:
        mm = re.match(r"el\s+(\d+)", init_lines[1])
        if not mm:
            raise ModelError("INIT-WF: expecting 'el <state>' or 'packets'")
        model.init_state = int(mm.group(1)) - 1
    for ln in init_lines[spf_start:]:
        if "gauss" in ln:
            k, rest = ln.split("gauss", 1)
            x0, p0, dx = [_read_float(v) for v in rest.split()[:3]]
            model.init_spf[int(k) - 1] = ("gauss", (x0, p0, dx))
        elif "gwp" in ln:
            k, rest = ln.split("gwp", 1)
            toks = rest.split()
            dist, x0, p0, dx = int(toks[0]), _read_float(toks[1]), _read_float(toks[2]), _read_float(toks[3])
            ovl = 0.7
            scw = 1.0
            mo = re.search(r"ovl\s*=\s*([-+0-9.eEdD]+)", rest)
            if mo:
                ovl = _read_float(mo.group(1))
            ms = re.search(r"scw\s*=\s*([-+0-9.eEdD]+)", rest)
            if ms:
                scw = _read_float(ms.group(1))
            model.init_spf[int(k) - 1] = ("gwp", (dist, x0, p0, dx, ovl, scw))
        elif "Leg" in ln:
            k, rest = ln.split("Leg", 1)
            LL, MM = (int(v) for v in rest.replace(",", " ").split()[:2])
            model.init_spf[int(k) - 1] = ("Leg", (LL, MM))
        else:
            raise ModelError(f"The chosen initial SPF is unknown: {ln}")
    # lattice indices of Gaussian modes placed by distribution 1 (init_calc.f90:1048-1060)
    for m in range(nmodes):
        if dvr_type[mode_dofs[m][0]] != "gwp":
            continue
        dists = {model.init_spf.get(d, ("", (0,)))[1][0] for d in mode_dofs[m]}
        gpath = os.path.join(base, f"gwpgrid_{m + 1}")
        if 1 in dists and os.path.exists(gpath):
            ns = int(nspf[m, :].max())
            rows = []
            with open(gpath) as fh:
                for line in fh:
                    if len(rows) == ns:
                        break
                    if line.strip():
                        rows.append([int(v) for v in line.split()[:len(mode_dofs[m])]])
            model.gwp_grid[m] = np.array(rows, dtype=np.int64).T
    return model.finalize()
