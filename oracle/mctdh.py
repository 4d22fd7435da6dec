"""CPU oracle: a NumPy restatement of the reference's G-MCTDH EOM + integrator path.

TEST INFRASTRUCTURE ONLY.  Nothing in the product imports this module; only
``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg
use it, and only as the checker / CPU reference arm.

PARITY STATUS: unpinned against the reference binary.  The reference is Fortran
(no Fortran compiler exists in this build environment) and ships no tests or
golden outputs, so this restatement is pinned instead against physics
known-answer tests in ``tests/test_oracle.py`` (analytic autocorrelation of a
displaced harmonic oscillator, the exact limit n_SPF = n_grid against direct
propagation, norm and energy conservation, Hermiticity).

Each routine follows the reference routine it names, in FP64, with the same
regularisations and control arithmetic:

  Calc_Derivs      derivatives.f90:39-237
  Calc_MeanField   gmctdh_objects.f90:481-604   (Hamiltonian part, term by term)
  Calc_rho1mode    gmctdh_objects.f90:408-477
  Calc_rhom1MF     gmctdh_objects.f90:1147-1194
  Calc_h1mode      hamilton.f90:416-531, MultTens* :577-661
  StdRegInv/Sol    maths.f90:8-162;  InverseSquareRoot(U) maths.f90:588-644
  Calc_S00/S00m1   gmctdh_objects.f90:323-404;  Calc_CY :1198-1333
  GauInt1D         hamilton.f90:745-849;  Gau10Int1D :853-902;  GauOvlMultiD gmctdh_objects.f90:1497-1519
  norm_wf/WF_Ovl   gmctdh_objects.f90:21-180;  DeltaPsi :206-275
  rkqs/rkck/rkdp   integrator.f90:36-221
  cmf2, A_to_B/B_to_A, propagate_SPF   cmf2_base.f90:47-345
  Lanczos, rk_SPF_ck                    cmf2_integration.f90:30-253
  Calc_DHD_B, Calc_Der_SPF, Calc_Err_SPF cmf2_derivatives.f90:1-338;  Calc_DHD hamilton.f90:535-574
  propagate_wf     propagator.f90:87-146, :257-306;  observables output.f90:35-87, :144-150

The reference works on complex-conjugated coefficient vectors so that BLAS
right-multiplications give the wanted left mode products (e.g.
gmctdh_objects.f90:531-532, :544).  The restatement uses the equivalent
left mode products on the unconjugated tensors; every conjugation pair of the
reference cancels exactly, so the arithmetic is the same up to rounding.
"""
from __future__ import annotations

import math
from typing import Dict, List, Optional, Tuple

import numpy as np

from macaw_gb300.model import Model, AU2FS, INT_RK45, INT_DOPRI, INT_ABM, INT_BS, INT_CMF2

_EPS = np.finfo(np.float64).eps

# Cash-Karp tableau (integrator.f90:107-121, cmf2_integration.f90:122-133)
CK = dict(
    A=(0.0, 0.2, 0.3, 0.6, 1.0, 0.875),
    B=((), (0.2,), (0.075, 0.225), (0.3, -0.9, 1.2),
       (-11.0 / 54.0, 2.5, -70.0 / 27.0, 35.0 / 27.0),
       (1631.0 / 55296.0, 175.0 / 512.0, 575.0 / 13824.0, 44275.0 / 110592.0, 253.0 / 4096.0)),
    C=(37.0 / 378.0, 0.0, 250.0 / 621.0, 125.0 / 594.0, 0.0, 512.0 / 1771.0),
    D=(2825.0 / 27648.0, 0.0, 18575.0 / 48384.0, 13525.0 / 55296.0, 277.0 / 14336.0, 0.25),
)
# Dormand-Prince tableau (integrator.f90:171-185)
DP = dict(
    A=(0.0, 0.2, 0.3, 0.8, 8.0 / 9.0, 1.0, 1.0),
    B=((), (0.2,), (0.075, 0.225), (44.0 / 45.0, -56.0 / 15.0, 32.0 / 9.0),
       (19372.0 / 6561.0, -25360.0 / 2187.0, 64448.0 / 6561.0, -212.0 / 729.0),
       (9017.0 / 3168.0, -355.0 / 33.0, 46732.0 / 5247.0, 49.0 / 176.0, -5103.0 / 18656.0)),
    C=(35.0 / 384.0, 0.0, 500.0 / 1113.0, 125.0 / 192.0, -2187.0 / 6784.0, 11.0 / 84.0),
    D=(5179.0 / 57600.0, 0.0, 7571.0 / 16695.0, 393.0 / 640.0, -92097.0 / 339200.0, 187.0 / 2100.0, 0.025),
)
RK_SAFETY, RK_PGROW, RK_PSHRNK, RK_MINSCAL, RK_MAXSCAL = 0.9, -0.2, -0.25, 0.1, 5.0
RK_ERRCON = (5.0 / RK_SAFETY) ** (1.0 / RK_PGROW)
EPS_B = 1e-8          # cmf2_integration.f90:13
NKRYLOV_MAX = 20      # cmf2_integration.f90:11


class OracleError(RuntimeError):
    pass


# ----------------------------------------------------------------------------
# Small dense helpers
# ----------------------------------------------------------------------------

def mode_product(M: np.ndarray, X: np.ndarray, m: int) -> np.ndarray:
    """Y(..., j', ...) = sum_j M(j', j) X(..., j, ...) along axis m."""
    return np.moveaxis(np.tensordot(M, X, axes=([1], [m])), 0, m)


def hole_contract(X: np.ndarray, Y: np.ndarray, m: int) -> np.ndarray:
    """C(j1, j2) = sum_{other indices} conj(X(.., j1, ..)) Y(.., j2, ..)."""
    axes = [k for k in range(X.ndim) if k != m]
    return np.tensordot(X.conj(), Y, axes=(axes, axes))


def herm_from_upper(U: np.ndarray) -> np.ndarray:
    """Full Hermitian matrix from the upper triangle (how zhemm/zheev 'U' read it)."""
    return np.triu(U) + np.triu(U, 1).conj().T


def std_reg_inv(Amat: np.ndarray, eps: float, regtype: str) -> np.ndarray:
    """StdRegInv (maths.f90:8-83): eigen-decomposition + regularised inverse."""
    w, U = np.linalg.eigh(herm_from_upper(Amat), UPLO="U")
    if regtype == "tikh":
        w = w / (w ** 2 + eps ** 2)
    elif regtype == "tik2":
        w2e2 = w ** 2 + eps ** 2
        w = w * (w2e2 + eps ** 2) / w2e2 ** 2
    elif regtype == "poly":
        w = np.where(w < eps, 0.5 * (eps + w ** 2 / eps), w)
        w = 1.0 / w
    elif regtype == "expo":
        ew = eps * np.exp(-(w / eps) ** 2)
        w = w / (w ** 2 + ew ** 2)
    elif regtype == "strd":
        w = np.where(w < eps * 64.0, w + eps * np.exp(-w / eps), w)
        w = 1.0 / w
    else:
        raise OracleError(f"no regularization type {regtype}")
    return (U * w) @ U.conj().T


def std_reg_sol(Amat: np.ndarray, Y: np.ndarray, eps: float, regtype: str) -> np.ndarray:
    """StdRegSol (maths.f90:87-162)."""
    w, U = np.linalg.eigh(herm_from_upper(Amat), UPLO="U")
    uy = U.conj().T @ Y
    if regtype == "tikh":
        uy = uy * w / (w ** 2 + eps ** 2)
    elif regtype == "poly":
        uy = np.where(w < eps, uy * 2 * eps / (eps ** 2 + w ** 2), uy / w)
    else:
        raise OracleError(f"regularization {regtype} not restated")
    return U @ uy


def inverse_square_root(Amat: np.ndarray, eps: float) -> np.ndarray:
    """InverseSquareRoot (maths.f90:588-618)."""
    w, U = np.linalg.eigh(herm_from_upper(Amat), UPLO="U")
    f = np.sqrt(w / (w ** 2 + eps ** 2))
    return (U * f) @ U.conj().T


def inverse_square_root_u(Amat: np.ndarray) -> np.ndarray:
    """InverseSquareRootU (maths.f90:621-644): inverse of the upper Cholesky factor."""
    Lc = np.linalg.cholesky(herm_from_upper(Amat))   # A = L L^H, U = L^H
    Uc = Lc.conj().T
    return np.triu(np.linalg.inv(Uc))


# ----------------------------------------------------------------------------
# Gaussian integrals (hamilton.f90:745-902, gmctdh_objects.f90:1476-1519)
# ----------------------------------------------------------------------------

# T(k, n) = Binomial(n, 2k) * (2k-1)!!  (hamilton.f90:761-785)
def _coeff_table():
    T = np.zeros((11, 21))
    for n in range(21):
        for k in range(0, n // 2 + 1):
            df = 1
            for x in range(2 * k - 1, 0, -2):
                df *= x
            T[k, n] = math.comb(n, 2 * k) * df
    return T


GAU_COEFF = _coeff_table()


def gau_int_1d(a1: float, a2: float, xi1: complex, xi2: complex, iop: int) -> complex:
    """<g1|op|g2>/<g1|g2> for g = exp(a x^2 + xi x) (GauInt1D, hamilton.f90:745-849)."""
    xi1c = np.conj(xi1)
    if iop == 0:
        return 1.0 + 0j
    if iop == -1:
        return -1j * (a1 * xi2 - a2 * xi1c) / (a1 + a2)
    if iop == -2:
        a12 = a1 + a2
        return ((a2 * xi1c - a1 * xi2) / a12) ** 2 + 2.0 * a1 * a2 / a12
    if iop == -3:
        g = a1 ** 2 - a2 ** 2 + (a2 * xi1c - a1 * xi2) * (xi1c + xi2)
        return -1j * g / (a1 + a2) ** 2
    if iop == 1:
        return (xi1c + xi2) / (-2.0 * (a1 + a2))
    if iop == 2:
        a12 = 2.0 * (a1 + a2)
        return ((xi1c + xi2) / a12) ** 2 - 1.0 / a12
    if 3 <= iop <= 19 and iop % 2 == 1:
        g = 0j
        c1 = xi1c + xi2
        a12 = -2.0 * (a1 + a2)
        for k in range(0, iop // 2 + 1):
            g = g + GAU_COEFF[k, iop] / a12 ** (iop - k) * c1 ** (iop - k - k)
        return g
    if 4 <= iop <= 20 and iop % 2 == 0:
        g = 0j
        a12 = -2.0 * (a1 + a2)
        c2 = (xi1c + xi2) ** 2 / a12
        c1 = 1.0 + 0j
        for k in range(iop // 2, -1, -1):
            g = g + GAU_COEFF[k, iop] * c1
            c1 = c1 * c2
        return g / a12 ** (iop // 2)
    raise OracleError(f"GauInt1D operator {iop} not restated")


def gau10_int_1d(a1: float, a2: float, xi1: complex, xi2: complex, iop: int) -> complex:
    """<dg1/dxi1|op|g2>/<g1|g2> (Gau10Int1D, hamilton.f90:853-902)."""
    if iop == -1:
        return -1j * xi2 * gau_int_1d(a1, a2, xi1, xi2, 1) - 2j * a2 * gau_int_1d(a1, a2, xi1, xi2, 2)
    if iop == -2:
        return ((a2 + a2 + xi2 ** 2) * gau_int_1d(a1, a2, xi1, xi2, 1)
                + 4.0 * a2 * xi2 * gau_int_1d(a1, a2, xi1, xi2, 2)
                + 4.0 * a2 ** 2 * gau_int_1d(a1, a2, xi1, xi2, 3))
    if iop == -3:
        return -1j * (gau_int_1d(a1, a2, xi1, xi2, 1) + 2.0 * xi2 * gau_int_1d(a1, a2, xi1, xi2, 2)
                      + 4.0 * a2 * gau_int_1d(a1, a2, xi1, xi2, 3))
    if 0 <= iop <= 19:
        return gau_int_1d(a1, a2, xi1, xi2, iop + 1)
    raise OracleError(f"Gau10Int1D operator {iop} not restated")


def gau_ovl_1d(a1: float, a2: float, xi1: complex, xi2: complex) -> complex:
    """GauOvl1D (gmctdh_objects.f90:1476-1493): <g1|g2> of normalised 1D Gaussians."""
    c = xi1.real ** 2 / a1 + xi2.real ** 2 / a2 - (np.conj(xi1) + xi2) ** 2 / (a1 + a2)
    return np.exp(0.25 * c) * math.sqrt(math.sqrt(4 * a1 * a2 / (a1 + a2) ** 2))


def gau_ovl_multid(a1: np.ndarray, a2: np.ndarray, xi1: np.ndarray, xi2: np.ndarray) -> complex:
    """Overlap of normalised multi-D Gaussians (GauOvlMultiD, gmctdh_objects.f90:1497-1519)."""
    if np.all(np.abs(a1 - a2) < _EPS):
        c = np.sum((xi1.real ** 2 + xi2.real ** 2 - 0.5 * (xi1.conj() + xi2) ** 2) / a1)
        return complex(np.exp(0.25 * c))
    c = np.sum(xi1.real ** 2 / a1 + xi2.real ** 2 / a2 - (xi1.conj() + xi2) ** 2 / (a1 + a2))
    d = math.sqrt(float(np.prod(4 * a1 * a2 / (a1 + a2) ** 2)))
    return complex(np.exp(0.25 * c) * math.sqrt(d))


# ----------------------------------------------------------------------------
# The oracle proper
# ----------------------------------------------------------------------------

class Oracle:
    """Stateful like the reference's modules: h1mode, rho, MeanField, rhom1MF,
    S00, ... are recomputed by the same calls in the same order."""

    def __init__(self, model: Model):
        self.m = model
        self.eom_calls = 0
        self.hb_calls = 0
        self.wppop = [1.0] * model.npackets

    # ---------------- SPF-side objects ----------------
    def apply_oper(self, mode: int, k: int, phi: np.ndarray) -> np.ndarray:
        """Apply operator k of DVR mode `mode` to a (G, n) SPF block
        (hamilton.f90:447-471, MultTens/MultTensDiag :577-629)."""
        md = self.m
        dofs = md.mode_dofs[mode]
        _, _, dops = md.oper[mode][k]
        n = phi.shape[1]
        shape = tuple(md.ngp[d] for d in dofs) + (n,)
        X = phi.reshape(shape, order="F")
        for kk, d in enumerate(dofs):
            code = dops[kk]
            if code == 0:
                continue
            kind, M = md.dof_op_matrix(d, code)
            if kind == "dense":
                # psi(.., g, ..) <- sum_g' psi(.., g', ..) M(g', g)   (zlacrm from the right)
                X = mode_product(M.T, X, kk)
            else:
                sh = [1] * len(shape)
                sh[kk] = md.ngp[d]
                X = X * M.reshape(sh)
        return X.reshape((-1, n), order="F")

    def gwp_params(self, psi: np.ndarray, i: int, s: int):
        md = self.m
        m = md.modes_gwp[i]
        nmd = len(md.mode_dofs[m])
        ns = int(md.nspf[m, s])
        xi = md.spf_block(psi, m, s)          # (nmd, ns)
        a = md.gwpa[:nmd, :ns, i]             # (nmd, ns)
        return xi, a

    def calc_s00(self, psi: np.ndarray, i: int):
        """Calc_S00 (gmctdh_objects.f90:323-381): full matrices S00[i][s1][s2]."""
        md = self.m
        m = md.modes_gwp[i]
        S = self.S00.setdefault(i, {})
        states = range(md.nstates) if md.multiset[m] else [0]
        for s in states:
            xi, a = self.gwp_params(psi, i, s)
            ns = xi.shape[1]
            M = np.eye(ns, dtype=np.complex128)
            for j1 in range(ns):
                for j2 in range(j1 + 1, ns):
                    M[j1, j2] = gau_ovl_multid(a[:, j1], a[:, j2], xi[:, j1], xi[:, j2])
                    M[j2, j1] = np.conj(M[j1, j2])
            S[(s, s)] = M
        if not md.multiset[m]:
            return
        for s2 in range(md.nstates):
            for s1 in range(s2):
                xi1, a1 = self.gwp_params(psi, i, s1)
                xi2, a2 = self.gwp_params(psi, i, s2)
                M = np.zeros((xi1.shape[1], xi2.shape[1]), dtype=np.complex128)
                for j1 in range(xi1.shape[1]):
                    for j2 in range(xi2.shape[1]):
                        M[j1, j2] = gau_ovl_multid(a1[:, j1], md.gwpa[:len(xi2), j2, i], xi1[:, j1], xi2[:, j2])
                S[(s1, s2)] = M
                S[(s2, s1)] = M.conj().T

    def s00(self, i: int, s1: int, s2: int) -> np.ndarray:
        m = self.m.modes_gwp[i]
        if not self.m.multiset[m]:
            s1 = s2 = 0
        return self.S00[i][(s1, s2)]

    def calc_s00m1(self, i: int):
        """Calc_S00m1 (gmctdh_objects.f90:385-404): Tikhonov inverse of S."""
        md = self.m
        m = md.modes_gwp[i]
        states = range(md.nstates) if md.multiset[m] else [0]
        for s in states:
            self.S00m1[(i, s)] = std_reg_inv(self.S00[i][(s, s)], md.eps_ovl, "tikh")

    def calc_h1mode(self, psi: np.ndarray, mode: int):
        """Calc_h1mode (hamilton.f90:416-531).  Same-state matrices are the
        Hermitian part 1/2 (phi^H op phi + (op phi)^H phi) as zher2k builds them."""
        md = self.m
        hm = self.h1mode.setdefault(mode, {})
        if not md.is_gwp_mode[mode]:
            for k, (l, r, dops) in enumerate(md.oper[mode]):
                if md.is_identity[mode, k]:
                    hm[k] = np.eye(int(md.nspf[mode, l]), dtype=np.complex128)
                    continue
                phi2 = md.spf_block(psi, mode, r)
                ophi = self.apply_oper(mode, k, phi2)
                if l == r:
                    X = phi2.conj().T @ ophi
                    hm[k] = 0.5 * (X + X.conj().T)
                else:
                    phi1 = md.spf_block(psi, mode, l)
                    hm[k] = phi1.conj().T @ ophi
        else:
            i = md.modes_gwp.index(mode)
            for k, (l, r, dops) in enumerate(md.oper[mode]):
                if md.is_identity[mode, k]:
                    hm[k] = self.s00(i, l, r).copy()
                    continue
                xi1, a1 = self.gwp_params(psi, i, l)
                xi2, a2 = self.gwp_params(psi, i, r)
                n1, n2 = xi1.shape[1], xi2.shape[1]
                S = self.s00(i, l, r)
                H = np.zeros((n1, n2), dtype=np.complex128)
                for j2 in range(n2):
                    for j1 in range(n1):
                        if l == r and j1 > j2:
                            continue
                        g = 1.0 + 0j
                        for kk in range(len(dops)):
                            g *= gau_int_1d(a1[kk, j1], a2[kk, j2], xi1[kk, j1], xi2[kk, j2], dops[kk])
                        H[j1, j2] = S[j1, j2] * g
                hm[k] = herm_from_upper(H) if l == r else H

    # ---------------- A-side objects ----------------
    def packets(self, A: np.ndarray) -> List[np.ndarray]:
        """The packets of a mixture: A(APacketOffset(W) + 1 : ...) with
        APacketOffset(W) = W * nAConftot (init_calc.f90:50-53)."""
        n = self.m.naconftot
        return [A[W * n:(W + 1) * n] for W in range(self.m.npackets)]

    def calc_rho1mode(self, mode: int, A: np.ndarray):
        """Calc_rho1mode (gmctdh_objects.f90:408-477), summed over the packets."""
        md = self.m
        for s in range(md.nstates):
            R = 0
            for AW in self.packets(A):
                X = md.a_state(AW, s)
                Y = X
                for i, m2 in enumerate(md.modes_gwp):
                    if m2 == mode:
                        continue
                    Y = mode_product(self.s00(i, s, s), Y, m2)
                R = R + hole_contract(Y, X, mode)
            self.rho[(mode, s)] = 0.5 * (R + R.conj().T)
        if not md.multiset[mode]:
            ra = self.rho[(mode, 0)].copy()
            for s in range(1, md.nstates):
                ra = ra + self.rho[(mode, s)]
            self.rho_ave[mode] = ra

    def _right_chain(self, X: np.ndarray, ioper: np.ndarray, skip: np.ndarray) -> List[np.ndarray]:
        """H_f x X, H_(f-1) x H_f x X, ... (gmctdh_objects.f90:527-550)."""
        f = self.m.nmodes
        R = [X]
        for im in range(f):
            jm = f - 1 - im
            if skip[jm]:
                R.append(R[-1])
                continue
            R.append(mode_product(self.h1mode[jm][int(ioper[jm])], R[-1], jm))
        return R

    def _left_chain(self, X: np.ndarray, ioper: np.ndarray, skip: np.ndarray) -> List[np.ndarray]:
        """X x H_1, X x H_1 x H_2, ... (gmctdh_objects.f90:552-573)."""
        f = self.m.nmodes
        L = [X]
        for im in range(f - 1):
            if skip[im]:
                L.append(L[-1])
                continue
            L.append(mode_product(self.h1mode[im][int(ioper[im])].conj().T, L[-1], im))
        return L

    def _add_mf(self, im: int, k: int, M: np.ndarray):
        key = (im, k)
        self.MF[key] = self.MF.get(key, 0) + M

    def calc_meanfield(self, A: np.ndarray, t: float):
        """Calc_MeanField (gmctdh_objects.f90:481-1141): Hamiltonian terms per
        packet (:513-604), type-1 dissipation alpha V rho V^+ (:606-745), type-2
        dissipation beta (W rho + rho W^+) (:747-845) and the Lagrange multipliers
        that conserve the total population and the packets' orthogonality
        (:612-620, 1128-1137).  The perturbative harmonic bath is not covered.

        Returns Adot (the reference stores its complex conjugate in Adot_tmp), sets
        self.MF[(mode, op)], self.energyMF, self.mult_diag and self.mult_lag (lower
        triangle)."""
        md = self.m
        f = md.nmodes
        n = md.naconftot
        P = md.npackets
        pk = self.packets(A)
        self.MF = {}
        adot = np.zeros(n * P, dtype=np.complex128)
        energy = 0.0

        def seg(W, s):
            o = W * n + int(md.astate_offset[s])
            return slice(o, o + int(md.naconf[s]))

        for t_ in range(md.nham):
            s1, s2 = int(md.lhs_el[t_]), int(md.rhs_el[t_])
            ae = md.ae[t_]
            for W, AW in enumerate(pk):
                R = self._right_chain(md.a_state(AW, s2), md.ioper[:, t_], md.skip_term[:, t_])
                L = self._left_chain(md.a_state(AW, s1), md.ioper[:, t_], md.skip_term[:, t_])
                Rf = R[f].reshape(-1, order="F")
                adot[seg(W, s1)] += md.der_factor * ae * Rf                             # :578
                energy += float((ae * np.vdot(A[seg(W, s1)], Rf)).real)                # :580
                for im in range(f):                                                     # :582-601
                    k = int(md.ioper[im, t_])
                    if md.is_identity[im, k]:
                        continue
                    self._add_mf(im, k, ae * hole_contract(L[im], R[f - 1 - im], im))
        self.energyMF = energy
        # dissipative terms
        self.mult_diag = 0.0
        self.mult_lag = np.zeros((P, P), dtype=np.complex128)
        pop = np.asarray(self.wppop, dtype=float)
        reg = md.eps_pop * np.exp(-(pop / md.eps_pop) ** 2)
        wpm1 = pop / (pop ** 2 + reg ** 2)                                              # :616-619
        Amat = A.reshape((n, P), order="F")
        for kd, idx in enumerate(md.diss1):                                             # :606-745
            aeD1 = md.aeD1[kd]
            dterms = md.dissipation[idx][2]
            iop, sk = md.ioper_diss[idx], md.skip_diss[idx]
            VA = np.zeros(n * P, dtype=np.complex128)
            for t_, term in enumerate(dterms):
                s1, s2 = term.lhs, term.rhs
                for W, AW in enumerate(pk):
                    X = md.a_state(AW, s2)
                    for im in range(f):                                                 # :630-646
                        if sk[im, t_]:
                            continue
                        X = mode_product(self.h1mode[im][int(iop[im, t_])], X, im)
                    VA[seg(W, s1)] += term.coeff * X.reshape(-1, order="F")            # :648
            VAm = VA.reshape((n, P), order="F")
            AVA = Amat.conj().T @ VAm                                                   # :661-662, <A_i|V A_j>
            self.mult_diag += aeD1 * -float(np.sum((np.abs(AVA) ** 2) * wpm1[:, None]))   # :664-672
            AVAAVpA = aeD1 * (AVA @ AVA.conj().T)                                       # :674
            for i in range(P):
                for j in range(i):
                    self.mult_lag[i, j] += AVAAVpA[i, j] * (wpm1[i] + wpm1[j])         # :675-676
            adot += (aeD1 * (VAm @ AVA.conj().T) * wpm1[None, :]).reshape(-1, order="F")  # :678-684
            AuxA = (1j * aeD1 * (Amat @ AVA.conj().T)) * wpm1[None, :]                # :686-692
            auxp = [AuxA[:, W] for W in range(P)]
            for t_, term in enumerate(dterms):                                          # :696-744
                s1, s2 = term.lhs, term.rhs
                for im in range(f):
                    k = int(iop[im, t_])
                    if md.is_identity[im, k]:
                        continue
                    for W, AW in enumerate(pk):
                        X = md.a_state(AW, s2)
                        for im2 in range(f):
                            if im2 == im or sk[im2, t_]:
                                continue
                            X = mode_product(self.h1mode[im2][int(iop[im2, t_])], X, im2)
                        self._add_mf(im, k, term.coeff * hole_contract(X, md.a_state(auxp[W], s1), im))
        for kd, idx in enumerate(md.diss2):                                             # :747-845
            dterms = md.dissipation[idx][2]
            iop, sk = md.ioper_diss[idx], md.skip_diss[idx]
            for t_, term in enumerate(dterms):
                aet = md.aeD2[kd] * term.coeff
                cd = md.der_factor * 1j * aet
                s1, s2 = term.lhs, term.rhs
                for W, AW in enumerate(pk):
                    R = self._right_chain(md.a_state(AW, s2), iop[:, t_], sk[:, t_])
                    L = self._left_chain(md.a_state(AW, s1), iop[:, t_], sk[:, t_])
                    Rf = R[f].reshape(-1, order="F")
                    adot[seg(W, s1)] += cd * Rf                                        # :805-806
                    self.mult_diag += -float((cd * np.vdot(A[seg(W, s1)], Rf)).real)  # :807-808
                    for W2 in range(W):                                                 # :809-813
                        self.mult_lag[W, W2] += np.conj(cd) * np.vdot(Rf, A[seg(W2, s1)])
                    for W2 in range(W + 1, P):                                          # :814-818
                        self.mult_lag[W2, W] += cd * np.conj(np.vdot(Rf, A[seg(W2, s1)]))
                    for im in range(f):                                                 # :820-840
                        k = int(iop[im, t_])
                        if md.is_identity[im, k]:
                            continue
                        self._add_mf(im, k, 1j * aet * hole_contract(L[im], R[f - 1 - im], im))
        for j in range(P):                                                              # :1128-1137
            for i in range(j + 1, P):
                dw = pop[i] - pop[j]
                r = md.eps_pop * math.exp(-(dw / md.eps_pop) ** 2)
                self.mult_lag[i, j] *= 1j * dw / (dw ** 2 + r ** 2)
        return adot

    def apply_multipliers(self, A: np.ndarray, dA: np.ndarray) -> np.ndarray:
        """dA += multLagDiag A + i A multLag with multLag Hermitian from its
        lower triangle and a zero diagonal (derivatives.f90:238-242)."""
        md = self.m
        P = md.npackets
        M = np.tril(self.mult_lag, -1)
        M = M + M.conj().T
        Amat = A.reshape((md.naconftot, P), order="F")
        return dA + self.mult_diag * A + (1j * (Amat @ M)).reshape(-1, order="F")

    def calc_rhom1mf(self):
        """Calc_rhom1MF (gmctdh_objects.f90:1147-1194) with 'poly' regularisation."""
        md = self.m
        self.rhom1MF = {}
        for mode in md.modes_dvr:
            if md.multiset[mode]:
                for s in range(md.nstates):
                    rinv = std_reg_inv(self.rho[(mode, s)], md.eps_rho, "poly")
                    for k, (l, r, _) in enumerate(md.oper[mode]):
                        if l != s or md.is_identity[mode, k]:
                            continue
                        self.rhom1MF[(mode, k)] = rinv @ self.MF.get((mode, k), np.zeros((rinv.shape[0], int(md.nspf[mode, r])), np.complex128))
            else:
                rinv = std_reg_inv(self.rho_ave[mode], md.eps_rho, "poly")
                for k in range(len(md.oper[mode])):
                    if md.is_identity[mode, k]:
                        continue
                    self.rhom1MF[(mode, k)] = rinv @ self.MF.get((mode, k), np.zeros_like(rinv))

    def dvr_spf_derivative(self, psi: np.ndarray, mode: int, dpsi: np.ndarray):
        """DVR SPF derivative with the (1 - P) projector (derivatives.f90:96-153,
        cmf2_derivatives.f90:118-173)."""
        md = self.m
        G = md.ngpm[mode]
        acc: Dict[int, np.ndarray] = {}
        for k, (l, r, _) in enumerate(md.oper[mode]):
            if md.is_identity[mode, k]:
                continue
            ophi = self.apply_oper(mode, k, md.spf_block(psi, mode, r))
            contrib = md.der_factor * (ophi @ self.rhom1MF[(mode, k)].T)
            acc[l] = acc.get(l, 0) + contrib
        states = range(md.nstates) if md.multiset[mode] else [0]
        for s in states:
            phi = md.spf_block(psi, mode, s)
            n = phi.shape[1]
            d = acc.get(s, np.zeros((G, n), np.complex128))
            if not isinstance(d, np.ndarray):
                d = np.zeros((G, n), np.complex128)
            ovl = phi.conj().T @ phi
            ovldot = phi.conj().T @ d
            x = np.linalg.solve(herm_from_upper(np.triu(ovl)), ovldot)     # zposv 'U'
            d = d - phi @ x
            o = int(md.ipsispf[mode, s])
            dpsi[o:o + G * n] = d.reshape(-1, order="F")

    # ---------------- G-MCTDH block ----------------
    def calc_cy(self, psi: np.ndarray, i: int):
        """Calc_CY (gmctdh_objects.f90:1198-1333), without the D-matrix variant."""
        md = self.m
        mode = md.modes_gwp[i]
        nmd = len(md.mode_dofs[mode])
        states = range(md.nstates) if md.multiset[mode] else [0]
        for s in states:
            xi, a = self.gwp_params(psi, i, s)
            ns = xi.shape[1]
            S = self.s00(i, s, s)
            gx = np.zeros((nmd, ns, ns), dtype=np.complex128)
            for j2 in range(ns):
                for j1 in range(j2 + 1):
                    for k in range(nmd):
                        gx[k, j1, j2] = gau_int_1d(a[k, j1], a[k, j2], xi[k, j1], xi[k, j2], 1)
            nG = ns * nmd
            Sa0 = np.zeros((nG, ns), dtype=np.complex128)
            for j2 in range(ns):
                for j1 in range(ns):
                    for k in range(nmd):
                        if j1 <= j2:
                            Sa0[j1 * nmd + k, j2] = S[j1, j2] * gx[k, j1, j2]
            for j2 in range(ns):
                for j1 in range(ns):
                    if j1 > j2:
                        for k in range(nmd):
                            Sa0[j1 * nmd + k, j2] = np.conj(Sa0[j2 * nmd + k, j1])
            Sa0Sm1 = Sa0 @ self.S00m1[(i, s)]
            self.Sa0Sm1[(i, s)] = Sa0Sm1
            Sab = np.zeros((nG, nG), dtype=np.complex128)
            for j2 in range(ns):
                for k2 in range(nmd):
                    for j1 in range(j2 + 1):
                        for k1 in range(nmd):
                            if k1 == k2:
                                v = gau_int_1d(a[k1, j1], a[k2, j2], xi[k1, j1], xi[k2, j2], 2)
                            else:
                                v = gx[k1, j1, j2] * gx[k2, j1, j2]
                            Sab[j1 * nmd + k1, j2 * nmd + k2] = S[j1, j2] * v
            # zher2k('U','N', -1/2, Sa0S00m1, Sa0): only the upper triangle is meaningful
            Sab = Sab - 0.5 * (Sa0Sm1 @ Sa0.conj().T + Sa0 @ Sa0Sm1.conj().T)
            rho = self.rho[(mode, s)] if md.multiset[mode] else self.rho_ave[mode]
            C = np.zeros((nG, nG), dtype=np.complex128)
            for j2 in range(ns):
                for j1 in range(j2 + 1):
                    C[j1 * nmd:(j1 + 1) * nmd, j2 * nmd:(j2 + 1) * nmd] = \
                        rho[j1, j2] * Sab[j1 * nmd:(j1 + 1) * nmd, j2 * nmd:(j2 + 1) * nmd]
            self.Cmat[(i, s)] = np.triu(C)
            Y = np.zeros(nG, dtype=np.complex128)
            for k_op, (l, r, dops) in enumerate(md.oper[mode]):
                if md.is_identity[mode, k_op]:
                    continue
                if md.multiset[mode] and l != s:
                    continue
                s2 = r
                xi2, a2 = self.gwp_params(psi, i, s2)
                ns2 = xi2.shape[1]
                S12 = self.s00(i, s, s2)
                Ha0 = np.zeros((nG, ns2), dtype=np.complex128)
                for j2 in range(ns2):
                    for j1 in range(ns):
                        gi = np.array([gau_int_1d(a[k, j1], md.gwpa[k, j2, i], xi[k, j1], xi2[k, j2], dops[k])
                                       for k in range(nmd)])
                        for k in range(nmd):
                            p = np.prod(gi[:k]) * np.prod(gi[k + 1:])
                            Ha0[j1 * nmd + k, j2] = S12[j1, j2] * p * gau10_int_1d(
                                a[k, j1], md.gwpa[k, j2, i], xi[k, j1], xi2[k, j2], dops[k])
                h = self.h1mode[mode][k_op]
                Ha0 = Ha0 - Sa0Sm1 @ h
                MF = self.MF.get((mode, k_op), np.zeros((ns, ns2), np.complex128))
                for j2 in range(ns2):
                    for j1 in range(ns):
                        Y[j1 * nmd:(j1 + 1) * nmd] += MF[j1, j2] * Ha0[j1 * nmd:(j1 + 1) * nmd, j2]
            self.Yvec[(i, s)] = Y

    # ---------------- Calc_Derivs ----------------
    def _prepare(self, A: np.ndarray, psi: np.ndarray):
        md = self.m
        self.S00: Dict[int, Dict] = {}
        self.S00m1: Dict = {}
        self.Sa0Sm1: Dict = {}
        self.Cmat: Dict = {}
        self.Yvec: Dict = {}
        self.h1mode: Dict[int, Dict[int, np.ndarray]] = {}
        self.rho: Dict = {}
        self.rho_ave: Dict = {}
        for i in range(len(md.modes_gwp)):
            self.calc_s00(psi, i)
            self.calc_s00m1(i)
        for mode in range(md.nmodes):
            self.calc_rho1mode(mode, A)
            self.calc_h1mode(psi, mode)

    def calc_derivs(self, A: np.ndarray, psi: np.ndarray, t: float) -> Tuple[np.ndarray, np.ndarray]:
        """Calc_Derivs (derivatives.f90:39-237) for npackets = 1."""
        md = self.m
        self.eom_calls += 1
        self._prepare(A, psi)
        # packet populations (derivatives.f90:70-83); one packet keeps the unit
        # population that WriteOutput leaves in WPpop (output.f90:47-53)
        self.wppop = [self.norm_wf(AW, psi) for AW in self.packets(A)] if md.npackets > 1 else [1.0]
        adot = self.calc_meanfield(A, t)
        self.calc_rhom1mf()
        for i in range(len(md.modes_gwp)):
            self.calc_cy(psi, i)
        dpsi = np.zeros(md.dimpsi, dtype=np.complex128)
        for mode in md.modes_dvr:
            self.dvr_spf_derivative(psi, mode, dpsi)
        if not md.modes_gwp:
            if md.npackets > 1:
                adot = self.apply_multipliers(A, adot)
            return adot, dpsi
        # Gaussian parameter derivatives (derivatives.f90:158-173)
        for i, mode in enumerate(md.modes_gwp):
            states = range(md.nstates) if md.multiset[mode] else [0]
            for s in states:
                x = std_reg_sol(self.Cmat[(i, s)], self.Yvec[(i, s)], md.eps_C, "tikh")
                o = int(md.ipsispf[mode, s])
                dpsi[o:o + len(x)] = md.der_factor * x
        # S^-1 and tau on the coefficients of every packet (derivatives.f90:177-235)
        dA = np.zeros_like(adot)
        nA = md.naconftot
        for W in range(md.npackets):
            for s in range(md.nstates):
                o = W * nA + int(md.astate_offset[s])
                n = int(md.naconf[s])
                shape = tuple(int(x) for x in md.nspf[:, s])
                X = adot[o:o + n].reshape(shape, order="F")
                for i, mode in enumerate(md.modes_gwp):
                    js = s if md.multiset[mode] else 0
                    X = mode_product(self.S00m1[(i, js)], X, mode)
                A0 = A[o:o + n].reshape(shape, order="F")
                for i, mode in enumerate(md.modes_gwp):
                    js = s if md.multiset[mode] else 0
                    nmd = len(md.mode_dofs[mode])
                    ns = int(md.nspf[mode, s])
                    op = int(md.ipsispf[mode, s])
                    dxi = dpsi[op:op + nmd * ns].reshape((nmd, ns), order="F")
                    xi = psi[op:op + nmd * ns].reshape((nmd, ns), order="F")
                    tau = self._gwp_tau(i, js, xi, dxi)
                    X = X - mode_product(tau, A0, mode)
                dA[o:o + n] = X.reshape(-1, order="F")
        if md.npackets > 1:
            dA = self.apply_multipliers(A, dA)                  # derivatives.f90:238-242
        return dA, dpsi

    # ---------------- norms and overlaps ----------------
    def _spf_overlap(self, psi1: np.ndarray, psi2: np.ndarray, mode: int, s: int) -> np.ndarray:
        md = self.m
        if not md.is_gwp_mode[mode]:
            return md.spf_block(psi1, mode, s).conj().T @ md.spf_block(psi2, mode, s)
        i = md.modes_gwp.index(mode)
        xi1, a = self.gwp_params(psi1, i, s)
        xi2, _ = self.gwp_params(psi2, i, s)
        ns = xi1.shape[1]
        M = np.zeros((ns, ns), dtype=np.complex128)
        for j1 in range(ns):
            for j2 in range(ns):
                M[j1, j2] = gau_ovl_multid(a[:, j1], a[:, j2], xi1[:, j1], xi2[:, j2])
        return M

    def norm_wf(self, A: np.ndarray, psi: np.ndarray) -> float:
        """norm_wf (gmctdh_objects.f90:21-97)."""
        md = self.m
        tot = 0.0
        for s in range(md.nstates):
            X = md.a_state(A, s)
            Y = X
            for mode in md.modes_dvr + md.modes_gwp:
                S = self._spf_overlap(psi, psi, mode, s)
                if md.is_gwp_mode[mode]:
                    S = herm_from_upper(np.triu(S, 1) + np.eye(S.shape[0]))
                else:
                    S = herm_from_upper(S)
                Y = mode_product(S, Y, mode)
            tot += float(np.vdot(X, Y).real)
        return tot

    def wf_ovl(self, A1, psi1, A2, psi2) -> complex:
        """WF_Ovl (gmctdh_objects.f90:101-180): <Psi1|Psi2>."""
        md = self.m
        tot = 0j
        for s in range(md.nstates):
            Y = md.a_state(A2, s)
            for mode in md.modes_dvr + md.modes_gwp:
                Y = mode_product(self._spf_overlap(psi1, psi2, mode, s), Y, mode)
            tot += complex(np.vdot(md.a_state(A1, s), Y))
        return tot

    def delta_psi(self, A1, psi1, A2, psi2) -> float:
        """DeltaPsi (gmctdh_objects.f90:206-248): for a mixture
        sqrt(2 sum_W |sqrt(o11 o22) - Re o12| / sum_W sqrt(o11 o22)) over the packets."""
        if self.m.npackets > 1:
            num = pop = 0.0
            for B1, B2 in zip(self.packets(A1), self.packets(A2)):
                o11 = self.norm_wf(B1, psi1)
                o22 = self.norm_wf(B2, psi2)
                o12 = self.wf_ovl(B1, psi1, B2, psi2)
                d = math.sqrt(o11 * o22)
                pop += d
                num += abs(d - o12.real)
            return math.sqrt(2.0 * num / pop)
        o11 = self.norm_wf(A1, psi1)
        o22 = self.norm_wf(A2, psi2)
        o12 = self.wf_ovl(A1, psi1, A2, psi2)
        return math.sqrt(abs(2.0 * (1.0 - o12.real / math.sqrt(o11 * o22))))

    # ---------------- adaptive RK ----------------
    def rk_attempt(self, A, psi, dA, dpsi, t, dt, method):
        """rkck / rkdp (integrator.f90:95-221): 5th-order state and error state."""
        tab = CK if method == INT_RK45 else DP
        kA, kp = [dA], [dpsi]
        nst = 6
        for st in range(1, nst):
            b = tab["B"][st]
            At = A + dt * sum(b[j] * kA[j] for j in range(len(b)))
            pt = psi + dt * sum(b[j] * kp[j] for j in range(len(b)))
            a_, p_ = self.calc_derivs(At, pt, t + tab["A"][st] * dt)
            kA.append(a_)
            kp.append(p_)
        C = tab["C"]
        Atemp = A + dt * sum(C[j] * kA[j] for j in range(6) if C[j] != 0.0)
        ptemp = psi + dt * sum(C[j] * kp[j] for j in range(6) if C[j] != 0.0)
        D = tab["D"]
        if method == INT_RK45:
            Aerr = A + dt * sum(D[j] * kA[j] for j in range(6) if D[j] != 0.0)
            perr = psi + dt * sum(D[j] * kp[j] for j in range(6) if D[j] != 0.0)
            return Atemp, ptemp, Aerr, perr, None, None
        a7, p7 = self.calc_derivs(Atemp, ptemp, t + dt)
        kA.append(a7)
        kp.append(p7)
        Aerr = A + dt * sum(D[j] * kA[j] for j in range(7) if D[j] != 0.0)
        perr = psi + dt * sum(D[j] * kp[j] for j in range(7) if D[j] != 0.0)
        return Atemp, ptemp, Aerr, perr, a7, p7

    def rk_fixed(self, A, psi, dA, dpsi, t, dt, method):
        """One attempt of fixed length (step replay): (A, psi, dA_next, dpsi_next, errmax)."""
        At, pt, Ae, pe, a7, p7 = self.rk_attempt(A, psi, dA, dpsi, t, dt, method)
        errmax = self.delta_psi(At, pt, Ae, pe) / self.m.eps_int
        return At, pt, a7, p7, errmax

    def rkqs(self, A, psi, dA, dpsi, t, htry, method):
        """rkqs (integrator.f90:36-91).  Returns (A, psi, dA, dpsi, hdid, hnext, attempts)."""
        md = self.m
        dt = htry
        attempts = 0
        while True:
            attempts += 1
            At, pt, Ae, pe, a7, p7 = self.rk_attempt(A, psi, dA, dpsi, t, dt, method)
            errmax = self.delta_psi(At, pt, Ae, pe) / md.eps_int
            if errmax < 1.0 or dt <= md.min_stepsize:
                break
            dt = max(RK_MINSCAL * dt, RK_SAFETY * dt * errmax ** RK_PSHRNK)
            dt = max(dt, md.min_stepsize)
        if errmax > RK_ERRCON:
            hnext = RK_SAFETY * dt * errmax ** RK_PGROW
        else:
            hnext = dt * RK_MAXSCAL
        hnext = max(hnext, md.min_stepsize)
        hnext = min(hnext, md.tout)
        if method == INT_DOPRI:
            dA, dpsi = a7, p7
        return At, pt, dA, dpsi, dt, hnext, attempts

    # ---------------- Adams PECE ----------------
    @staticmethod
    def adams_weights(h_prev, dt, k):
        """Weights of Adams (integrator.f90:259-341): the predictor XX(0:k-1) and the
        correctors of order k+1 (XX(-1:k-1)) and k+2 (XX(-1:k)) from the matrix
        M(j,i) = (x_(n-i) - x_n)^j (column -1: dt^j) and B(j) = dt^(j+1)/(j+1)."""
        M = np.zeros((k + 2, k + 2))   # rows j = 0..k+1, columns i = -1..k (index i + 1)
        M[0, :] = 1.0
        hsum = 0.0
        for i in range(1, k + 1):
            hsum -= h_prev[i - 1]
            d = hsum
            for j in range(1, k + 2):
                M[j, i + 1] = d
                d *= hsum
        B = np.zeros(k + 2)
        B[0] = dt
        d = dt
        for j in range(1, k + 2):
            M[j, 0] = d
            d *= dt
            B[j] = d / (j + 1)
        pred = np.linalg.solve(M[0:k, 1:k + 1], B[0:k])           # XX(0..k-1)
        corr1 = np.linalg.solve(M[0:k + 1, 0:k + 1], B[0:k + 1])  # XX(-1..k-1)
        corr2 = np.linalg.solve(M[0:k + 2, 0:k + 2], B[0:k + 2])  # XX(-1..k)
        return pred, corr1, corr2

    def adams(self, A, psi, dA, dpsi, hist, h_prev, t, htry):
        """Adams (integrator.f90:244-380).  hist[i] = (dA, dpsi) at x_(n-1-i); h_prev[i] =
        x_(n-i) - x_(n-1-i).  Returns (A, psi, dA, dpsi, hist, h_prev, hdid, hnext)."""
        md = self.m
        k = md.int_order
        minscal, maxscal, safety = 0.3, 4.0, 0.95
        pow_shrink = -1.0 / (k + 1)
        dt = htry
        while True:
            pred, c1, c2 = self.adams_weights(h_prev, dt, k)

            def combine(w, nprev):
                At = A + w[0] * dA
                pt = psi + w[0] * dpsi
                for i in range(1, nprev + 1):
                    At = At + w[i] * hist[i - 1][0]
                    pt = pt + w[i] * hist[i - 1][1]
                return At, pt
            At, pt = combine(pred, k - 1)
            dAn, dpn = self.calc_derivs(At, pt, t + dt)
            At, pt = combine(c1[1:], k - 1)
            An, pn = dAn * c1[0] + At, dpn * c1[0] + pt
            for _ in range(md.int_par1):
                dA1, dp1 = self.calc_derivs(An, pn, t + dt)
                An, pn = dA1 * c1[0] + At, dp1 * c1[0] + pt
            At, pt = combine(c2[1:], k)
            An1, pn1 = dAn * c2[0] + At, dpn * c2[0] + pt
            for _ in range(md.int_par1):
                dA1, dp1 = self.calc_derivs(An1, pn1, t + dt)
                An1, pn1 = dA1 * c2[0] + At, dp1 * c2[0] + pt
            errmax = self.delta_psi(An, pn, An1, pn1) / md.eps_int
            if errmax < 1.0:
                break
            dt = max(minscal * dt, safety * dt * errmax ** pow_shrink)
            if dt < md.min_stepsize:
                raise OracleError("Adams step size too small")
        # errmax ** pow_shrink is +Infinity for errmax = 0 in the reference's IEEE arithmetic
        grow = errmax ** pow_shrink if errmax > 0.0 else math.inf
        hnext = min(maxscal * dt, dt * grow)
        hnext = min(hnext, md.tout)
        hist = [(dA, dpsi)] + hist[:-1]
        h_prev = [dt] + h_prev[:-1]
        dA2, dpsi2 = self.calc_derivs(An1, pn1, t + dt)
        return An1, pn1, dA2, dpsi2, hist, h_prev, dt, hnext

    # ---------------- Bulirsch-Stoer ----------------
    BS_KMAXX = 8
    BS_NSEQ = (2, 4, 6, 8, 10, 12, 14, 16, 18)
    BS_SAFE1, BS_SAFE2 = 0.25, 0.7
    BS_REDMAX, BS_REDMIN, BS_SCALMAX = 1e-5, 0.7, 0.1

    def bs_setup(self):
        """SetupBS (integrator.f90:387-414): work coefficients Ak, the tableau alf(k, q)
        and the row kMax; tNew and hnext start at impossible values."""
        kmaxx = self.BS_KMAXX
        Ak = [0.0] * (kmaxx + 2)   # 1-based: Ak[1..iMax]
        Ak[1] = self.BS_NSEQ[0] + 1.0
        for k in range(1, kmaxx + 1):
            Ak[k + 1] = Ak[k] + self.BS_NSEQ[k]
        alf = np.zeros((kmaxx + 1, kmaxx + 1))
        for iq in range(2, kmaxx + 1):
            for k in range(1, iq):
                alf[k, iq] = (self.BS_SAFE1 * self.m.eps_int) ** (
                    (Ak[k + 1] - Ak[iq + 1]) / ((Ak[iq + 1] - Ak[1] + 1.0) * (2 * k + 1)))
        kopt = kmaxx
        for ko in range(2, kmaxx):
            if Ak[ko + 1] > Ak[ko] * alf[ko - 1, ko]:
                kopt = ko
                break
        self.bs = dict(Ak=Ak, alf=alf, kmax=kopt, kopt=kopt, tnew=-1e16, first=True,
                       tstore=[0.0] * (kmaxx + 2), qA=[None] * (kmaxx + 2), qpsi=[None] * (kmaxx + 2))

    def bs_mmid(self, A0, psi0, dA, dpsi, t, htot, nstep):
        """mmid (integrator.f90:522-555): modified midpoint rule."""
        dt = htot / nstep
        Am, pm = A0, psi0
        An, pn = A0 + dt * dA, psi0 + dt * dpsi
        tx = t + dt
        dAo, dpo = self.calc_derivs(An, pn, tx)
        dt2 = dt * 2
        for _ in range(2, nstep + 1):
            As, ps = Am + dt2 * dAo, pm + dt2 * dpo
            Am, pm = An, pn
            An, pn = As, ps
            tx = tx + dt
            dAo, dpo = self.calc_derivs(An, pn, tx)
        return 0.5 * (Am + An + dt * dAo), 0.5 * (pm + pn + dt * dpo)

    def bs_pzextr(self, iest, test, Aest, pest):
        """pzextr (integrator.f90:559-608): polynomial extrapolation to zero step."""
        b = self.bs
        b["tstore"][iest] = test
        A0, p0 = Aest.copy(), pest.copy()
        A1, p1 = Aest.copy(), pest.copy()
        if iest == 1:
            b["qA"][1], b["qpsi"][1] = Aest.copy(), pest.copy()
            return A0, p0, A1, p1
        At, pt = Aest.copy(), pest.copy()
        for k1 in range(1, iest):
            delta = 1.0 / (b["tstore"][iest - k1] - test)
            f1 = test * delta
            f2 = b["tstore"][iest - k1] * delta
            qa, qp = b["qA"][k1], b["qpsi"][k1]
            b["qA"][k1], b["qpsi"][k1] = A1.copy(), p1.copy()
            cda, cdp = At - qa, pt - qp
            A1, p1 = f1 * cda, f1 * cdp
            At, pt = f2 * cda, f2 * cdp
            A0, p0 = A0 + A1, p0 + p1
        b["qA"][iest], b["qpsi"][iest] = A1.copy(), p1.copy()
        return A0, p0, A0 + A1, p0 + p1

    def bsstep(self, A, psi, dA, dpsi, t, htry, hnext_prev):
        """bsstep (integrator.f90:418-518).  Returns (A, psi, hdid, hnext)."""
        b = self.bs
        md = self.m
        dt = htry
        Asave, psave = A.copy(), psi.copy()
        if dt != hnext_prev or t != b["tnew"]:
            b["first"] = True
            b["kopt"] = b["kmax"]
        reduct = False
        converged = False
        error = [0.0] * (self.BS_KMAXX + 2)
        Ak, alf, kmax = b["Ak"], b["alf"], b["kmax"]
        while True:
            red = None
            k = 1
            while k <= kmax:
                b["tnew"] = t + dt
                As, ps = self.bs_mmid(Asave, psave, dA, dpsi, t, dt, self.BS_NSEQ[k - 1])
                test = (dt / self.BS_NSEQ[k - 1]) ** 2
                A0, p0, A1, p1 = self.bs_pzextr(k, test, As, ps)
                if k != 1:
                    errmax = self.delta_psi(A0, p0, A1, p1) / md.eps_int
                    error[k - 1] = (errmax / self.BS_SAFE1) ** (1.0 / (2 * k - 1))
                kopt = b["kopt"]
                if k != 1 and (k >= kopt - 1 or b["first"]):
                    if errmax < 1.0:
                        converged = True
                        break
                    if k == kmax or k == kopt + 1:
                        red = self.BS_SAFE2 / error[k - 1]
                        break
                    elif k == kopt:
                        if alf[kopt - 1, kopt] < error[k - 1]:
                            red = 1.0 / error[k - 1]
                            break
                    elif kopt == kmax:
                        if alf[k - 1, kmax - 1] < error[k - 1]:
                            red = alf[k - 1, kmax - 1] * self.BS_SAFE2 / error[k - 1]
                            break
                    elif alf[k - 1, kopt] < error[k - 1]:
                        red = alf[k - 1, kopt - 1] / error[k - 1]
                        break
                k += 1
            if converged:
                break
            red = max(min(red, self.BS_REDMIN), self.BS_REDMAX)
            dt = dt * red
            reduct = True
        hdid = dt
        b["first"] = False
        workmin = 1e16
        scal = None
        for kk in range(1, k):
            fact = max(error[kk], self.BS_SCALMAX)
            work = fact * Ak[kk + 1]
            if work < workmin:
                scal = fact
                workmin = work
                b["kopt"] = kk + 1
        hnext = dt / scal
        kopt = b["kopt"]
        if kopt >= k and kopt != kmax and not reduct:
            fact = max(scal / alf[kopt - 1, kopt], self.BS_SCALMAX)
            if Ak[kopt + 1] * fact <= workmin:
                hnext = dt / fact
                b["kopt"] = kopt + 1
        return A0, p0, hdid, hnext

    def _propagate_bs(self, A, psi, A0, psi0, t, step, maxtime, record_steps):
        """propagate_wf with Bulirsch-Stoer (propagator.f90:210-248)."""
        md = self.m
        self.bs_setup()
        snext = -1e15
        outputs, steps = [], []
        while t < maxtime:
            outputs.append(self.observables(A, psi, A0, psi0, t))
            tnext = t + md.tout
            while True:
                dA, dpsi = self.calc_derivs(A, psi, t)
                A, psi, sdone, snext = self.bsstep(A, psi, dA, dpsi, t, step, snext)
                if record_steps:
                    steps.append((t, step, sdone, snext, 1))
                t = t + sdone
                if t >= tnext - md.min_stepsize:
                    break
                q = int((tnext - t) / snext)
                step = (tnext - t) if q == 0 else (tnext - t) / (q + 1)
        return outputs, steps, (A, psi, t)

    # ---------------- CMF2 ----------------
    def calc_dhd_b(self, B: np.ndarray) -> np.ndarray:
        """Calc_DHD_B (cmf2_derivatives.f90:1-80): H_B * B (no der_factor)."""
        md = self.m
        self.hb_calls += 1
        HB = np.zeros_like(B)
        for t_ in range(md.nham):
            s1, s2 = int(md.lhs_el[t_]), int(md.rhs_el[t_])
            X = md.a_state(B, s2)
            for mode in md.modes_dvr:
                k = int(md.ioper[mode, t_])
                if md.is_identity[mode, k]:
                    continue
                X = mode_product(self.h1mode[mode][k], X, mode)
            for i, mode in enumerate(md.modes_gwp):
                k = int(md.ioper[mode, t_])
                if md.is_identity[mode, k]:
                    continue
                X = mode_product(self.dhd[(i, k)], X, mode)
            o1 = int(md.astate_offset[s1])
            HB[o1:o1 + int(md.naconf[s1])] += md.ae[t_] * X.reshape(-1, order="F")
        return HB

    def calc_dhd(self, DD: Dict):
        """Calc_DHD (hamilton.f90:535-574): D^H h D for GWP modes."""
        md = self.m
        self.dhd = {}
        for i, mode in enumerate(md.modes_gwp):
            for k, (l, r, _) in enumerate(md.oper[mode]):
                n1, n2 = int(md.nspf[mode, l]), int(md.nspf[mode, r])
                if md.is_identity[mode, k]:
                    self.dhd[(i, k)] = np.eye(n1, n2, dtype=np.complex128)
                    continue
                jl = l if md.multiset[mode] else 0
                jr = r if md.multiset[mode] else 0
                M = DD[(i, jl)].conj().T @ self.h1mode[mode][k] @ DD[(i, jr)]
                if l == r:
                    M = herm_from_upper(M)
                M = np.where(np.abs(M) > _EPS, M, 0)
                self.dhd[(i, k)] = M

    def lanczos(self, B0: np.ndarray, dt: float, build: bool) -> np.ndarray:
        """Lanczos (cmf2_integration.f90:30-103)."""
        md = self.m
        if build:
            n = B0.shape[0]
            BK = [B0 / np.linalg.norm(B0)]
            alpha = np.zeros(NKRYLOV_MAX)
            beta = np.zeros(NKRYLOV_MAX)
            w = self.calc_dhd_b(BK[0])
            alpha[0] = float(np.vdot(BK[0], w).real)
            w = w - alpha[0] * BK[0]
            beta[0] = np.linalg.norm(w)
            BK.append(w / beta[0])
            error = beta[0] * abs(dt)
            j = 2
            while True:
                if j == NKRYLOV_MAX:
                    raise OracleError("Maximum number of Krylov vectors reached")
                w = self.calc_dhd_b(BK[j - 1])
                alpha[j - 1] = float(np.vdot(BK[j - 1], w).real)
                w = w - beta[j - 2] * BK[j - 2]
                w = w - alpha[j - 1] * BK[j - 1]
                beta[j - 1] = np.linalg.norm(w)
                BK.append(w / beta[j - 1])
                error = error * beta[j - 1] / float(j) * abs(dt)
                if error < EPS_B:
                    break
                j += 1
            nk = j
            T = np.diag(alpha[:nk]) + np.diag(beta[:nk - 1], 1) + np.diag(beta[:nk - 1], -1)
            ev, U = np.linalg.eigh(T)                                         # dstev('V')
            self.lan_alpha = ev
            self.lan_U = U
            self.lan_BU = np.stack(BK[:nk], axis=1) @ U
            self.lan_nk = nk
        aux = self.lan_U[0, :] * np.exp(md.der_factor * self.lan_alpha * dt)
        BT = self.lan_BU @ aux
        return BT / np.linalg.norm(BT)

    def calc_der_spf_dvr(self, psi: np.ndarray, mode: int) -> np.ndarray:
        dpsi = np.zeros(self.m.dimpsi, dtype=np.complex128)
        self.dvr_spf_derivative(psi, mode, dpsi)
        return dpsi

    @staticmethod
    def _trace_rho(rho: np.ndarray, ovl: np.ndarray) -> float:
        """Tr(rho . ovl) over the upper triangle (cmf2_derivatives.f90:278-291)."""
        err = 0.0
        n = ovl.shape[0]
        for j2 in range(n):
            for j1 in range(j2):
                err += 2 * float((rho[j1, j2] * np.conj(ovl[j1, j2])).real)
            err += float((rho[j2, j2] * ovl[j2, j2]).real)
        return err

    def _rho_of(self, mode: int, s: int) -> np.ndarray:
        return self.rho[(mode, s)] if self.m.multiset[mode] else self.rho_ave[mode]

    def calc_err_spf_dvr(self, psi1, psi2, mode) -> float:
        """Calc_Err_SPF, DVR branch (cmf2_derivatives.f90:239-283)."""
        md = self.m
        err = 0.0
        states = range(md.nstates) if md.multiset[mode] else [0]
        for s in states:
            d = md.spf_block(psi1, mode, s) - md.spf_block(psi2, mode, s)
            err += self._trace_rho(self._rho_of(mode, s), d.conj().T @ d)
        return math.sqrt(abs(err))

    def calc_err_spf_gwp(self, psi1, psi2, i) -> float:
        """Calc_Err_SPF, Gaussian branch (cmf2_derivatives.f90:294-332): the
        overlap of the parameter difference from Gaussian overlaps."""
        md = self.m
        mode = md.modes_gwp[i]
        err = 0.0
        states = range(md.nstates) if md.multiset[mode] else [0]
        for s in states:
            x, a = self.gwp_params(psi1, i, s)
            y, _ = self.gwp_params(psi2, i, s)
            ns = x.shape[1]
            ovl = np.zeros((ns, ns), dtype=np.complex128)
            for j in range(ns):
                ovl[j, j] = 2.0 - 2.0 * gau_ovl_multid(a[:, j], a[:, j], x[:, j], y[:, j]).real
            for j2 in range(ns):
                for j1 in range(j2):
                    g = lambda u, v: gau_ovl_multid(a[:, j1], a[:, j2], u, v)
                    ovl[j1, j2] = g(x[:, j1], x[:, j2]) + g(y[:, j1], y[:, j2]) \
                        - g(x[:, j1], y[:, j2]) - g(y[:, j1], x[:, j2])
            err += self._trace_rho(self._rho_of(mode, s), ovl)
        return math.sqrt(abs(err))

    def _gwp_tau(self, i: int, s: int, xi: np.ndarray, dxi: np.ndarray) -> np.ndarray:
        """tau = (Sa0 S^-1)^H dxi per Gaussian plus the phase term
        1/2 sum_k Re xi Re dxi / a on the diagonal (derivatives.f90:201-234,
        cmf2_derivatives.f90:207-226)."""
        md = self.m
        mode = md.modes_gwp[i]
        nmd = len(md.mode_dofs[mode])
        ns = xi.shape[1]
        Sa0Sm1 = self.Sa0Sm1[(i, s)]
        tau = np.zeros((ns, ns), dtype=np.complex128)
        for j2 in range(ns):
            for j1 in range(ns):
                tau[j1, j2] = np.vdot(Sa0Sm1[j2 * nmd:(j2 + 1) * nmd, j1], dxi[:, j2])
        for j2 in range(ns):
            dd = 0.0
            for k in range(nmd):
                dd += xi[k, j2].real * dxi[k, j2].real / md.gwpa[k, j2, i]
            tau[j2, j2] += dd * 0.5
        return tau

    def calc_der_spf_gwp(self, psi: np.ndarray, DD: Dict, i: int):
        """Calc_Der_SPF, Gaussian branch (cmf2_derivatives.f90:175-232): S00, its
        Tikhonov inverse, h1mode and C, Y on the current parameters with the
        frozen density matrices and mean fields; the Tikhonov solve times
        der_factor; dD = -tau D."""
        md = self.m
        mode = md.modes_gwp[i]
        self.calc_s00(psi, i)
        self.calc_s00m1(i)
        self.calc_h1mode(psi, mode)
        self.calc_cy(psi, i)
        nmd = len(md.mode_dofs[mode])
        dpsi = np.zeros(md.dimpsi, dtype=np.complex128)
        dDD = {}
        states = range(md.nstates) if md.multiset[mode] else [0]
        for s in states:
            ns = int(md.nspf[mode, s])
            x = md.der_factor * std_reg_sol(self.Cmat[(i, s)], self.Yvec[(i, s)], md.eps_C, "tikh")
            o = int(md.ipsispf[mode, s])
            dpsi[o:o + len(x)] = x
            xi = psi[o:o + nmd * ns].reshape((nmd, ns), order="F")
            tau = self._gwp_tau(i, s, xi, x.reshape((nmd, ns), order="F"))
            dDD[(i, s)] = -tau @ DD[(i, s)]
        return dpsi, dDD

    def _spf_slices(self, mode):
        md = self.m
        states = range(md.nstates) if md.multiset[mode] else [0]
        rows = len(md.mode_dofs[mode]) if md.is_gwp_mode[mode] else md.ngpm[mode]
        out = []
        for s in states:
            o = int(md.ipsispf[mode, s])
            n = int(md.nspf[mode, s]) * rows
            out.append(slice(o, o + n))
        return out

    def rk_spf_ck(self, psi: np.ndarray, mode: int, htry: float, dopri: bool = False, DD: Optional[Dict] = None):
        """rk_SPF_ck / rk_SPF_dp (cmf2_integration.f90:105-253, :257-412).
        Dormand-Prince adds a 7th derivative at the 5th-order solution (:386-393).
        Gaussian modes carry their D matrices along (DDtemp, dDD)."""
        md = self.m
        sl = self._spf_slices(mode)
        tab = DP if dopri else CK
        gwp = md.is_gwp_mode[mode]
        i = md.modes_gwp.index(mode) if gwp else -1
        keys = [(i, s) for s in (range(md.nstates) if md.multiset[mode] else [0])] if gwp else []

        def der(p, D):
            if gwp:
                return self.calc_der_spf_gwp(p, D, i)
            return self.calc_der_spf_dvr(p, mode), {}

        def comb(p0, D0, coef, kp, kd):
            p = p0.copy()
            for s_ in sl:
                p[s_] = p0[s_] + dt * sum(cj * kp[j][s_] for j, cj in enumerate(coef) if cj != 0.0)
            D = dict(D0) if D0 is not None else None
            for key in keys:
                D[key] = D0[key] + dt * sum(cj * kd[j][key] for j, cj in enumerate(coef) if cj != 0.0)
            return p, D

        dt = htry
        while True:
            kp, kd = [], []
            d1, d2 = der(psi, DD)
            kp.append(d1)
            kd.append(d2)
            for st in range(1, 6):
                pt, Dt = comb(psi, DD, tab["B"][st], kp, kd)
                d1, d2 = der(pt, Dt)
                kp.append(d1)
                kd.append(d2)
            ptemp, Dtemp = comb(psi, DD, tab["C"], kp, kd)
            if dopri:
                d1, d2 = der(ptemp, Dtemp)
                kp.append(d1)
                kd.append(d2)
            perr, _ = comb(psi, DD, tab["D"], kp, kd)
            if gwp:
                error = self.calc_err_spf_gwp(ptemp, perr, i) / md.eps_psi
            else:
                error = self.calc_err_spf_dvr(ptemp, perr, mode) / md.eps_psi
            if error < 1.0:
                break
            dt = max(RK_MINSCAL * dt, RK_SAFETY * dt * error ** RK_PSHRNK)
        if error > RK_ERRCON:
            hnext = RK_SAFETY * dt * error ** RK_PGROW
        else:
            hnext = dt * RK_MAXSCAL
        out = psi.copy()
        for s_ in sl:
            out[s_] = ptemp[s_]
        if gwp:
            DD = dict(DD)
            for key in keys:
                DD[key] = Dtemp[key]
        return out, dt, hnext, DD

    def propagate_spf(self, dt: float, mode: int, psi: np.ndarray, DD: Optional[Dict] = None):
        """propagate_SPF (cmf2_base.f90:210-260): Cash-Karp (1) or Dormand-Prince (2).
        Returns psi, or (psi, DD) when D matrices are given."""
        md = self.m
        if md.int_type_psi not in (1, 2):
            raise OracleError("SPF integrator must be rk45 (1) or dopri (2)")
        done = 0.0
        step = dt
        while True:
            psi, sdone, snext, DD = self.rk_spf_ck(psi, mode, step, dopri=md.int_type_psi == 2, DD=DD)
            done += sdone
            if done >= dt:
                break
            snext = max(snext, md.min_stepsize * 2)
            step = (dt - done) / (int((dt - done) / snext) + 1)
            step = min(step, dt - done)
        return psi if DD is None else (psi, DD)

    def _propagate_spf_all(self, dt, psi, DD):
        """DVR modes, then Gaussian modes (cmf2_base.f90:108-115)."""
        md = self.m
        for mode in md.modes_dvr:
            psi = self.propagate_spf(dt, mode, psi)
        for mode in md.modes_gwp:
            psi, DD = self.propagate_spf(dt, mode, psi, DD)
        return psi, DD

    def _gwp_chain(self, X: np.ndarray, mats: Dict) -> np.ndarray:
        """Per state, mode products with mats[(i, set)] on the Gaussian modes."""
        md = self.m
        out = X.copy()
        for s in range(md.nstates):
            o = int(md.astate_offset[s])
            T = md.a_state(X, s)
            for i, mode in enumerate(md.modes_gwp):
                T = mode_product(mats[(i, s if md.multiset[mode] else 0)], T, mode)
            out[o:o + int(md.naconf[s])] = T.reshape(-1, order="F")
        return out

    def a_to_b(self, A: np.ndarray, DD: Dict) -> np.ndarray:
        """A_to_B (cmf2_base.f90:264-305): B = D^H S A on the Gaussian modes."""
        mats = {key: D.conj().T @ self.s00(key[0], key[1], key[1]) for key, D in DD.items()}
        return self._gwp_chain(A, mats)

    def b_to_a(self, B: np.ndarray, DD: Dict) -> np.ndarray:
        """B_to_A (cmf2_base.f90:309-345): A = D B on the Gaussian modes."""
        return self._gwp_chain(B, DD)

    def _inverse_sqrt_s00(self) -> Dict:
        """D = S^-1/2 by Cholesky (InverseSquareRootU) per Gaussian mode and set
        (cmf2_base.f90:63-73)."""
        md = self.m
        DD = {}
        for i, mode in enumerate(md.modes_gwp):
            for s in (range(md.nstates) if md.multiset[mode] else [0]):
                DD[(i, s)] = inverse_square_root_u(np.triu(self.S00[i][(s, s)]))
        return DD

    def _operators_and_mf(self, A, psi, t):
        self._prepare(A, psi)
        self.calc_meanfield(A, t)
        self.calc_rhom1mf()

    def cmf2_fixed(self, A, psi, t, h):
        """One CMF2 attempt of length h completed as accepted (step replay)."""
        return self.cmf2(A, psi, t, h, fixed=True)

    def cmf2(self, A, psi, t, htry, fixed=False):
        """cmf2 (cmf2_base.f90:47-206).  Returns (A, psi, hdid, hnext, tries);
        with fixed=True one attempt of length htry is completed: (A, psi, error).
        Gaussian modes propagate in the orthonormalised coefficients B = D^H S A
        with D = S^-1/2 recomputed at the step start."""
        md = self.m
        gwp = bool(md.modes_gwp)
        DD0 = {}
        if gwp:
            self.S00 = {}
            for i in range(len(md.modes_gwp)):
                self.calc_s00(psi, i)
            DD0 = self._inverse_sqrt_s00()
        hdid = htry
        tries = 0
        while True:
            tries += 1
            self._operators_and_mf(A, psi, t)
            if gwp:
                self.calc_dhd(DD0)
                B0 = self.a_to_b(A, DD0)
            else:
                B0 = A.copy()
            BHalf = self.lanczos(B0, 0.5 * hdid, True)
            psiHalf, DDHalf = self._propagate_spf_all(0.5 * hdid, psi.copy(), dict(DD0))
            AHalf = self.b_to_a(BHalf, DDHalf) if gwp else BHalf.copy()
            self._operators_and_mf(AHalf, psiHalf, t + 0.5 * hdid)
            psiHalf2, DDHalf2 = self._propagate_spf_all(0.5 * hdid, psi.copy(), dict(DD0))
            err_psi = self.delta_psi(AHalf, psiHalf, AHalf, psiHalf2)
            psiHalf2, DDHalf2 = self._propagate_spf_all(0.5 * hdid, psiHalf2, DDHalf2)
            if gwp:
                for i in range(len(md.modes_gwp)):
                    self.calc_s00(psiHalf2, i)
            self.h1mode = {}
            for mode in range(md.nmodes):
                self.calc_h1mode(psiHalf2, mode)
            if gwp:
                self.calc_dhd(DDHalf2)
            B02 = self.lanczos(BHalf, -0.5 * hdid, True)
            err_A = np.linalg.norm(B02 - B0) * 0.5
            error = max(err_A, err_psi) / md.eps_int
            if fixed:
                Bend = self.lanczos(BHalf, 0.5 * hdid, False)
                return (self.b_to_a(Bend, DDHalf2) if gwp else Bend), psiHalf2, error
            if error > 1.0:
                hdid = hdid / math.sqrt(error) * 0.95
                continue
            Bend = self.lanczos(BHalf, 0.5 * hdid, False)
            hnext = min(hdid / math.sqrt(error), hdid * 1.5) if error > 0 else hdid * 1.5
            hnext = min(hnext, md.tout)
            return (self.b_to_a(Bend, DDHalf2) if gwp else Bend), psiHalf2, hdid, hnext, tries

    # ---------------- observables and driver ----------------
    def observables(self, A, psi, A0, psi0, t):
        """WriteOutput quantities (output.f90:35-87, :144-150): populations from
        rho of mode 1, energy = energyMF / sum(pop), norm = sum(pop), C(t)."""
        md = self.m
        self._prepare(A, psi)
        self.calc_meanfield(A, t)
        pop = np.zeros(md.nstates)
        for s in range(md.nstates):
            r = self.rho[(0, s)]
            if md.is_gwp_mode[0]:
                S = self.s00(0, s, s)
                n = r.shape[0]
                v = 0.0
                for j2 in range(n):
                    for j1 in range(j2):
                        v += 2.0 * float((r[j1, j2] * S[j1, j2]).real)
                    v += float((r[j2, j2] * S[j2, j2]).real)
                pop[s] = v
            else:
                pop[s] = float(np.trace(r).real)
        auto = sum(self.wf_ovl(B0, psi0, B, psi) for B0, B in zip(self.packets(A0), self.packets(A)))  # :143-149
        wp = np.array([self.norm_wf(B, psi) for B in self.packets(A)])                    # :46-60
        wp = wp / wp.sum()
        ent = -sum(w * math.log(w) for w in wp if w >= 1e-8) / math.log(md.npackets) if md.npackets > 1 else 0.0
        return dict(t=t, pop=pop, norm=float(pop.sum()), energy=self.energyMF / pop.sum(), auto=auto,
                    wppop=np.sort(wp)[::-1], entropy=ent)

    def expectation(self, A, psi) -> np.ndarray:
        """Expectation (output.f90:449-500): for each expectation operator
        sum_t ae_t <A_l| prod_m h_m |A_r> with h1mode on every mode (identity
        matrices on grid modes, S00 on Gaussian modes), as written (the
        conjugate of the accumulated zdotu)."""
        md = self.m
        self._prepare(A, psi)
        out = np.zeros(len(md.expect), dtype=np.complex128)
        for AW in self.packets(A):                       # summed over the packets (:461)
            for i, op in enumerate(md.expect):
                for t, term in enumerate(op):
                    X = md.a_state(AW, term.rhs)
                    for mode in range(md.nmodes):
                        X = mode_product(self.h1mode[mode][int(md.ioper_expect[i][mode, t])], X, mode)
                    out[i] += term.coeff * np.vdot(md.a_state(AW, term.lhs), X)
        return out

    def natpop(self, A, psi):
        """Natural populations (eigenvalues of rho, decreasing; Gaussian modes:
        of conj(S^1/2) rho conj(S^1/2)), gross Gaussian populations and the
        population errors of neglecting one Gaussian, decreasing
        (output.f90:88-140).  Dicts keyed (mode, state)."""
        md = self.m
        self._prepare(A, psi)
        nat, ggp, perr = {}, {}, {}
        for mode in md.modes_dvr:
            for s in range(md.nstates):
                nat[(mode, s)] = np.linalg.eigvalsh(herm_from_upper(np.triu(self.rho[(mode, s)])))[::-1]
        for i, mode in enumerate(md.modes_gwp):
            for s in range(md.nstates):
                js = s if md.multiset[mode] else 0
                S = self.s00(i, js, js)
                w, U = np.linalg.eigh(herm_from_upper(np.triu(S)))         # SquareRoot (maths.f90:556-585)
                S12 = ((U * np.sqrt(w)) @ U.conj().T).conj()                 # zlacgv
                r = self.rho[(mode, s)]
                M = S12 @ herm_from_upper(np.triu(r)) @ S12                  # two zhemm 'R'
                nat[(mode, s)] = np.linalg.eigvalsh(herm_from_upper(np.triu(M)))[::-1]
                n = S.shape[0]
                g, e = np.zeros(n), np.zeros(n)
                for j1 in range(n):
                    for j2 in range(j1):
                        v = float((r[j2, j1] * S[j2, j1]).real)
                        g[j1] += v
                        e[j1] += 2 * v
                    e[j1] -= float(r[j1, j1].real)
                    for j2 in range(j1, n):
                        v = float((r[j1, j2] * S[j1, j2]).real)
                        g[j1] += v
                        e[j1] += 2 * v
                    e[j1] = abs(e[j1])
                ggp[(mode, s)] = g
                perr[(mode, s)] = np.sort(e)[::-1]
        return nat, ggp, perr

    def density(self, A, psi, dof: int, trafo: Optional[np.ndarray] = None,
                xrange: Optional[Tuple[float, float]] = None):
        """Calc_Density (output.f90:332-445) along one DOF, per state.  Grid DOFs:
        the density matrix in the coordinate representation of the DOF from rho and
        the SPFs matricised along it (MatricisePsi, hamilton.f90:664-699), its
        diagonal, and the populations of the basis functions trafo(kg, :) DM trafo(kg, :).
        Gaussian DOFs: the density on ngp equidistant points of xrange from rho, the
        Gaussian parameters and the 1D overlaps of the other DOFs of the mode."""
        md = self.m
        self._prepare(A, psi)
        mode = next(m for m in range(md.nmodes) if dof in md.mode_dofs[m])
        k = md.mode_dofs[mode].index(dof)
        nG = md.ngp[dof]
        dens = np.zeros((nG, md.nstates))
        pop = np.zeros((nG, md.nstates))
        if md.is_gwp_mode[mode]:
            i = md.modes_gwp.index(mode)
            delta = (xrange[1] - xrange[0]) / (nG - 1)
            x = xrange[0] + delta * np.arange(nG)
            nmd = len(md.mode_dofs[mode])
            pi24 = 1.0 / math.asin(1.0) ** 2
            for s in range(md.nstates):
                xi, a = self.gwp_params(psi, i, s)
                R = herm_from_upper(np.triu(self.rho[(mode, s)]))
                ns = xi.shape[1]
                for j1 in range(ns):
                    for j2 in range(ns):
                        a1, a2 = a[k, j1], a[k, j2]
                        c = R[j1, j2] * (pi24 * a1 * a2 * math.exp(xi[k, j1].real ** 2 / a1
                                                                   + xi[k, j2].real ** 2 / a2)) ** 0.25
                        for kg in range(nmd):
                            if kg != k:
                                c *= gau_ovl_1d(a[kg, j1], a[kg, j2], xi[kg, j1], xi[kg, j2])
                        dens[:, s] += (c * np.exp(x ** 2 * (a1 + a2) + x * (np.conj(xi[k, j1]) + xi[k, j2]))).real
            return dens * delta, pop
        ngs = [md.ngp[d] for d in md.mode_dofs[mode]]
        for s in range(md.nstates):
            phi = md.spf_block(psi, mode, s)
            n = phi.shape[1]
            P = np.moveaxis(phi.reshape(ngs + [n], order="F"), k, -2).reshape(-1, nG, n)
            R = herm_from_upper(np.triu(self.rho[(mode, s)]))
            DM = np.einsum("rbj,jq,raq->ab", P.conj(), R, P)
            dens[:, s] = DM.diagonal().real
            if trafo is not None:
                pop[:, s] = np.einsum("ka,ab,kb->k", trafo, DM, trafo).real
        return dens, pop

    def propagate(self, A, psi, tfinal: Optional[float] = None, max_steps: Optional[int] = None,
                  record_steps: bool = False):
        """propagate_wf (propagator.f90:87-146 RK, :257-306 CMF2).  Returns the list
        of outputs written every tout and the step history."""
        md = self.m
        A = A.copy()
        psi = psi.copy()
        A0, psi0 = A.copy(), psi.copy()
        tfin = md.tfinal if tfinal is None else tfinal
        maxtime = tfin + md.tout * 0.1
        t = md.tinit
        step = md.tout * md.eps_int
        outputs = []
        steps = []
        nsteps = 0
        if md.int_type == INT_ABM:
            return self._propagate_adams(A, psi, A0, psi0, t, step, maxtime, record_steps)
        if md.int_type == INT_BS:
            return self._propagate_bs(A, psi, A0, psi0, t, step, maxtime, record_steps)
        if md.int_type == INT_DOPRI:
            # Dormand-Prince carries the last stage's derivative into the next step
            # (rkqs, integrator.f90:82-85).  The reference's first step reads
            # dAVector before anything has computed it (propagator.f90:98, 116);
            # the derivative at the start is evaluated here instead, as the device
            # path does.
            dA, dpsi = self.calc_derivs(A, psi, t)
        while t < maxtime:
            outputs.append(self.observables(A, psi, A0, psi0, t))
            tnext = t + md.tout
            while True:
                if md.int_type == INT_CMF2:
                    A, psi, sdone, snext, tries = self.cmf2(A, psi, t, step)
                else:
                    if md.int_type == INT_RK45:
                        dA, dpsi = self.calc_derivs(A, psi, t)
                    elif md.int_type != INT_DOPRI:
                        raise OracleError(f"integrator type {md.int_type} is not an RK method")
                    A, psi, dA, dpsi, sdone, snext, tries = self.rkqs(A, psi, dA, dpsi, t, step, md.int_type)
                if record_steps:
                    steps.append((t, step, sdone, snext, tries))
                t = t + sdone
                nsteps += 1
                if max_steps is not None and nsteps >= max_steps:
                    return outputs, steps, (A, psi, t)

                if t >= tnext - md.min_stepsize:
                    break
                q = int((tnext - t) / snext)
                step = (tnext - t) if q == 0 else (tnext - t) / (q + 1)
        return outputs, steps, (A, psi, t)

    def _propagate_adams(self, A, psi, A0, psi0, t, step, maxtime, record_steps):
        """propagate_wf with Adams (propagator.f90:150-198): the first int_order steps
        with Cash-Karp rkqs, storing the derivatives and step lengths."""
        md = self.m
        k = md.int_order
        hist = [None] * k
        h_prev = [0.0] * k
        dA, dpsi = self.calc_derivs(A, psi, t)
        iprop = 0
        outputs, steps = [], []
        while t < maxtime:
            outputs.append(self.observables(A, psi, A0, psi0, t))
            tnext = t + md.tout
            while True:
                if iprop < k:
                    hist[k - 1 - iprop] = (dA, dpsi)
                    A, psi, _, _, sdone, snext, tries = self.rkqs(A, psi, dA, dpsi, t, step, INT_RK45)
                    dA, dpsi = self.calc_derivs(A, psi, t)
                    h_prev[k - 1 - iprop] = sdone
                    iprop += 1
                    if record_steps:
                        steps.append((t, step, sdone, snext, tries))
                    t = t + sdone
                    if t >= tnext - md.min_stepsize:
                        break
                    q = int((tnext - t) / snext)
                    step = (tnext - t) if q == 0 else (tnext - t) / (q + 1)
                    continue
                A, psi, dA, dpsi, hist, h_prev, sdone, snext = self.adams(A, psi, dA, dpsi, hist, h_prev, t, step)
                if record_steps:
                    steps.append((t, step, sdone, snext, 1))
                t = t + sdone
                if t >= tnext:
                    break
                step = (tnext - t) / (int((tnext - t) / snext) + 1)
                step = min(step, tnext - t)
        return outputs, steps, (A, psi, t)
