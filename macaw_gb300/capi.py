"""ctypes binding of ``libmacaw_gb300.so`` (the C-ABI of include/macaw_gb300.h).

``GpuCore`` mirrors the reference routines the C-ABI replaces, with the same
names and argument meaning: ``calc_derivs`` (derivatives.f90:39), ``rkqs``
(integrator.f90:36), ``cmf2`` (cmf2_base.f90:47), ``norm_wf`` / ``wf_ovl``
(gmctdh_objects.f90:21, :101) and the inner loop of ``propagate_wf``
(propagator.f90:110-146).  Errors come back as ``MctdhError`` carrying the
C-ABI status, the way the reference would ``stop``.  There is no CPU path:
if the library or a GPU is missing, construction raises.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Dict, List, Optional, Tuple

import numpy as np

from .model import Model, INT_CMF2

_HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(_HERE, "libmacaw_gb300.so")

I64P = C.POINTER(C.c_int64)
DP = C.POINTER(C.c_double)

STATUS = {0: "ok", -1: "unsupported feature", -2: "eigensolver did not converge", -3: "Krylov cap reached",
          -4: "step underflow", -5: "non-finite state", -6: "CUDA error", -7: "bad argument"}


class MctdhError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {STATUS.get(code, 'error')}: {msg}")
        self.code = code


class Setup(C.Structure):
    _fields_ = [
        ("nstates", C.c_int64), ("nmodes", C.c_int64), ("ndof", C.c_int64), ("nham", C.c_int64),
        ("maxdof", C.c_int64),
        ("nspf", I64P), ("nmodedof", I64P), ("idof", I64P), ("multiset", I64P), ("is_gwp", I64P),
        ("ngp", I64P), ("dvr_grid", DP), ("dvr_grid_off", I64P), ("dvr_mats", DP), ("dvr_mat_off", I64P),
        ("ae", DP), ("lhs_el", I64P), ("rhs_el", I64P), ("nopermax", C.c_int64), ("noper", I64P),
        ("oper", I64P), ("ioper", I64P), ("is_identity", I64P), ("skip_term", I64P), ("ipsispf", I64P),
        ("dimpsi", C.c_int64), ("gwpa", DP), ("ns00max", C.c_int64),
        ("eps_rho", C.c_double), ("eps_ovl", C.c_double), ("eps_C", C.c_double), ("eps_int", C.c_double),
        ("eps_A", C.c_double), ("eps_psi", C.c_double), ("min_stepsize", C.c_double),
        ("writetime", C.c_double), ("der_factor_re", C.c_double), ("der_factor_im", C.c_double),
        ("int_type_psi", C.c_int64), ("precision", C.c_int64),
        ("int_order", C.c_int64), ("int_par1", C.c_int64),
        ("nexpect", C.c_int64), ("expect_nterms", I64P), ("expect_ae", DP), ("expect_lhs", I64P),
        ("expect_rhs", I64P), ("expect_ioper", I64P),
        ("npackets", C.c_int64), ("eps_pop", C.c_double), ("term_kind", I64P), ("term_diss1", I64P),
        ("ndiss1", C.c_int64), ("diss1_ae", DP),
        ("nopparam", C.c_int64), ("ngpmax", C.c_int64), ("grid_oper", DP),
        ("oper_dvr", DP), ("oper_dvr_off", I64P), ("reginv_cold", C.c_int64),
    ]


_lib = None


def load_library() -> C.CDLL:
    """Load the in-tree shared library; raise loudly if it was not built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIBPATH):
        raise MctdhError(-6, f"{LIBPATH} is missing: run __graft_entry__.build() (there is no CPU fallback)")
    lib = C.CDLL(LIBPATH)
    vp = C.c_void_p
    lib.mctdh_create.argtypes = [C.POINTER(Setup), C.POINTER(vp)]
    lib.mctdh_destroy.argtypes = [vp]
    lib.mctdh_calc_derivs.argtypes = [vp, DP, DP, DP, DP, C.c_double]
    lib.mctdh_rkqs.argtypes = [vp, DP, DP, DP, DP, C.c_double, C.c_double, DP, DP, C.c_int64]
    lib.mctdh_cmf2.argtypes = [vp, DP, DP, C.c_double, C.c_double, DP, DP]
    lib.mctdh_rk_attempt.argtypes = [vp, DP, DP, DP, DP, C.c_double, C.c_double, C.c_int64, DP]
    lib.mctdh_cmf2_attempt.argtypes = [vp, DP, DP, C.c_double, C.c_double, DP]
    lib.mctdh_set_state.argtypes = [vp, DP, DP, C.c_int64]
    lib.mctdh_get_state.argtypes = [vp, DP, DP]
    lib.mctdh_propagate.argtypes = [vp, C.c_int64, C.c_double, DP, DP, I64P, I64P, I64P]
    lib.mctdh_observables.argtypes = [vp, C.c_double, DP, DP, DP, DP, DP]
    lib.mctdh_norm_wf.argtypes = [vp, DP, DP, DP]
    lib.mctdh_expect.argtypes = [vp, DP]
    lib.mctdh_packets.argtypes = [vp, DP, DP]
    lib.mctdh_device_bytes.argtypes = [vp, I64P]
    lib.mctdh_natpop.argtypes = [vp, DP, DP, DP]
    lib.mctdh_densmat.argtypes = [vp, C.c_int64, C.c_int64, DP]
    lib.mctdh_density.argtypes = [vp, C.c_int64, DP, C.c_int64, C.c_double, C.c_double, DP, DP]
    lib.mctdh_wf_ovl.argtypes = [vp, DP, DP, DP, DP, DP, DP]
    lib.mctdh_launch_count.argtypes = [vp]
    lib.mctdh_tensor_core_status.argtypes = [I64P, I64P]
    lib.mctdh_tensor_core_config.argtypes = [C.c_int64, C.c_int64]
    lib.mctdh_ens_autotune.argtypes = [vp, C.c_int64]
    lib.mctdh_ens_tuning.argtypes = [vp, I64P, I64P, I64P, DP, DP, I64P]
    lib.mctdh_ens_eom_cost.argtypes = [vp, DP, DP]
    lib.mctdh_ens_persistent.argtypes = [vp, I64P, I64P]
    lib.mctdh_step.argtypes = [vp, C.c_int64, C.c_double, C.c_double, DP, DP, I64P]
    lib.mctdh_event_record.argtypes = [vp, C.c_int64]
    lib.mctdh_event_elapsed.argtypes = [vp, C.c_int64, C.c_int64, DP]
    lib.mctdh_profile.argtypes = [vp, C.c_int64]
    lib.mctdh_timing.argtypes = [vp, C.c_int64]
    lib.mctdh_timing_read.argtypes = [vp, C.c_int64, I64P, DP]
    lib.mctdh_write_timings.argtypes = [vp, C.c_char_p, C.c_double]
    lib.mctdh_counters.argtypes = [vp, I64P, I64P, I64P]
    lib.mctdh_fp64_peak.argtypes = [DP]
    FP = C.POINTER(C.c_float)
    lib.mctdh_mlp_create.argtypes = [I64P, C.c_int64, C.c_uint64, C.POINTER(vp)]
    lib.mctdh_mlp_destroy.argtypes = [vp]
    lib.mctdh_mlp_nparams.argtypes = [vp, I64P]
    lib.mctdh_mlp_set_params.argtypes = [vp, FP]
    lib.mctdh_mlp_get_params.argtypes = [vp, FP]
    lib.mctdh_mlp_predict.argtypes = [vp, FP, FP, C.c_int64]
    lib.mctdh_mlp_grad.argtypes = [vp, FP, FP, C.c_int64, FP, DP]
    lib.mctdh_mlp_train.argtypes = [vp, FP, FP, C.c_int64, C.c_int64, C.c_int64, C.c_double, DP]
    for name in ("mctdh_mlp_create", "mctdh_mlp_destroy", "mctdh_mlp_nparams", "mctdh_mlp_set_params",
                 "mctdh_mlp_get_params", "mctdh_mlp_predict", "mctdh_mlp_grad", "mctdh_mlp_train"):
        getattr(lib, name).restype = C.c_int64
    lib.mctdh_mfx_size.argtypes = [vp, I64P]
    lib.mctdh_mfx_record.argtypes = [vp, C.c_int64]
    lib.mctdh_mfx_fetch.argtypes = [vp, C.c_int64, DP, DP, DP, DP, I64P]
    lib.mctdh_mfx_attach.argtypes = [vp, vp, DP, DP, C.c_double]
    lib.mctdh_mfx_stats.argtypes = [vp, I64P, I64P, I64P, DP]
    lib.mctdh_mfx_predict.argtypes = [vp, DP, DP, C.c_double, C.c_double, DP, DP]
    lib.mctdh_mfx_orders.argtypes = [vp, C.c_int64, C.c_int64]
    lib.mctdh_mfx_gate.argtypes = [vp, C.c_double]
    lib.mctdh_mfx_log.argtypes = [vp, C.c_int64, DP, I64P]
    lib.mctdh_ens_create.argtypes = [vp, C.c_int64, C.POINTER(vp)]
    lib.mctdh_ens_destroy.argtypes = [vp]
    lib.mctdh_ens_set_state.argtypes = [vp, C.c_int64, DP, DP, C.c_int64]
    lib.mctdh_ens_get_state.argtypes = [vp, C.c_int64, DP, DP]
    lib.mctdh_ens_calc_derivs.argtypes = [vp]
    lib.mctdh_ens_get_derivs.argtypes = [vp, C.c_int64, DP, DP]
    lib.mctdh_ens_propagate.argtypes = [vp, C.c_int64, C.c_double, DP, DP, I64P, I64P]
    lib.mctdh_ens_observables.argtypes = [vp, C.c_int64, DP, DP, DP, DP, DP]
    lib.mctdh_ens_counters.argtypes = [vp, I64P, I64P, I64P]
    lib.mctdh_ens_stream.argtypes = [vp, C.POINTER(vp)]
    lib.mctdh_ens_last_error.argtypes = [vp]
    lib.mctdh_ens_last_error.restype = C.c_char_p
    for name in ("mctdh_ens_create", "mctdh_ens_destroy", "mctdh_ens_set_state", "mctdh_ens_get_state",
                 "mctdh_ens_calc_derivs", "mctdh_ens_get_derivs", "mctdh_ens_propagate", "mctdh_ens_observables",
                 "mctdh_ens_counters", "mctdh_ens_stream", "mctdh_ens_autotune", "mctdh_ens_tuning", "mctdh_ens_eom_cost", "mctdh_ens_persistent",
                 "mctdh_tensor_core_status", "mctdh_tensor_core_config"):
        getattr(lib, name).restype = C.c_int64
    for name in ("mctdh_mfx_size", "mctdh_mfx_record", "mctdh_mfx_fetch", "mctdh_mfx_attach", "mctdh_mfx_stats",
                 "mctdh_mfx_predict", "mctdh_mfx_log", "mctdh_mfx_orders", "mctdh_mfx_gate",
                 "mctdh_timing", "mctdh_timing_read", "mctdh_write_timings"):
        getattr(lib, name).restype = C.c_int64
    lib.mctdh_density_matrix_noalloc.argtypes = [C.c_void_p, I64P, C.c_int64, C.c_int64, C.c_void_p,
                                                 C.c_int64, C.c_void_p]
    lib.mctdh_profile_read.argtypes = [vp, C.c_int64, DP, I64P, DP, DP]
    lib.mctdh_last_error.argtypes = [vp]
    lib.mctdh_last_error.restype = C.c_char_p
    for name in ("mctdh_create", "mctdh_destroy", "mctdh_calc_derivs", "mctdh_rkqs", "mctdh_cmf2",
                 "mctdh_rk_attempt", "mctdh_cmf2_attempt",
                 "mctdh_set_state", "mctdh_get_state", "mctdh_propagate", "mctdh_observables",
                 "mctdh_norm_wf", "mctdh_wf_ovl", "mctdh_launch_count", "mctdh_step",
                 "mctdh_expect", "mctdh_natpop", "mctdh_densmat", "mctdh_density", "mctdh_packets", "mctdh_device_bytes",
                 "mctdh_event_record", "mctdh_event_elapsed", "mctdh_profile", "mctdh_profile_read",
                 "mctdh_counters", "mctdh_fp64_peak", "mctdh_density_matrix_noalloc"):
        getattr(lib, name).restype = C.c_int64
    _lib = lib
    return lib


EXPORTED = ["mctdh_create", "mctdh_destroy", "mctdh_calc_derivs", "mctdh_rkqs", "mctdh_cmf2",
            "mctdh_rk_attempt", "mctdh_cmf2_attempt",
            "mctdh_set_state", "mctdh_get_state", "mctdh_propagate", "mctdh_observables",
            "mctdh_norm_wf", "mctdh_wf_ovl", "mctdh_launch_count", "mctdh_last_error", "mctdh_step",
            "mctdh_expect", "mctdh_natpop", "mctdh_densmat", "mctdh_density", "mctdh_packets", "mctdh_device_bytes",
            "mctdh_event_record", "mctdh_event_elapsed", "mctdh_profile", "mctdh_profile_read",
            "mctdh_counters", "mctdh_fp64_peak", "mctdh_density_matrix_noalloc", "mctdh_tensor_core_status",
            "mctdh_tensor_core_config", "mctdh_ens_autotune", "mctdh_ens_tuning", "mctdh_ens_eom_cost",
            "mctdh_ens_persistent",
            "mctdh_mlp_create", "mctdh_mlp_destroy", "mctdh_mlp_nparams", "mctdh_mlp_set_params",
            "mctdh_mlp_get_params", "mctdh_mlp_predict", "mctdh_mlp_grad", "mctdh_mlp_train",
            "mctdh_mfx_size", "mctdh_mfx_record", "mctdh_mfx_fetch", "mctdh_mfx_attach", "mctdh_mfx_stats",
            "mctdh_mfx_predict", "mctdh_mfx_log", "mctdh_mfx_orders", "mctdh_mfx_gate",
            "mctdh_timing", "mctdh_timing_read", "mctdh_write_timings",
            "mctdh_ens_create", "mctdh_ens_destroy", "mctdh_ens_set_state", "mctdh_ens_get_state",
            "mctdh_ens_calc_derivs", "mctdh_ens_get_derivs", "mctdh_ens_propagate", "mctdh_ens_observables",
            "mctdh_ens_counters", "mctdh_ens_stream", "mctdh_ens_last_error"]

KERNEL_CLASSES = ["mode_product", "hole_contract", "reduce", "h1_spf_ops", "reg_inverse", "term_sum",
                  "spf_derivative", "elementwise", "gaussian_block"]


def _i64(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.int64))


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64))


def _ptr(a: np.ndarray, t=C.c_double):
    return a.ctypes.data_as(C.POINTER(t))


def build_setup(model: Model, precision: int = 0, warm_start: bool = True) -> Tuple[Setup, list]:
    """Flatten the model into the C struct (Fortran column-major conventions)."""
    keep: list = []
    nm, ns, nd = model.nmodes, model.nstates, model.ndof
    maxdof = max(len(d) for d in model.mode_dofs)

    def I(a):
        arr = _i64(a)
        keep.append(arr)
        return _ptr(arr, C.c_int64)

    def F(a):
        arr = _f64(a)
        keep.append(arr)
        return _ptr(arr)

    idof = np.full((maxdof, nm), -1, dtype=np.int64)
    for m in range(nm):
        idof[:len(model.mode_dofs[m]), m] = model.mode_dofs[m]
    grid_parts, grid_off, mat_parts, mat_off = [], [], [], []
    go = mo = 0
    for d in range(nd):
        if model.dvr_type[d] == "gwp":
            grid_off.append(-1)
            mat_off.append(-1)
            continue
        g = model.grid[d]
        grid_parts.append(g)
        grid_off.append(go)
        go += len(g)
        mats = np.concatenate([model.d1[d].reshape(-1, order="F"), model.d2[d].reshape(-1, order="F"),
                               model.xd1[d].reshape(-1, order="F")])
        mat_parts.append(mats)
        mat_off.append(mo)
        mo += len(mats)
    grid = np.concatenate(grid_parts) if grid_parts else np.zeros(1)
    mats = np.concatenate(mat_parts) if mat_parts else np.zeros(1)
    w = 2 + maxdof
    oper = np.zeros((w, model.nopermax, nm), dtype=np.int64)
    for m in range(nm):
        for k, (l, r, dops) in enumerate(model.oper[m]):
            oper[0, k, m] = l
            oper[1, k, m] = r
            oper[2:2 + len(dops), k, m] = dops
    # dissipative terms follow the Hamiltonian's: kind 1 (aeExtra, its type-1
    # operator), kind 2 (i aeD2 aeExtra)
    kinds = [0] * model.nham
    diss1_of = [-1] * model.nham
    coeffs = list(model.ae)
    lhs, rhs = list(model.lhs_el), list(model.rhs_el)
    iop_cols, skip_cols = [model.ioper], [model.skip_term]
    dissipation = getattr(model, "dissipation", [])
    for ty in (1, 2):
        for j, idx in enumerate(model.diss1 if ty == 1 else model.diss2):
            for term in dissipation[idx][2]:
                kinds.append(ty)
                diss1_of.append(j if ty == 1 else -1)
                coeffs.append(complex(term.coeff) if ty == 1 else 1j * model.aeD2[j] * complex(term.coeff))
                lhs.append(term.lhs)
                rhs.append(term.rhs)
            iop_cols.append(model.ioper_diss[idx])
            skip_cols.append(model.skip_diss[idx])
    nterm = len(kinds)
    coeffs = np.asarray(coeffs, dtype=np.complex128)
    ae = np.empty(2 * nterm)
    ae[0::2] = coeffs.real
    ae[1::2] = coeffs.imag
    gwpa = getattr(model, "gwpa", None)
    if gwpa is None or gwpa.size == 0:
        gwpa = np.zeros(1)
    else:
        # GWPa(maxdof, ns00max, nmodgwp): pad the DOF axis to maxdof
        g = np.zeros((maxdof, max(int(model.ns00max), 1), gwpa.shape[2]))
        g[:gwpa.shape[0], :gwpa.shape[1], :] = gwpa
        gwpa = g
    s = Setup()
    s.nstates, s.nmodes, s.ndof, s.nham, s.maxdof = ns, nm, nd, nterm, maxdof
    s.nspf = I(model.nspf.reshape(-1, order="F"))
    s.nmodedof = I([len(d) for d in model.mode_dofs])
    s.idof = I(idof.reshape(-1, order="F"))
    s.multiset = I([1 if x else 0 for x in model.multiset])
    s.is_gwp = I([1 if x else 0 for x in model.is_gwp_mode])
    s.ngp = I(model.ngp)
    s.dvr_grid = F(grid)
    s.dvr_grid_off = I(grid_off)
    s.dvr_mats = F(mats)
    s.dvr_mat_off = I(mat_off)
    s.ae = F(ae)
    s.lhs_el = I(lhs)
    s.rhs_el = I(rhs)
    s.nopermax = model.nopermax
    s.noper = I([len(o) for o in model.oper])
    s.oper = I(oper.reshape(-1, order="F"))
    s.ioper = I(np.concatenate(iop_cols, axis=1).reshape(-1, order="F"))
    s.is_identity = I(model.is_identity.astype(np.int64).reshape(-1, order="F"))
    s.skip_term = I(np.concatenate(skip_cols, axis=1).astype(np.int64).reshape(-1, order="F"))
    s.ipsispf = I(model.ipsispf.reshape(-1, order="F"))
    s.dimpsi = model.dimpsi
    s.gwpa = F(np.asarray(gwpa).reshape(-1, order="F"))
    s.ns00max = model.ns00max
    s.eps_rho, s.eps_ovl, s.eps_C = model.eps_rho, model.eps_ovl, model.eps_C
    s.eps_int, s.eps_A, s.eps_psi = model.eps_int, model.eps_A, model.eps_psi
    s.min_stepsize, s.writetime = model.min_stepsize, model.tout
    s.der_factor_re, s.der_factor_im = model.der_factor.real, model.der_factor.imag
    s.int_type_psi = model.int_type_psi
    s.precision = precision
    s.reginv_cold = 0 if warm_start else 1
    s.int_order = getattr(model, "int_order", 4)
    s.int_par1 = getattr(model, "int_par1", 0)
    expect = getattr(model, "expect", [])
    s.nexpect = len(expect)
    if expect:
        terms = [t for op in expect for t in op]
        eae = np.empty(2 * len(terms))
        eae[0::2] = [t.coeff.real for t in terms]
        eae[1::2] = [complex(t.coeff).imag for t in terms]
        s.expect_nterms = I([len(op) for op in expect])
        s.expect_ae = F(eae)
        s.expect_lhs = I([t.lhs for t in terms])
        s.expect_rhs = I([t.rhs for t in terms])
        s.expect_ioper = I(np.concatenate(model.ioper_expect, axis=1).reshape(-1, order="F"))
    s.npackets = getattr(model, "npackets", 1)
    s.eps_pop = getattr(model, "eps_pop", 1e-6)
    if nterm > model.nham:
        s.term_kind = I(kinds)
        s.term_diss1 = I(diss1_of)
        s.ndiss1 = len(model.diss1)
        s.diss1_ae = F(model.aeD1 if model.aeD1 else [0.0])
    # parametrised operators: gridOper(ngpmax, nopparam, ndof), and operDVR of
    # the Legendre dofs
    nop = len(getattr(model, "op_params", []))
    s.nopparam = nop
    s.ngpmax = max(model.ngp) if model.ngp else 0
    if nop:
        go_arr = np.zeros((s.ngpmax, nop, nd))
        for (d, j), v in model.grid_oper.items():
            go_arr[:len(v), j - 1, d] = v
        s.grid_oper = F(go_arr.reshape(-1, order="F"))
    oper_dvr = getattr(model, "oper_dvr", {})
    if oper_dvr:
        parts, offs, o = [], [], 0
        for d in range(nd):
            if d in oper_dvr:
                parts.append(oper_dvr[d].reshape(-1, order="F"))
                offs.append(o)
                o += parts[-1].size
            else:
                offs.append(-1)
        s.oper_dvr = F(np.concatenate(parts))
        s.oper_dvr_off = I(offs)
    return s, keep


def _cbuf(x: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(x, dtype=np.complex128))


class GpuCore:
    """One device context for one model (one CUDA stream on the current device)."""

    def __init__(self, model: Model, precision: int = 0, warm_start: bool = True):
        self.lib = load_library()
        self.model = model
        setup, self._keep = build_setup(model, precision, warm_start)
        h = C.c_void_p()
        rc = self.lib.mctdh_create(C.byref(setup), C.byref(h))
        if rc != 0:
            raise MctdhError(rc, self.lib.mctdh_last_error(None).decode())
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.mctdh_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int):
        if rc != 0:
            raise MctdhError(rc, self.lib.mctdh_last_error(self.h).decode())

    # -- reference-shaped calls on host buffers --
    def calc_derivs(self, A, psi, t: float = 0.0):
        A, psi = _cbuf(A), _cbuf(psi)
        dA = np.empty_like(A)
        dpsi = np.empty_like(psi)
        self._check(self.lib.mctdh_calc_derivs(self.h, _ptr(A), _ptr(psi), _ptr(dA), _ptr(dpsi), t))
        return dA, dpsi

    def rkqs(self, A, psi, dA, dpsi, t: float, htry: float, method: int = 1):
        A, psi, dA, dpsi = _cbuf(A).copy(), _cbuf(psi).copy(), _cbuf(dA).copy(), _cbuf(dpsi).copy()
        hdid, hnext = C.c_double(), C.c_double()
        self._check(self.lib.mctdh_rkqs(self.h, _ptr(A), _ptr(psi), _ptr(dA), _ptr(dpsi), t, htry,
                                        C.byref(hdid), C.byref(hnext), method))
        return A, psi, dA, dpsi, hdid.value, hnext.value

    def cmf2(self, A, psi, t: float, htry: float):
        A, psi = _cbuf(A).copy(), _cbuf(psi).copy()
        hdid, hnext = C.c_double(), C.c_double()
        self._check(self.lib.mctdh_cmf2(self.h, _ptr(A), _ptr(psi), t, htry, C.byref(hdid), C.byref(hnext)))
        return A, psi, hdid.value, hnext.value

    def rk_attempt(self, A, psi, dA, dpsi, t: float, dt: float, method: int = 1):
        """Fixed-length rkck/rkdp attempt (step replay): returns (A, psi, dA, dpsi, errmax)."""
        A, psi, dA, dpsi = _cbuf(A).copy(), _cbuf(psi).copy(), _cbuf(dA).copy(), _cbuf(dpsi).copy()
        err = C.c_double()
        self._check(self.lib.mctdh_rk_attempt(self.h, _ptr(A), _ptr(psi), _ptr(dA), _ptr(dpsi), t, dt,
                                              method, C.byref(err)))
        return A, psi, dA, dpsi, err.value

    def cmf2_attempt(self, A, psi, t: float, h: float):
        """One CMF2 attempt of length h completed as accepted (step replay)."""
        A, psi = _cbuf(A).copy(), _cbuf(psi).copy()
        err = C.c_double()
        self._check(self.lib.mctdh_cmf2_attempt(self.h, _ptr(A), _ptr(psi), t, h, C.byref(err)))
        return A, psi, err.value

    def norm_wf(self, A, psi) -> float:
        A, psi = _cbuf(A), _cbuf(psi)
        out = C.c_double()
        self._check(self.lib.mctdh_norm_wf(self.h, _ptr(A), _ptr(psi), C.byref(out)))
        return out.value

    def wf_ovl(self, A1, psi1, A2, psi2) -> complex:
        A1, psi1, A2, psi2 = _cbuf(A1), _cbuf(psi1), _cbuf(A2), _cbuf(psi2)
        re, im = C.c_double(), C.c_double()
        self._check(self.lib.mctdh_wf_ovl(self.h, _ptr(A1), _ptr(psi1), _ptr(A2), _ptr(psi2),
                                          C.byref(re), C.byref(im)))
        return complex(re.value, im.value)

    # -- device-resident propagation --
    def set_state(self, A, psi, as_start: bool = True):
        A, psi = _cbuf(A), _cbuf(psi)
        self._check(self.lib.mctdh_set_state(self.h, _ptr(A), _ptr(psi), 1 if as_start else 0))

    def device_bytes(self) -> int:
        """Device memory held by the context (bytes)."""
        b = C.c_int64()
        self._check(self.lib.mctdh_device_bytes(self.h, C.byref(b)))
        return int(b.value)

    def packets(self):
        """Packet populations (normalised, decreasing) and the entropy of the
        resident mixture (output.f90:44-60)."""
        w = np.empty(max(1, getattr(self.model, "npackets", 1)))
        e = C.c_double()
        self._check(self.lib.mctdh_packets(self.h, w.ctypes.data_as(DP), C.byref(e)))
        return w, e.value

    def get_state(self):
        A = np.empty(self.model.naconftot * getattr(self.model, "npackets", 1), dtype=np.complex128)
        psi = np.empty(self.model.dimpsi, dtype=np.complex128)
        self._check(self.lib.mctdh_get_state(self.h, _ptr(A), _ptr(psi)))
        return A, psi

    def observables(self, t: float) -> Dict:
        e, nrm, ar, ai = C.c_double(), C.c_double(), C.c_double(), C.c_double()
        pop = np.zeros(self.model.nstates)
        self._check(self.lib.mctdh_observables(self.h, t, C.byref(e), _ptr(pop), C.byref(nrm),
                                               C.byref(ar), C.byref(ai)))
        return dict(t=t, pop=pop, norm=nrm.value, energy=e.value, auto=complex(ar.value, ai.value))

    def expect(self) -> np.ndarray:
        """Expectation values of the model's expectation operators for the resident
        state (Expectation, output.f90:449-500)."""
        out = np.zeros(max(len(getattr(self.model, "expect", [])), 1), dtype=np.complex128)
        self._check(self.lib.mctdh_expect(self.h, out.ctypes.data_as(DP)))
        return out[:len(getattr(self.model, "expect", []))]

    def natpop(self):
        """Natural populations (nspfmax, nmodes, nstates), decreasing; gross Gaussian
        populations and population errors (ns00max, nmodgwp, nstates) (output.f90:88-140)."""
        m = self.model
        nat = np.zeros((int(m.nspf.max()), m.nmodes, m.nstates), order="F")
        shape = (max(int(m.ns00max), 1), len(m.modes_gwp), m.nstates)
        ggp, perr = np.zeros(shape, order="F"), np.zeros(shape, order="F")
        self._check(self.lib.mctdh_natpop(self.h, nat.ctypes.data_as(DP), ggp.ctypes.data_as(DP),
                                          perr.ctypes.data_as(DP)))
        return nat, ggp, perr

    def densmat(self, mode: int, state: int) -> np.ndarray:
        """rho(mode, state) of the resident state (the densmat file, output.f90:276-300)."""
        n = int(self.model.nspf[mode, state])
        rho = np.zeros((n, n), dtype=np.complex128, order="F")
        self._check(self.lib.mctdh_densmat(self.h, mode, state, rho.ctypes.data_as(DP)))
        return rho

    def density(self, dof: int):
        """Calc_Density (output.f90:332-445) along dof: (density, basis populations),
        each (ngp, nstates); the populations are zero for Gaussian DOFs."""
        m = self.model
        ng = m.ngp[dof]
        dens = np.zeros((ng, m.nstates), order="F")
        pop = np.zeros((ng, m.nstates), order="F")
        if m.dvr_type[dof] == "gwp":
            x0, x1 = m.dvrpar[dof]
            self._check(self.lib.mctdh_density(self.h, dof, None, 0, x0, x1, dens.ctypes.data_as(DP), None))
        else:
            tr = np.asfortranarray(m.trafo[dof])
            self._check(self.lib.mctdh_density(self.h, dof, tr.ctypes.data_as(DP), ng, 0.0, 0.0,
                                               dens.ctypes.data_as(DP), pop.ctypes.data_as(DP)))
        return dens, pop

    def propagate_interval(self, int_type: int, tnext: float, t: float, step: float):
        tt, ss = C.c_double(t), C.c_double(step)
        ns, na, ne = C.c_int64(), C.c_int64(), C.c_int64()
        self._check(self.lib.mctdh_propagate(self.h, int_type, tnext, C.byref(tt), C.byref(ss),
                                             C.byref(ns), C.byref(na), C.byref(ne)))
        return tt.value, ss.value, ns.value, na.value, ne.value

    def step(self, int_type: int, t: float, htry: float):
        """One accepted step on the resident state: (hdid, hnext, attempts)."""
        hdid, hnext, att = C.c_double(), C.c_double(), C.c_int64()
        self._check(self.lib.mctdh_step(self.h, int_type, t, htry, C.byref(hdid), C.byref(hnext), C.byref(att)))
        return hdid.value, hnext.value, att.value

    def event_record(self, slot: int):
        self._check(self.lib.mctdh_event_record(self.h, slot))

    def event_elapsed(self, s0: int, s1: int) -> float:
        ms = C.c_double()
        self._check(self.lib.mctdh_event_elapsed(self.h, s0, s1, C.byref(ms)))
        return ms.value

    TIMERS = ("CalcDerivs", "normWF/wf_ovl", "Calc_MeanField", "Calc_CY", "Calc_h1mode",
              "Calc_Der_SPF_DVR", "Calc_Der_SPF_GWP", "Lanczos")

    def timing(self, mode: int):
        """The reference's routine timers on CUDA events: 0 off, 1 on, 2 on and reset."""
        self._check(self.lib.mctdh_timing(self.h, mode))

    def timing_read(self) -> Dict[str, Dict]:
        out = {}
        for i, name in enumerate(self.TIMERS):
            n, ms = C.c_int64(), C.c_double()
            self._check(self.lib.mctdh_timing_read(self.h, i + 1, C.byref(n), C.byref(ms)))
            out[name] = dict(calls=n.value, ms=ms.value)
        return out

    def write_timings(self, path: str, walltime_s: float):
        """The reference's `timing` file (timingmod.f90:72-103)."""
        self._check(self.lib.mctdh_write_timings(self.h, path.encode(), float(walltime_s)))

    def profile(self, enable: int):
        self._check(self.lib.mctdh_profile(self.h, enable))

    def profile_read(self) -> Dict[str, Dict]:
        out = {}
        for kid, name in enumerate(KERNEL_CLASSES):
            ms, fl, by = C.c_double(), C.c_double(), C.c_double()
            n = C.c_int64()
            self._check(self.lib.mctdh_profile_read(self.h, kid, C.byref(ms), C.byref(n), C.byref(fl), C.byref(by)))
            out[name] = dict(ms=ms.value, launches=n.value, flops=fl.value, bytes=by.value)
        return out

    def counters(self) -> Dict[str, int]:
        a, b, d = C.c_int64(), C.c_int64(), C.c_int64()
        self._check(self.lib.mctdh_counters(self.h, C.byref(a), C.byref(b), C.byref(d)))
        return dict(launches=a.value, eom=b.value, hb=d.value)

    # -- learned mean-field extrapolation (CMF2) --
    def mfx_size(self) -> int:
        e = C.c_int64()
        self._check(self.lib.mctdh_mfx_size(self.h, C.byref(e)))
        return e.value

    def mfx_record(self, enable: int = 2):
        self._check(self.lib.mctdh_mfx_record(self.h, enable))

    def mfx_fetch(self):
        """Recorded plain-CMF2 steps: (t0[n], h[n], snap0[n, E], snaphalf[n, E])."""
        n = C.c_int64()
        self._check(self.lib.mctdh_mfx_fetch(self.h, 0, None, None, None, None, C.byref(n)))
        E = self.mfx_size()
        k = n.value
        t0, h = np.zeros(k), np.zeros(k)
        s0 = np.zeros((k, E), dtype=np.complex128)
        sh = np.zeros((k, E), dtype=np.complex128)
        if k:
            self._check(self.lib.mctdh_mfx_fetch(self.h, k, _ptr(t0), _ptr(h), _ptr(s0), _ptr(sh), C.byref(n)))
        return t0, h, s0, sh

    def mfx_attach(self, mlp, fscale, tscale, tol: float):
        """Attach a trained extrapolator (None detaches) with its input column scales
        (20) and output column scales (4)."""
        if mlp is None:
            self._check(self.lib.mctdh_mfx_attach(self.h, None, None, None, tol))
        else:
            fs = np.ascontiguousarray(fscale, dtype=np.float64)
            ts = np.ascontiguousarray(tscale, dtype=np.float64)
            if fs.size != 20 or ts.size != 4:
                raise ValueError("fscale needs 20 entries and tscale 4")
            self._check(self.lib.mctdh_mfx_attach(self.h, mlp.h, fs.ctypes.data_as(DP), ts.ctypes.data_as(DP), tol))
            o0, o1 = getattr(mlp, "orders", (4, 4))
            self._check(self.lib.mctdh_mfx_orders(self.h, int(o0), int(o1)))
        self._mlp_ref = mlp

    def mfx_predict(self, hist, ts, tau0, tau1):
        """The attached extrapolator on a given history (5, E) at times ts: the
        predicted snapshots at tau0 (a step start) and tau1 (its half step)."""
        Hs = np.ascontiguousarray(hist, dtype=np.complex128)
        T = np.ascontiguousarray(ts, dtype=np.float64)
        E = Hs.shape[1]
        p0 = np.zeros(E, dtype=np.complex128)
        p1 = np.zeros(E, dtype=np.complex128)
        self._check(self.lib.mctdh_mfx_predict(self.h, Hs.ctypes.data_as(DP), T.ctypes.data_as(DP), tau0, tau1,
                                               p0.ctypes.data_as(DP), p1.ctypes.data_as(DP)))
        return p0, p1

    def mfx_gate(self, gate: float):
        """Extrapolate only after steps whose first attempt had error / tolerance < gate."""
        self._check(self.lib.mctdh_mfx_gate(self.h, float(gate)))

    def mfx_log(self):
        """One row per CMF2 attempt: t, h, error / eps_int, extrapolated, step-end mismatch."""
        n = C.c_int64()
        self._check(self.lib.mctdh_mfx_log(self.h, 0, None, C.byref(n)))
        rows = np.zeros((n.value, 5))
        if n.value:
            self._check(self.lib.mctdh_mfx_log(self.h, n.value, rows.ctypes.data_as(DP), C.byref(n)))
        return rows

    def mfx_stats(self):
        a, b, r, x = C.c_int64(), C.c_int64(), C.c_int64(), C.c_double()
        self._check(self.lib.mctdh_mfx_stats(self.h, C.byref(a), C.byref(b), C.byref(r), C.byref(x)))
        return dict(mlp_steps=a.value, fallbacks=b.value, rejected=r.value, last_rel=x.value)

    def launch_count(self) -> int:
        return int(self.lib.mctdh_launch_count(self.h))

    def propagate(self, A, psi, tfinal: Optional[float] = None, int_type: Optional[int] = None):
        """propagate_wf (propagator.f90:87-146, :257-306) on the device; returns the
        outputs written every tout, like the oracle's ``propagate``."""
        md = self.model
        it = md.int_type if int_type is None else int_type
        self.set_state(A, psi, as_start=True)
        tfin = md.tfinal if tfinal is None else tfinal
        maxtime = tfin + md.tout * 0.1
        t = md.tinit
        step = md.tout * md.eps_int
        outs = []
        stats = dict(steps=0, attempts=0, eom=0)
        while t < maxtime:
            outs.append(self.observables(t))
            t, step, ns, na, ne = self.propagate_interval(it, t + md.tout, t, step)
            stats["steps"] += ns
            stats["attempts"] += na
            stats["eom"] += ne
        self.stats = stats
        return outs


def tensor_core_status() -> Dict[str, int]:
    """Whether the tensor-core kernels are in use (MACAW_GB300_TC) and whether one
    of them gave up waiting for its MMAs since the previous call."""
    lib = load_library()
    en, to = C.c_int64(), C.c_int64()
    rc = lib.mctdh_tensor_core_status(C.byref(en), C.byref(to))
    if rc != 0:
        raise MctdhError(rc, "tensor-core status")
    return {"enabled": en.value, "timeouts": to.value}


def tensor_core_config(min_n: int = 0, stages: int = 0) -> None:
    """Smallest SPF count served by the tensor-core mode product and its pipeline
    stages (0 keeps a setting)."""
    rc = load_library().mctdh_tensor_core_config(min_n, stages)
    if rc != 0:
        raise MctdhError(rc, "tensor-core config")


def fp64_peak_tflops() -> float:
    """Measured FP64 FMA throughput of the current GPU (TFLOP/s)."""
    lib = load_library()
    v = C.c_double()
    rc = lib.mctdh_fp64_peak(C.byref(v))
    if rc != 0:
        raise MctdhError(rc, "FP64 calibration failed")
    return v.value


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.float32))


class Ensemble:
    """Independent wavepackets of uneven shape advanced together (mctdh_ens_*): one
    launch per EOM stage over all members, lockstep adaptive RK."""

    def __init__(self, models, precision: int = 0, autotune: bool = True):
        self.lib = load_library()
        self.models = list(models)
        built = [build_setup(m, precision) for m in self.models]
        self._keep = [b[1] for b in built]
        arr = (Setup * len(built))(*[b[0] for b in built])
        self._arr = arr
        h = C.c_void_p()
        rc = self.lib.mctdh_ens_create(C.cast(arr, C.c_void_p), len(built), C.byref(h))
        if rc != 0:
            raise MctdhError(rc, self.lib.mctdh_ens_last_error(None).decode())
        self.h = h
        if autotune == "persistent":
            self._check(self.lib.mctdh_ens_autotune(self.h, 2))   # planned shapes, persistent CTAs
        elif not autotune:
            self._check(self.lib.mctdh_ens_autotune(self.h, 0))

    def autotune(self):
        """Tune the launch shapes now, on the members' current states."""
        self._check(self.lib.mctdh_ens_autotune(self.h, 1))
        return self.tuning()

    def tuning(self) -> Dict:
        tpb, cap, tc, cand = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int64()
        ms, ms0 = C.c_double(), C.c_double()
        self._check(self.lib.mctdh_ens_tuning(self.h, C.byref(tpb), C.byref(cap), C.byref(tc), C.byref(ms),
                                              C.byref(ms0), C.byref(cand)))
        pp, ph = C.c_int64(), C.c_int64()
        self._check(self.lib.mctdh_ens_persistent(self.h, C.byref(pp), C.byref(ph)))
        return dict(tiles_per_block=tpb.value, block_cap=cap.value, tensor_cores=tc.value, eom_ms=ms.value,
                    default_eom_ms=ms0.value, candidates=cand.value, persistent_prod_ctas=pp.value,
                    persistent_hole_ctas=ph.value)

    def eom_cost(self) -> Dict:
        """Algorithmic FLOPs and bytes of one merged EOM evaluation."""
        fl, by = C.c_double(), C.c_double()
        self._check(self.lib.mctdh_ens_eom_cost(self.h, C.byref(fl), C.byref(by)))
        return dict(flops=fl.value, bytes=by.value)

    def close(self):
        if getattr(self, "h", None):
            self.lib.mctdh_ens_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int):
        if rc != 0:
            raise MctdhError(rc, self.lib.mctdh_ens_last_error(self.h).decode())

    def __len__(self):
        return len(self.models)

    def set_state(self, i: int, A, psi, as_start: bool = True):
        A, psi = _cbuf(A), _cbuf(psi)
        self._check(self.lib.mctdh_ens_set_state(self.h, i, _ptr(A), _ptr(psi), 1 if as_start else 0))

    def get_state(self, i: int):
        m = self.models[i]
        A = np.empty(m.naconftot, dtype=np.complex128)
        psi = np.empty(m.dimpsi, dtype=np.complex128)
        self._check(self.lib.mctdh_ens_get_state(self.h, i, _ptr(A), _ptr(psi)))
        return A, psi

    def calc_derivs(self):
        """EOM of every member at its resident state; returns [(dA, dpsi)]."""
        self._check(self.lib.mctdh_ens_calc_derivs(self.h))
        out = []
        for i, m in enumerate(self.models):
            dA = np.empty(m.naconftot, dtype=np.complex128)
            dpsi = np.empty(m.dimpsi, dtype=np.complex128)
            self._check(self.lib.mctdh_ens_get_derivs(self.h, i, _ptr(dA), _ptr(dpsi)))
            out.append((dA, dpsi))
        return out

    def propagate(self, int_type: int, tnext: float, t, step):
        """Advance every member to tnext; t and step (arrays, per member) are updated
        in place.  Returns (lockstep rounds, EOM evaluations)."""
        T = np.ascontiguousarray(t, dtype=np.float64)
        S = np.ascontiguousarray(step, dtype=np.float64)
        nr, ne = C.c_int64(), C.c_int64()
        self._check(self.lib.mctdh_ens_propagate(self.h, int_type, tnext, T.ctypes.data_as(DP),
                                                 S.ctypes.data_as(DP), C.byref(nr), C.byref(ne)))
        t[:] = T
        step[:] = S
        return nr.value, ne.value

    def observables(self, i: int, t: float = 0.0):
        m = self.models[i]
        e, nrm, ar, ai = C.c_double(), C.c_double(), C.c_double(), C.c_double()
        pop = np.zeros(m.nstates)
        self._check(self.lib.mctdh_ens_observables(self.h, i, C.byref(e), pop.ctypes.data_as(DP), C.byref(nrm),
                                                   C.byref(ar), C.byref(ai)))
        return dict(t=t, pop=pop, norm=nrm.value, energy=e.value, auto=complex(ar.value, ai.value))

    def counters(self):
        a, b, r = C.c_int64(), C.c_int64(), C.c_int64()
        self._check(self.lib.mctdh_ens_counters(self.h, C.byref(a), C.byref(b), C.byref(r)))
        return dict(launches=a.value, eom=b.value, rounds=r.value)

    def stream(self) -> int:
        p = C.c_void_p()
        self._check(self.lib.mctdh_ens_stream(self.h, C.byref(p)))
        return p.value or 0


class Mlp:
    """The extrapolator network on the GPU (BF16 weights/activations, FP32 accumulation)."""

    def __init__(self, widths=(8, 256, 256, 256, 4), seed: int = 1):
        self.lib = load_library()
        self.widths = tuple(int(w) for w in widths)
        w = _i64(self.widths)
        h = C.c_void_p()
        rc = self.lib.mctdh_mlp_create(_ptr(w, C.c_int64), len(self.widths) - 1, seed, C.byref(h))
        if rc != 0:
            raise MctdhError(rc, self.lib.mctdh_last_error(None).decode())
        self.h = h
        n = C.c_int64()
        self.lib.mctdh_mlp_nparams(self.h, C.byref(n))
        self.nparams = n.value

    def close(self):
        if getattr(self, "h", None):
            self.lib.mctdh_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != 0:
            raise MctdhError(rc, self.lib.mctdh_last_error(None).decode())

    def get_params(self) -> np.ndarray:
        p = np.zeros(self.nparams, dtype=np.float32)
        self._check(self.lib.mctdh_mlp_get_params(self.h, _ptr(p, C.c_float)))
        return p

    def set_params(self, p):
        p = _f32(p)
        self._check(self.lib.mctdh_mlp_set_params(self.h, _ptr(p, C.c_float)))

    def predict(self, X) -> np.ndarray:
        X = _f32(X)
        Y = np.zeros((X.shape[0], self.widths[-1]), dtype=np.float32)
        self._check(self.lib.mctdh_mlp_predict(self.h, _ptr(X, C.c_float), _ptr(Y, C.c_float), X.shape[0]))
        return Y

    def grad(self, X, T):
        X, T = _f32(X), _f32(T)
        g = np.zeros(self.nparams, dtype=np.float32)
        loss = C.c_double()
        self._check(self.lib.mctdh_mlp_grad(self.h, _ptr(X, C.c_float), _ptr(T, C.c_float), X.shape[0],
                                            _ptr(g, C.c_float), C.byref(loss)))
        return loss.value, g

    def train(self, X, T, batch=4096, epochs=10, lr=1e-3) -> float:
        X, T = _f32(X), _f32(T)
        loss = C.c_double()
        self._check(self.lib.mctdh_mlp_train(self.h, _ptr(X, C.c_float), _ptr(T, C.c_float), X.shape[0], batch,
                                             epochs, lr, C.byref(loss)))
        return loss.value
