"""The allocation-free density-matrix entry point (mctdh_density_matrix_noalloc).

It is for callers that cannot call cudaMalloc where they need the result, such
as code running under CUDA stream capture or a driver with a fixed device-memory
budget: they pass device buffers for A and rho, and the block partials live in a
scratch area the library reserves once per GPU.  The test calls it through the
C-ABI twice in a row, on different modes and states, and checks each result
against the existing context-based entry point (mctdh_norm_wf: for orthonormal
SPFs <Psi|Psi> = sum over states of Tr rho_m) and against the oracle's
contraction, within the EOM tolerance of the GPU parity tests.
"""
import ctypes as C

import numpy as np
import pytest

from oracle.mctdh import hole_contract
from tests.helpers import small_qvc, random_state

pytestmark = pytest.mark.gpu

RTOL = 1e-11


def _call(lib, torch, model, A, s, mode):
    nspf = np.ascontiguousarray(model.nspf[:, s].astype(np.int64))
    a_dev = torch.from_numpy(np.ascontiguousarray(model.a_state(A, s).reshape(-1, order="F"))).cuda()
    n = int(nspf[mode])
    ld = n + 1
    rho_dev = torch.full((n * ld,), complex(np.nan, np.nan), dtype=torch.complex128, device="cuda")
    rc = lib.mctdh_density_matrix_noalloc(C.c_void_p(a_dev.data_ptr()), nspf.ctypes.data_as(C.POINTER(C.c_int64)),
                                          model.nmodes, mode, C.c_void_p(rho_dev.data_ptr()), ld, None)
    assert rc == 0, lib.mctdh_last_error(None).decode()
    torch.cuda.synchronize()
    return rho_dev.cpu().numpy().reshape((ld, n), order="F")[:n, :]


def test_density_matrix_noalloc_matches_existing_entry_point():
    torch = pytest.importorskip("torch")
    from macaw_gb300.capi import GpuCore
    model = small_qvc()
    A, psi = random_state(model, seed=17)
    gpu = GpuCore(model)
    norm = gpu.norm_wf(A, psi)
    lib = gpu.lib
    for mode in (0, model.nmodes - 1):     # two calls in a row on different shapes
        tr = 0.0
        for s in range(model.nstates):
            rho = _call(lib, torch, model, A, s, mode)
            X = model.a_state(A, s)
            R = hole_contract(X, X, mode)
            ref = 0.5 * (R + R.conj().T)
            assert np.linalg.norm(rho - ref) <= RTOL * np.linalg.norm(ref)
            tr += float(np.trace(rho).real)
        assert abs(tr - norm) <= RTOL * abs(norm)
    gpu.close()


def _call_tensor(lib, torch, X, mode):
    """The entry point on one tensor X (Fortran order), rho with ld = n + 1."""
    nspf = np.array(X.shape, dtype=np.int64)
    a_dev = torch.from_numpy(np.ascontiguousarray(X.reshape(-1, order="F"))).cuda()
    n = int(nspf[mode])
    ld = n + 1
    rho_dev = torch.full((n * ld,), complex(np.nan, np.nan), dtype=torch.complex128, device="cuda")
    rc = lib.mctdh_density_matrix_noalloc(C.c_void_p(a_dev.data_ptr()), nspf.ctypes.data_as(C.POINTER(C.c_int64)),
                                          len(nspf), mode, C.c_void_p(rho_dev.data_ptr()), ld, None)
    assert rc == 0, lib.mctdh_last_error(None).decode()
    torch.cuda.synchronize()
    return rho_dev.cpu().numpy().reshape((ld, n), order="F")[:n, :]


def _herm_ref(X, mode):
    R = hole_contract(X, X, mode)
    return 0.5 * (R + R.conj().T)


def test_density_matrix_noalloc_wide_mode_and_block_cap():
    """The branches the small model does not reach: a contracted mode of 32 SPFs
    (1,024 pairs, four per thread), a tensor of 2,000 fibre tiles whose block
    count is capped at the scratch area's 128 partials, then a small case again
    (a stale partial of the large call would show up there)."""
    torch = pytest.importorskip("torch")
    from macaw_gb300.capi import load_library
    lib = load_library()
    rng = np.random.default_rng(23)

    def rnd(shape):
        return rng.normal(size=shape) + 1j * rng.normal(size=shape)

    cases = [((24, 32, 20), 1), ((40, 40, 40, 6), 3), ((20, 40, 40, 6), 0), ((3, 4, 2), 1)]
    for shape, mode in cases:
        X = np.asfortranarray(rnd(shape))
        rho = _call_tensor(lib, torch, X, mode)
        ref = _herm_ref(X, mode)
        assert np.linalg.norm(rho - ref) <= RTOL * np.linalg.norm(ref), (shape, mode)


def test_density_matrix_noalloc_rejects_oversized_mode():
    torch = pytest.importorskip("torch")
    from macaw_gb300.capi import load_library
    lib = load_library()
    nspf = np.array([4, 33, 2], dtype=np.int64)
    a_dev = torch.zeros(int(np.prod(nspf)), dtype=torch.complex128, device="cuda")
    rho_dev = torch.zeros(33 * 33, dtype=torch.complex128, device="cuda")
    rc = lib.mctdh_density_matrix_noalloc(C.c_void_p(a_dev.data_ptr()), nspf.ctypes.data_as(C.POINTER(C.c_int64)),
                                          3, 1, C.c_void_p(rho_dev.data_ptr()), 33, None)
    assert rc == -7
    assert b"exceed the maximum" in lib.mctdh_last_error(None)
    host = np.zeros(16, dtype=np.complex128)
    nspf = np.array([4, 4], dtype=np.int64)
    rc = lib.mctdh_density_matrix_noalloc(host.ctypes.data_as(C.c_void_p), nspf.ctypes.data_as(C.POINTER(C.c_int64)),
                                          2, 0, C.c_void_p(rho_dev.data_ptr()), 4, None)
    assert rc == -7
    if torch.cuda.device_count() > 1:
        # a buffer of another GPU is refused on the host; nothing is launched
        other = torch.zeros(16, dtype=torch.complex128, device="cuda:1")
        rc = lib.mctdh_density_matrix_noalloc(C.c_void_p(other.data_ptr()),
                                              nspf.ctypes.data_as(C.POINTER(C.c_int64)),
                                              2, 0, C.c_void_p(rho_dev.data_ptr()), 4, None)
        assert rc == -7
