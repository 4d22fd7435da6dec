"""The tensor-core (tcgen05, exact three-way TF32 split, FP32 accumulation in
TMEM) mode products of the split-FP32 path against the FP64 oracle.

With the threshold lowered to one SPF, precision 1 runs every FP32 mode product
of nin, nout <= 16 on the tensor cores: the mean-field chains, the A-vector term
products and the H_B * B products of the Lanczos steps.  Each product is carried
to ~2^-33 and the sums are FP32, the accuracy class of FP32 CUDA-core
arithmetic: one EOM evaluation agrees with the FP64 oracle to 1e-6 relative at
the benchmark size (qvc12, 8 SPFs) and on SPF counts that pad the MMA shape (3,
5 and 12 SPFs), with both pipeline variants, and no kernel reports a timed-out
MMA wait.
"""
import numpy as np
import pytest

from macaw_gb300.generate import qvc12
from oracle.mctdh import Oracle
from tests.helpers import random_state, small_qvc
from tests.test_gpu_parity import _rel

pytestmark = pytest.mark.gpu

TC_RTOL = 1e-6


@pytest.fixture(scope="module")
def capi():
    from macaw_gb300 import capi
    st = capi.tensor_core_status()
    if not st["enabled"]:
        pytest.skip("tensor-core kernels switched off (MACAW_GB300_TC=0)")
    capi.tensor_core_config(min_n=1)
    yield capi
    capi.tensor_core_config(min_n=17, stages=1)


def _check(capi, model, seed):
    A, psi = random_state(model, seed=seed)
    ref_dA, ref_dpsi = Oracle(model).calc_derivs(A, psi, 0.0)
    dA, dpsi = capi.GpuCore(model, precision=1).calc_derivs(A, psi, 0.0)
    assert _rel(dA, ref_dA) < TC_RTOL
    assert _rel(dpsi, ref_dpsi) < TC_RTOL
    assert capi.tensor_core_status()["timeouts"] == 0


@pytest.mark.parametrize("stages", [2, 1])
def test_tc_eom_benchmark_size(capi, stages):
    capi.tensor_core_config(stages=stages)
    _check(capi, qvc12(eps_int=1e-5, eps_lanczos=1e-8, eps_spf=1e-7), 61)


@pytest.mark.parametrize("nspf", [3, 5, 12])
def test_tc_eom_padded_shapes(capi, nspf):
    capi.tensor_core_config(stages=2)
    _check(capi, small_qvc(ndof=6, grid=5, nspf=nspf), 62 + nspf)
