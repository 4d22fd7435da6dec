"""C-ABI checks that need no GPU: the in-tree library loads, exports every
entry point include/macaw_gb300.h declares, and refuses to run without a GPU."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "macaw_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int64_t|const char\s*\*)\s*(mctdh_\w+)\s*\(", text, re.M)))


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__
    __graft_entry__.build()
    from macaw_gb300 import capi
    return capi.load_library()


def test_header_declares_entry_points():
    syms = declared_symbols()
    for name in ("mctdh_create", "mctdh_calc_derivs", "mctdh_rkqs", "mctdh_cmf2", "mctdh_propagate",
                 "mctdh_observables", "mctdh_destroy"):
        assert name in syms


def test_library_exports_every_declared_symbol(lib):
    for name in declared_symbols():
        assert hasattr(lib, name), name


def test_binding_covers_header():
    from macaw_gb300 import capi
    assert set(declared_symbols()) <= set(capi.EXPORTED)


def test_create_without_gpu_fails_loudly(lib):
    """No CPU fallback: on a machine without a CUDA device mctdh_create returns -6."""
    from macaw_gb300.capi import GpuCore, MctdhError
    from tests.helpers import small_lvc
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("a GPU is present")
    with pytest.raises(MctdhError) as ei:
        GpuCore(small_lvc())
    assert ei.value.code == -6
