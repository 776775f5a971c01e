"""The drop-in boundary, checked without a GPU: librn_ao.so loads, exports every symbol
include/rn_ao.h declares, and fails loudly (RN_ERR_NO_DEVICE, never a CPU answer) when no
device is present."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "rn_ao.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|void)\s+(rn_\w+)\s*\(", text, re.M)))


@pytest.fixture(scope="module")
def lib():
    import rn_ao
    if not os.path.exists(rn_ao.LIB_PATH):
        import rn_build
        rn_build.build_library()
    return rn_ao.lib()


def test_header_declares_the_exports():
    import rn_ao
    assert declared_symbols() == sorted(rn_ao.EXPORTS)


def test_library_exports_every_declared_symbol(lib):
    for name in declared_symbols():
        assert hasattr(lib, name), name


def test_abi_version(lib):
    assert lib.rn_ao_version() == 1


def _cuda_present() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_cuda_present(), reason="a GPU is present; the no-device path is not reachable")
def test_no_device_fails_loudly(lib):
    import rn_ao
    with pytest.raises(rn_ao.RnError) as e:
        rn_ao.init()
    assert e.value.code == 2
    a = np.zeros((2, 2), np.float32)
    m = np.ones((2, 2), np.uint8)
    with pytest.raises(rn_ao.RnError) as e:
        rn_ao.reconcile(a, a, m, 0.1)
    assert e.value.code == 2
    g = rn_ao.GBuffer(np.zeros((2, 2, 3), np.float32), np.zeros((2, 2, 3), np.float32), m)
    with pytest.raises(rn_ao.RnError):
        rn_ao.compute_ssao(g, 24, 2.0)


def test_argument_errors_before_any_device_work(lib):
    import rn_ao
    st = rn_ao.Status()
    # null arguments are rejected before the device is touched
    assert lib.rn_reconcile(None, None, None, 1, 1, C.c_float(0.1), 0, None, None, C.byref(st)) == 1
    assert b"null" in st.message
    assert lib.rn_accel_build(None, 5, 0, C.byref(C.c_void_p()), C.byref(st)) == 1
    assert lib.rn_ploc_build(None, 3, 16, 0, None, None, None, C.byref(st)) == 1


def test_host_and_device_arrays_do_not_mix():
    import rn_ao

    class FakeCuda:
        is_cuda = True
    with pytest.raises(rn_ao.RnError):
        rn_ao._Args(np.zeros(3, np.float32), FakeCuda())
