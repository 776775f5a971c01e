"""The C++ drop-in on the GPU: raw::computeRTVisibility / computeRTAO / computeSSAO /
reconcile as the shim implements them (ao_shim.cpp over librn_ao.so), called the way the
renderer calls them, must give the oracle's outputs bit for bit, keep the reference's
test control (RAW_NATIVE_AO_ORACLE=skew must change the answer), and allocate in the
caller's arena exactly what the reference allocates (the error map only)."""
import ctypes as C
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHIM = os.path.join(ROOT, "raw-native_gb300", "librn_ao_shim.so")
_F = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_U8 = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")


@pytest.fixture(scope="module")
def shim(rn):
    if not os.path.exists(SHIM):
        import rn_build
        rn_build.build_shim()
    L = C.CDLL(SHIM)
    L.shim_rt_visibility.argtypes = [C.c_int, C.c_int, _F, _F, _U8, _F, C.c_int, C.c_int, C.c_float, C.c_void_p,
                                     C.c_int, C.c_int, _F, C.c_void_p, C.c_void_p, C.c_char_p, C.c_int]
    L.shim_ssao.argtypes = [C.c_int, C.c_int, _F, _F, _U8, C.c_int, C.c_float, _F, C.c_char_p, C.c_int]
    L.shim_reconcile.argtypes = [C.c_int, C.c_int, _F, _F, _U8, C.c_float, _F, _F, C.POINTER(C.c_uint64),
                                 C.c_char_p, C.c_int]
    return L


def _inputs(oracle, w, h):
    tris, nrm9, light = oracle.test_scene()
    _, pos, nrm, mask = oracle.rasterize(tris, nrm9, oracle.DEFAULT_CAMERA, w, h)
    return tris, light, pos, nrm, mask


def _vis(shim, w, h, pos, nrm, mask, tris, spp, radius, to_light, skew=0):
    ao, sky, sun = (np.zeros((h, w), np.float32) for _ in range(3))
    msg = C.create_string_buffer(256)
    tl = (C.c_float * 3)(*to_light)
    rc = shim.shim_rt_visibility(w, h, pos, nrm, mask, np.ascontiguousarray(tris), len(tris), spp, radius,
                                 C.cast(tl, C.c_void_p), 0, skew, ao, sky.ctypes.data_as(C.c_void_p),
                                 sun.ctypes.data_as(C.c_void_p), msg, 256)
    assert rc == 0, msg.value
    return ao, sky, sun


def test_shim_frame_equals_oracle(shim, oracle):
    w, h = 256, 256
    tris, light, pos, nrm, mask = _inputs(oracle, w, h)
    ao, sky, sun = _vis(shim, w, h, pos, nrm, mask, tris, 64, 2.0, -light)
    rao, rsky, rsun = oracle.trace(pos, nrm, mask, tris, 64, 2.0, to_light=-light, threads=os.cpu_count() or 1)
    assert np.array_equal(ao, rao) and np.array_equal(sky, rsky) and np.array_equal(sun, rsun)
    ss = np.zeros((h, w), np.float32)
    msg = C.create_string_buffer(256)
    assert shim.shim_ssao(w, h, pos, nrm, mask, 24, 2.0, ss, msg, 256) == 0, msg.value
    assert np.array_equal(ss, oracle.ssao(pos, nrm, mask, 24, 2.0, os.cpu_count() or 1))
    err = np.zeros((h, w), np.float32)
    st = np.zeros(4, np.float32)
    used = C.c_uint64()
    assert shim.shim_reconcile(w, h, ss, ao, mask, 0.12, err, st, C.byref(used), msg, 256) == 0, msg.value
    rerr, rst = oracle.reconcile(ss, ao, mask, 0.12)
    assert np.array_equal(err, rerr)
    assert int(st[2]) == rst["pixels"] and st[1] == np.float32(rst["maxError"]) and bool(st[3]) == rst["within"]
    assert abs(st[0] - rst["rmse"]) <= 1e-6
    assert used.value == w * h * 4          # the reference allocates the error map, and only that, in the arena


def test_shim_skew_control_breaks_parity(shim, oracle):
    # RAW_NATIVE_AO_ORACLE=skew (query 1% short) is the reference's false-success control
    w, h = 128, 128
    tris, light, pos, nrm, mask = _inputs(oracle, w, h)
    ao, _, _ = _vis(shim, w, h, pos, nrm, mask, tris, 64, 2.0, -light, skew=1)
    ref = oracle.trace(pos, nrm, mask, tris, 64, 2.0, threads=os.cpu_count() or 1)
    assert not np.array_equal(ao, ref)


def test_shim_reports_gpu_errors(shim, oracle):
    w, h = 16, 16
    tris, light, pos, nrm, mask = _inputs(oracle, w, h)
    ao = np.zeros((h, w), np.float32)
    msg = C.create_string_buffer(256)
    # samples = 0 is refused by the library; the shim turns it into the renderer's error path
    rc = shim.shim_rt_visibility(w, h, pos, nrm, mask, np.ascontiguousarray(tris), len(tris), 0, 2.0, None, 0, 0, ao,
                                 None, None, msg, 256)
    assert rc == -1 and b"computeRTAO" in msg.value
