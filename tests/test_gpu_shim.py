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
    L.shim_render_gpu.argtypes = ([C.c_int, C.c_int] + [C.c_void_p] * 5 + [C.c_int, C.c_void_p, C.c_int, C.c_int,
                                  C.c_float, C.c_int] + [C.c_void_p] * 14 + [C.c_char_p, C.c_int, C.c_char_p, C.c_int])
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


# ---------------------------------------------------------------- the --gpu renderer (gpu_shim.cpp)
def _render_gpu(shim, oracle, cam, w, h, prev_vp, rtao=True, lighting=2, frame_only=False):
    tris, nrm9, light = oracle.test_scene()
    alb = oracle.test_scene_albedo()
    def z(k=1):
        return np.zeros((h, w, k) if k > 1 else (h, w), np.float32)
    o = dict(depth=z(), position=z(3), normal=z(3), albedo=z(3), mask=np.zeros((h, w), np.uint8), motion=z(2),
             ao_rt=z(), ao_ss=z(), error_map=z(), frame=z(3), hdr=z(3))
    stats, motion2, vp16 = np.zeros(4, np.float32), np.zeros(2, np.int32), np.zeros(16, np.float32)
    adapter, msg = C.create_string_buffer(512), C.create_string_buffer(512)
    p = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    light4 = np.array([*light, 1.0], np.float32)
    rc = shim.shim_render_gpu(w, h, p(np.array(cam, np.float32)), p(np.ascontiguousarray(prev_vp, np.float32)),
                              p(np.ascontiguousarray(tris)), p(np.ascontiguousarray(nrm9)), p(np.ascontiguousarray(alb)),
                              len(tris), p(light4), int(rtao), lighting, C.c_float(0.12), int(frame_only),
                              *[p(o[k]) for k in ("depth", "position", "normal", "albedo", "mask", "motion", "ao_rt",
                                                  "ao_ss", "error_map", "frame", "hdr")],
                              p(stats), p(motion2), p(vp16), adapter, 512, msg, 512)
    assert rc == 0, msg.value
    return o, stats, motion2, vp16, adapter.value.decode()


@pytest.mark.parametrize("model,rtao", [(2, True), (1, True), (1, False)])
def test_render_gpu_frame_result_equals_the_oracle(shim, oracle, model, rtao):
    """raw::renderGpu (gpu_shim.cpp over rn_render_frame), as gpu_run.cpp calls it: every plane
    of the FrameResult equals the CPU path's (the oracle's restatement of renderWithParams) bit
    for bit, under a moving camera; the reconcile, motion counts and view-projection too; gpuInit
    names the device."""
    import importlib
    tf = importlib.import_module("test_gpu_frame")
    cam = (4.0, 4.0, 6.0, 0.0, 1.0, 0.0, 0.0, 1.0, 0.0, 0.9)
    prev = (4.3, 3.8, 5.7, 0.0, 1.0, 0.0, 0.0, 1.0, 0.0, 0.9)
    w, h = 257, 191
    cpu = tf._cpu_frame(oracle, cam, prev, w, h, model, rtao)
    g, stats, motion2, vp16, adapter = _render_gpu(shim, oracle, cam, w, h, cpu["pv"], rtao, model)
    vendor, arch, _, backend, _ = adapter.split("|")
    assert vendor == "NVIDIA" and arch.startswith("sm_") and backend == "cuda"
    keys = ["position", "normal", "mask", "albedo", "ao_ss", "frame", "hdr", "motion"] + (["ao_rt"] if rtao else [])
    for k in keys:
        assert np.array_equal(g[k], cpu[k]), k
    cov = cpu["mask"] > 0
    assert np.array_equal(g["depth"][cov], cpu["depth"][cov]) and np.isinf(g["depth"][~cov]).all()
    assert motion2[0] == cpu["valid"] and motion2[1] == int(cov.sum())
    assert np.array_equal(vp16, np.asarray(oracle.view_proj(cam, w, h), np.float32).ravel())
    if rtao:
        err, st = oracle.reconcile(cpu["ao_ss"], cpu["ao_rt"], cpu["mask"], 0.12)
        assert np.array_equal(g["error_map"], err)
        assert int(stats[2]) == st["pixels"] and stats[1] == st["maxError"] and abs(stats[0] - st["rmse"]) <= 1e-6
        assert bool(stats[3]) == st["within"]
    else:
        assert int(stats[2]) == 0 and not g["error_map"].any()


def test_render_gpu_frame_only_reads_back_the_frame(shim, oracle):
    cam = (4.0, 4.0, 6.0, 0.0, 1.0, 0.0, 0.0, 1.0, 0.0, 0.9)
    w, h = 200, 120
    vp = np.asarray(oracle.view_proj(cam, w, h), np.float32).ravel()
    full = _render_gpu(shim, oracle, cam, w, h, vp)[0]
    only = _render_gpu(shim, oracle, cam, w, h, vp, frame_only=True)[0]
    assert np.array_equal(only["frame"], full["frame"]) and full["frame"].any()
    assert not only["hdr"].any() and not only["mask"].any()
