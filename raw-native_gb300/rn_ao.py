"""Python face of librn_ao.so, the sm_103a AO path of raw-native.

The names follow the reference's C++ API so a test reads like the reference's own:
``LinearAccel`` (raw/renderer/accel.hpp:15-23), ``compute_rtao`` / ``compute_rt_visibility``
(raw/renderer/ray_ao.hpp:6-14), ``compute_ssao`` (raw/renderer/ssao.hpp:5-6), ``reconcile``
(raw/cert/reconcile.hpp:12-13) and ``build_ploc`` (raw/renderer/rt_bvh.hpp:45).

Arrays may be numpy arrays (host: the library copies in and out) or CUDA tensors (device:
the work is queued on torch's current stream and nothing is copied). Every call goes to the
GPU library; there is no CPU path, and a missing library or device raises ``RnError``.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "librn_ao.so")

RN_DEVICE_PTRS, RN_SKY, RN_SUN_FORCED, RN_DEVICE_TRIG = 0x1, 0x2, 0x4, 0x8
RT_SAMPLES, SS_SAMPLES, AO_RADIUS, TOLERANCE = 64, 24, 2.0, 0.12

ERROR_NAMES = {0: "RN_OK", 1: "RN_ERR_INVALID", 2: "RN_ERR_NO_DEVICE", 3: "RN_ERR_CUDA", 4: "RN_ERR_NO_MEMORY",
               5: "RN_ERR_OVERFLOW", 6: "RN_ERR_BUDGET", 7: "RN_ERR_STATE"}

# Every symbol include/rn_ao.h declares.
EXPORTS = ("rn_ao_version", "rn_init", "rn_set_stream", "rn_synchronize", "rn_accel_build", "rn_accel_free",
           "rn_accel_info", "rn_ao_visibility", "rn_ssao", "rn_reconcile", "rn_ao_frame", "rn_ploc_build",
           "rn_occluded", "rn_closest", "rn_hybrid", "rn_raster_gbuffer", "rn_ao_trace_stats", "rn_reconcile_noalloc", "rn_batch_create",
           "rn_batch_run", "rn_batch_info", "rn_batch_free", "rn_ao_batch", "rn_tc_gemm", "rn_unet_create",
           "rn_unet_free", "rn_unet_param_count", "rn_unet_forward", "rn_unet_train_step", "rn_unet_get_params",
           "rn_unet_set_params", "rn_unet_get_grads", "rn_unet_get_state", "rn_unet_set_state",
           "rn_unet_set_clip", "rn_unet_last_grad_norm", "rn_unet_backward", "rn_unet_grad_count",
           "rn_unet_grads_flat", "rn_unet_apply",
           "rn_tune_set", "rn_tune_get", "rn_tune_load", "rn_tc_conv3x3", "rn_surrogate_ao", "rn_gtao", "rn_selftest_wait_budget",
           "rn_render_frame", "rn_device_info", "rn_pt_scene_create", "rn_pt_scene_free", "rn_pt_scene_info",
           "rn_pathtrace")


class RnError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__("%s: %s" % (ERROR_NAMES.get(code, str(code)), message))
        self.code = code
        self.message = message


class Status(C.Structure):
    _fields_ = [("code", C.c_int), ("message", C.c_char * 240)]


class DeviceDesc(C.Structure):
    _fields_ = [("name", C.c_char * 256), ("cc_major", C.c_int), ("cc_minor", C.c_int), ("sm_count", C.c_int),
                ("driver_version", C.c_int), ("runtime_version", C.c_int), ("total_bytes", C.c_uint64)]


def device_info() -> dict:
    """rn_device_info: the device the library runs on."""
    d, st = DeviceDesc(), Status()
    _check(lib().rn_device_info(C.byref(d), C.byref(st)), st)
    return dict(name=d.name.decode(), cc=(d.cc_major, d.cc_minor), sm_count=d.sm_count,
                driver_version=d.driver_version, runtime_version=d.runtime_version, total_bytes=d.total_bytes)


class GBuf(C.Structure):
    _fields_ = [("w", C.c_int), ("h", C.c_int), ("position", C.c_void_p), ("normal", C.c_void_p),
                ("mask", C.c_void_p)]


class SurrogateStats(C.Structure):
    _fields_ = [("tiles_covered", C.c_uint32), ("tiles_fallback", C.c_uint32), ("mean_depth", C.c_float),
                ("reserved", C.c_float)]


class FrameScene(C.Structure):
    _fields_ = [("tris", C.c_void_p), ("normals", C.c_void_p), ("albedo", C.c_void_p), ("ntri", C.c_uint32),
                ("light_dir", C.c_float * 3), ("light_intensity", C.c_float), ("has_light", C.c_int)]


class FrameOptions(C.Structure):
    _fields_ = [("tolerance", C.c_float), ("rtao", C.c_int), ("lighting", C.c_int), ("spp", C.c_int),
                ("radius", C.c_float), ("ss_samples", C.c_int)]


class View(C.Structure):
    _fields_ = [("w", C.c_int), ("h", C.c_int), ("spp", C.c_int), ("radius", C.c_float), ("position", C.c_void_p),
                ("normal", C.c_void_p), ("mask", C.c_void_p), ("ao", C.c_void_p), ("sky", C.c_void_p),
                ("sun", C.c_void_p), ("ao_ss", C.c_void_p), ("err", C.c_void_p)]


class ReconcileOut(C.Structure):
    _fields_ = [("rmse", C.c_float), ("max_error", C.c_float), ("pixels", C.c_int32),
                ("within_tolerance", C.c_int32), ("sum_sq", C.c_double)]


FRAME_PLANES = (("depth", 1, np.float32), ("position", 3, np.float32), ("normal", 3, np.float32),
                ("albedo", 3, np.float32), ("motion", 2, np.float32), ("mask", 1, np.uint8), ("ao_rt", 1, np.float32),
                ("sky", 1, np.float32), ("sun", 1, np.float32), ("ao_ss", 1, np.float32),
                ("error_map", 1, np.float32), ("frame", 3, np.float32), ("hdr", 3, np.float32))


class FrameOut(C.Structure):
    _fields_ = [(k, C.c_void_p) for k, _, _ in FRAME_PLANES] + [
        ("rec", ReconcileOut), ("motion_valid", C.c_int), ("motion_total", C.c_int), ("view_proj", C.c_float * 16)]


_lib = None


def lib() -> C.CDLL:
    """Load librn_ao.so; raise when it is not built (no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RnError(2, "librn_ao.so is not built (%s); build it with raw-native_gb300/rn_build.py" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        vp, st = C.c_void_p, C.POINTER(Status)
        L.rn_ao_version.restype = C.c_int
        L.rn_init.argtypes = [st]
        L.rn_set_stream.argtypes = [vp, st]
        L.rn_synchronize.argtypes = [st]
        L.rn_accel_build.argtypes = [vp, C.c_uint32, C.c_int, C.POINTER(vp), st]
        L.rn_accel_free.argtypes = [vp]
        L.rn_accel_free.restype = None
        L.rn_accel_info.argtypes = [vp, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), st]
        L.rn_ao_visibility.argtypes = [C.POINTER(GBuf), vp, C.c_int, C.c_float, vp, C.c_int, vp, vp, vp, st]
        L.rn_ssao.argtypes = [C.POINTER(GBuf), C.c_int, C.c_float, C.c_int, vp, st]
        L.rn_reconcile.argtypes = [vp, vp, vp, C.c_int, C.c_int, C.c_float, C.c_int, vp, C.POINTER(ReconcileOut), st]
        L.rn_ao_frame.argtypes = [C.POINTER(GBuf), vp, C.c_int, C.c_float, C.c_int, C.c_float, vp, C.c_int, vp, vp,
                                  vp, vp, vp, C.POINTER(ReconcileOut), st]
        L.rn_ploc_build.argtypes = [vp, C.c_uint32, C.c_int, C.c_int, vp, C.POINTER(C.c_int32),
                                    C.POINTER(C.c_uint32), st]
        L.rn_occluded.argtypes = [vp, vp, vp, C.c_uint32, C.c_int, vp, st]
        L.rn_closest.argtypes = [vp, vp, vp, C.c_uint32, C.c_int, vp, vp, st]
        L.rn_hybrid.argtypes = [C.POINTER(GBuf), vp, vp, vp, vp, C.c_int, vp, vp, vp, st]
        L.rn_raster_gbuffer.argtypes = [vp, vp, C.c_uint32, vp, C.c_int, C.c_int, C.c_int, vp, vp, vp, vp, st]
        L.rn_reconcile_noalloc.argtypes = [vp, vp, vp, C.c_int, C.c_int, C.c_float, vp, vp,
                                           C.POINTER(ReconcileOut), st]
        L.rn_batch_create.argtypes = [vp, C.POINTER(View), C.c_int, C.c_int, C.c_float, vp, C.c_int,
                                      C.POINTER(vp), st]
        L.rn_batch_run.argtypes = [vp, C.POINTER(ReconcileOut), st]
        L.rn_batch_info.argtypes = [vp, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), st]
        L.rn_batch_free.argtypes = [vp]
        L.rn_batch_free.restype = None
        L.rn_ao_batch.argtypes = [vp, C.POINTER(View), C.c_int, C.c_int, C.c_float, vp, C.c_int,
                                  C.POINTER(ReconcileOut), st]
        L.rn_tc_gemm.argtypes = [vp, C.c_int, vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, vp, vp, C.c_int, vp,
                                 C.c_int, st]
        L.rn_unet_create.argtypes = [C.c_int, C.c_int, C.c_int, C.c_uint64, C.c_uint32, C.POINTER(vp), st]
        L.rn_unet_get_state.argtypes = [vp, vp, C.POINTER(C.c_uint64), st]
        L.rn_unet_set_state.argtypes = [vp, vp, C.c_uint64, st]
        L.rn_unet_set_clip.argtypes = [vp, C.c_float, st]
        L.rn_tune_set.argtypes = [C.c_char_p, C.c_int, st]
        L.rn_selftest_wait_budget.argtypes = [C.c_uint32, st]
        L.rn_render_frame.argtypes = [C.POINTER(FrameScene), vp, vp, C.c_int, C.c_int, C.POINTER(FrameOptions), C.c_int,
                                      C.POINTER(FrameOut), st]
        L.rn_gtao.argtypes = [C.POINTER(GBuf), vp, C.c_float, C.c_int, C.c_int, C.c_int, vp, st]
        L.rn_surrogate_ao.argtypes = [vp, C.POINTER(GBuf), vp, vp, C.c_int, C.c_float, C.c_float, vp, vp, vp, vp,
                                      C.POINTER(SurrogateStats), st]
        L.rn_tc_conv3x3.argtypes = [vp, C.c_int, vp, C.c_int, C.c_int, C.c_int, C.c_int, vp, C.c_int, C.c_int, vp, vp,
                                    vp, vp, C.c_int, st]
        L.rn_tune_get.argtypes = [C.c_char_p, C.POINTER(C.c_int), st]
        L.rn_tune_load.argtypes = [C.c_char_p, st]
        L.rn_unet_last_grad_norm.argtypes = [vp, C.POINTER(C.c_float), C.POINTER(C.c_float), st]
        L.rn_unet_free.argtypes = [vp]
        L.rn_unet_free.restype = None
        L.rn_unet_param_count.argtypes = [vp, C.POINTER(C.c_uint64), st]
        L.rn_unet_forward.argtypes = [vp, vp, C.c_int, vp, st]
        L.rn_unet_train_step.argtypes = [vp, vp, vp, C.c_int, C.c_float, C.POINTER(C.c_float), st]
        L.rn_unet_backward.argtypes = [vp, vp, vp, C.c_int, C.POINTER(C.c_float), st]
        L.rn_unet_grad_count.argtypes = [vp, C.POINTER(C.c_uint64), st]
        L.rn_unet_grads_flat.argtypes = [vp, vp, C.c_int, st]
        L.rn_unet_apply.argtypes = [vp, C.c_float, st]
        for f in (L.rn_unet_get_params, L.rn_unet_set_params, L.rn_unet_get_grads):
            f.argtypes = [vp, vp, st]
        L.rn_ao_trace_stats.argtypes = [C.POINTER(GBuf), vp, C.c_int, C.c_float, vp, C.c_int, C.c_uint32,
                                        C.POINTER(C.c_uint64), st]
        _lib = L
    return _lib


def _check(rc: int, st: Status) -> None:
    if rc != 0:
        raise RnError(rc, st.message.decode(errors="replace"))


# ---------------------------------------------------------------- launch-shape tuning
TUNE_KEYS = {"trace_min_blocks": (2, 3, 4), "batch_min_blocks": (2, 3, 4), "trace_frontier": (0, 1), "trace_frontier_min_spp": (1, 8, 16, 32),
             "trace_frontier_tail": (0, 4, 8, 16),
             "trace_packet": (4, 8, 16),
             "trace_stack": (48, 96), "ssao_tile_h": (4, 8, 16), "conv_bn_max": (64, 128, 256), "conv_halo": (0, 1), "conv_pair": (0, 1),
             "accel_radius": (8, 16, 32, 64), "accel_leaf": (1, 2, 4, 8), "accel_leaf_small": (1, 2, 4, 8),
             "frame_direct": (0, 1), "hybrid_min_blocks": (5, 6, 8), "pt_slice": (0, 1, 4, 16), "pt_regen": (0, 4, 8, 16),
             "pt_wave": (0, 1, 64, 256, 1024, 2048), "pt_shade_blocks": (4, 6, 8),
             "trace_pool": (0, 16, 24, 32), "ploc_tail": (0, 4096, 16384, 32768, 65536, 262144),
             "ploc_tail_ctas": (1, 4, 8, 16), "ploc_fused": (0, 1),
             "collapse_block": (0, 16384, 65536, 262144),
             "conv_tmem_a": (0, 1), "conv_fan": (0, 1), "conv_fan_bn": (32, 64), "trace_leaf_pass": (0, 1),
             "trace_pool_sort": (0, 1)}


def tune_set(key: str, value: int) -> None:
    st = Status()
    _check(lib().rn_tune_set(key.encode(), int(value), C.byref(st)), st)


def tune_get(key: str) -> int:
    v = C.c_int()
    st = Status()
    _check(lib().rn_tune_get(key.encode(), C.byref(v), C.byref(st)), st)
    return v.value


def tune_all() -> dict:
    return {k: tune_get(k) for k in TUNE_KEYS}


def tune_load(path: str) -> None:
    st = Status()
    _check(lib().rn_tune_load(os.fsencode(path), C.byref(st)), st)


TUNE_FILE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tune_sm103.txt")


def init(load_tune: bool = True) -> None:
    """rn_init; then the autotuner's launch shapes: the file named by RN_TUNE_FILE, else the
    package's tune_sm103.txt when present."""
    st = Status()
    _check(lib().rn_init(C.byref(st)), st)
    if load_tune:
        path = os.environ.get("RN_TUNE_FILE") or (TUNE_FILE if os.path.exists(TUNE_FILE) else None)
        if path:
            tune_load(path)


def synchronize() -> None:
    st = Status()
    _check(lib().rn_synchronize(C.byref(st)), st)


# ---------------------------------------------------------------- array plumbing
def _is_cuda(a) -> bool:
    return hasattr(a, "is_cuda") and a.is_cuda


def _use_torch_stream() -> None:
    """Queue the library's work on torch's current stream. torch's default stream has handle
    0, the legacy default stream: pass cudaStreamLegacy (1) so the work orders with it."""
    import torch
    handle = torch.cuda.current_stream().cuda_stream or 1
    st = Status()
    _check(lib().rn_set_stream(C.c_void_p(handle), C.byref(st)), st)


class _Args:
    """Collects pointers for one call; all arrays are either host or CUDA."""

    def __init__(self, *arrays):
        present = [a for a in arrays if a is not None]
        self.device = bool(present) and _is_cuda(present[0])
        for a in present:
            if _is_cuda(a) != self.device:
                raise RnError(1, "mix of host and CUDA arrays in one call")
        self.keep = []
        if self.device:
            _use_torch_stream()

    def ptr(self, a, dtype):
        if a is None:
            return None
        if self.device:
            import torch
            tdt = {np.float32: torch.float32, np.uint8: torch.uint8, np.int32: torch.int32}[dtype]
            if a.dtype != tdt or not a.is_contiguous():
                raise RnError(1, "CUDA array must be contiguous %s" % tdt)
            return C.c_void_p(a.data_ptr())
        arr = np.ascontiguousarray(a, dtype=dtype)
        self.keep.append(arr)
        return C.c_void_p(arr.ctypes.data)

    def out(self, like, shape, dtype):
        if self.device:
            import torch
            tdt = {np.float32: torch.float32, np.uint8: torch.uint8, np.int32: torch.int32}[dtype]
            return torch.empty(shape, dtype=tdt, device=like.device)
        return np.empty(shape, dtype)

    @property
    def flags(self) -> int:
        return RN_DEVICE_PTRS if self.device else 0


@dataclasses.dataclass
class GBuffer:
    """raw::GBuffer's AO inputs (raw/renderer/gbuffer.hpp:7-21): position and normal as
    (h, w, 3) float32, mask as (h, w) uint8."""
    position: object
    normal: object
    mask: object

    @property
    def shape(self):
        return tuple(self.mask.shape)


def _gbuf(g: GBuffer, args: _Args) -> GBuf:
    h, w = g.shape
    return GBuf(w, h, args.ptr(g.position, np.float32), args.ptr(g.normal, np.float32), args.ptr(g.mask, np.uint8))


# ---------------------------------------------------------------- accelerator
class LinearAccel:
    """The occlusion accelerator over a triangle list (n, 9) float32, built on the GPU
    (PLOC, collapsed to 4-wide nodes). Replaces raw::LinearAccel::build."""

    def __init__(self, tris):
        args = _Args(tris)
        n = int(tris.shape[0]) if tris is not None else 0
        self._h = C.c_void_p()
        st = Status()
        _check(lib().rn_accel_build(args.ptr(tris, np.float32), n, args.flags, C.byref(self._h), C.byref(st)), st)
        self.ntri = n

    def info(self) -> dict:
        a, b, c = C.c_uint32(), C.c_uint32(), C.c_uint32()
        st = Status()
        _check(lib().rn_accel_info(self._h, C.byref(a), C.byref(b), C.byref(c), C.byref(st)), st)
        return dict(wide_nodes=a.value, leaf_tris=b.value, ploc_rounds=c.value)

    def close(self) -> None:
        if self._h:
            lib().rn_accel_free(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h


# ---------------------------------------------------------------- the three passes
def compute_rt_visibility(g: GBuffer, accel: LinearAccel, samples: int, radius: float, to_light=None,
                          sun_forced: bool = False, device_trig: bool = False):
    """computeRTVisibility when to_light is given: (ao, sky, sun); computeRTAO otherwise: ao."""
    args = _Args(g.position, g.normal, g.mask)
    gb = _gbuf(g, args)
    h, w = g.shape
    ao = args.out(g.mask, (h, w), np.float32)
    sky = sun = None
    flags = args.flags | (RN_DEVICE_TRIG if device_trig else 0)
    tl = None
    if to_light is not None:
        flags |= RN_SKY | (RN_SUN_FORCED if sun_forced else 0)
        sky = args.out(g.mask, (h, w), np.float32)
        sun = args.out(g.mask, (h, w), np.float32)
        tl = (C.c_float * 3)(*[float(v) for v in to_light])
    st = Status()
    rc = lib().rn_ao_visibility(C.byref(gb), accel.handle, int(samples), float(radius),
                                C.cast(tl, C.c_void_p) if tl is not None else None, flags,
                                args.ptr(ao, np.float32), args.ptr(sky, np.float32), args.ptr(sun, np.float32),
                                C.byref(st))
    _check(rc, st)
    return ao if to_light is None else (ao, sky, sun)


def compute_rtao(g: GBuffer, accel: LinearAccel, samples: int, radius: float, device_trig: bool = False):
    return compute_rt_visibility(g, accel, samples, radius, None, device_trig=device_trig)


def compute_ssao(g: GBuffer, samples: int = SS_SAMPLES, radius: float = AO_RADIUS, device_trig: bool = False):
    args = _Args(g.position, g.normal, g.mask)
    gb = _gbuf(g, args)
    out = args.out(g.mask, g.shape, np.float32)
    st = Status()
    flags = args.flags | (RN_DEVICE_TRIG if device_trig else 0)
    _check(lib().rn_ssao(C.byref(gb), int(samples), float(radius), flags, args.ptr(out, np.float32), C.byref(st)), st)
    return out


def render_frame(tris, normals, albedo, camera, w: int, h: int, light=None, prev_view_proj=None, rtao: bool = True,
                 lighting: int = 2, spp: int = RT_SAMPLES, radius: float = AO_RADIUS, ss_samples: int = SS_SAMPLES,
                 tolerance: float = TOLERANCE):
    """raw::renderWithParams on the GPU: dict of every plane (numpy for numpy inputs, CUDA
    tensors for CUDA inputs) plus rec (ReconcileResult without its map), motion_valid,
    motion_total and view_proj. light = (direction, intensity) of scene.lights[0] or None."""
    args = _Args(tris, normals, albedo)
    n = int(tris.shape[0])
    like = tris
    outs = {k: args.out(like, (h, w, c) if c > 1 else (h, w), dt) for k, c, dt in FRAME_PLANES}
    sc = FrameScene(args.ptr(tris, np.float32), args.ptr(normals, np.float32), args.ptr(albedo, np.float32), n,
                    (C.c_float * 3)(*(light[0] if light is not None else (0.0, -1.0, 0.0))),
                    float(light[1]) if light is not None else 1.0, 1 if light is not None else 0)
    opt = FrameOptions(float(tolerance), 1 if rtao else 0, int(lighting), int(spp), float(radius), int(ss_samples))
    fo = FrameOut()
    for k, _, dt in FRAME_PLANES:
        setattr(fo, k, args.ptr(outs[k], dt))
    cam = (C.c_float * 10)(*[float(v) for v in camera])
    prev = (C.c_float * 16)(*[float(v) for v in prev_view_proj]) if prev_view_proj is not None else None
    st = Status()
    _check(lib().rn_render_frame(C.byref(sc), C.cast(cam, C.c_void_p), C.cast(prev, C.c_void_p) if prev is not None else None,
                                 int(w), int(h), C.byref(opt), args.flags, C.byref(fo), C.byref(st)), st)
    outs["rec"] = _result(None, fo.rec)
    outs["motion_valid"], outs["motion_total"] = fo.motion_valid, fo.motion_total
    outs["view_proj"] = np.array(list(fo.view_proj), np.float32)
    return outs


def selftest_wait_budget(spin_limit: int = 1 << 16) -> None:
    """Runs the device-side wait-budget self-test; raises RnError (code RN_ERR_BUDGET)."""
    st = Status()
    _check(lib().rn_selftest_wait_budget(int(spin_limit), C.byref(st)), st)


def gtao(g: GBuffer, camera, radius: float = 0.5, slices: int = 16, steps: int = 16):
    """raw::post::gtao of the G-buffer seen from camera (eye, target, up, fovy)."""
    args = _Args(g.position, g.normal, g.mask)
    gb = _gbuf(g, args)
    out = args.out(g.mask, g.shape, np.float32)
    cam = (C.c_float * 10)(*[float(v) for v in camera])
    st = Status()
    _check(lib().rn_gtao(C.byref(gb), C.cast(cam, C.c_void_p), float(radius), int(slices), int(steps), args.flags,
                         args.ptr(out, np.float32), C.byref(st)), st)
    return out


@dataclasses.dataclass
class ReconcileResult:
    """raw::ReconcileResult (raw/cert/reconcile.hpp:6-11) plus the FP64 sum it came from."""
    error_map: object
    rmse: float
    max_error: float
    pixels: int
    within_tolerance: bool
    sum_sq: float


def _result(err, r: ReconcileOut) -> ReconcileResult:
    return ReconcileResult(err, r.rmse, r.max_error, r.pixels, bool(r.within_tolerance), r.sum_sq)


def reconcile(approx, truth, mask, tolerance: float = TOLERANCE, error_map: bool = True) -> ReconcileResult:
    args = _Args(approx, truth, mask)
    h, w = tuple(mask.shape)
    err = args.out(mask, (h, w), np.float32) if error_map else None
    r = ReconcileOut()
    st = Status()
    _check(lib().rn_reconcile(args.ptr(approx, np.float32), args.ptr(truth, np.float32), args.ptr(mask, np.uint8),
                              w, h, float(tolerance), args.flags, args.ptr(err, np.float32), C.byref(r),
                              C.byref(st)), st)
    return _result(err, r)


def ao_frame(g: GBuffer, accel: LinearAccel, samples: int = RT_SAMPLES, radius: float = AO_RADIUS,
             ss_samples: int = SS_SAMPLES, tolerance: float = TOLERANCE, to_light=None, sun_forced=False,
             outputs=None, device_trig: bool = False):
    """The AO passes of one frame (render.cpp:29-54): returns dict(ao, sky, sun, ss, err, rec).
    `outputs` may pass preallocated arrays under the same keys."""
    args = _Args(g.position, g.normal, g.mask)
    gb = _gbuf(g, args)
    h, w = g.shape
    o = dict(outputs or {})
    for k in ("ao", "ss", "err") + (("sky", "sun") if to_light is not None else ()):
        if o.get(k) is None:
            o[k] = args.out(g.mask, (h, w), np.float32)
    flags = args.flags | (RN_DEVICE_TRIG if device_trig else 0)
    tl = None
    if to_light is not None:
        flags |= RN_SKY | (RN_SUN_FORCED if sun_forced else 0)
        tl = (C.c_float * 3)(*[float(v) for v in to_light])
    r = ReconcileOut()
    st = Status()
    p = {k: (args.ptr(v, np.float32) if v is not None else None) for k, v in o.items()}
    rc = lib().rn_ao_frame(C.byref(gb), accel.handle, int(samples), float(radius), int(ss_samples), float(tolerance),
                           C.cast(tl, C.c_void_p) if tl is not None else None, flags, p["ao"], p.get("sky"),
                           p.get("sun"), p["ss"], p["err"], C.byref(r), C.byref(st))
    _check(rc, st)
    o["rec"] = _result(o["err"], r)
    return o


def rasterize(tris, normals, camera, w: int, h: int, want_depth: bool = False):
    """raw::rasterize on the GPU: GBuffer (and depth when asked). tris/normals (n, 9) float32;
    camera = eye(3), target(3), up(3), fovy."""
    args = _Args(tris, normals)
    n = int(tris.shape[0])
    like = tris
    pos = args.out(like, (h, w, 3), np.float32)
    nrm = args.out(like, (h, w, 3), np.float32)
    mask = args.out(like, (h, w), np.uint8)
    depth = args.out(like, (h, w), np.float32) if want_depth else None
    cam = (C.c_float * 10)(*[float(v) for v in camera])
    st = Status()
    _check(lib().rn_raster_gbuffer(args.ptr(tris, np.float32), args.ptr(normals, np.float32), n,
                                   C.cast(cam, C.c_void_p), int(w), int(h), args.flags, args.ptr(depth, np.float32),
                                   args.ptr(pos, np.float32), args.ptr(nrm, np.float32), args.ptr(mask, np.uint8),
                                   C.byref(st)), st)
    g = GBuffer(pos, nrm, mask)
    return (g, depth) if want_depth else g


def trace_stats(g: GBuffer, accel: LinearAccel, samples: int, radius: float, to_light=None, tile_stride: int = 1):
    """Traversal counters of the visibility pass: dict(rays, nodes, tris, sky_rays)."""
    args = _Args(g.position, g.normal, g.mask)
    gb = _gbuf(g, args)
    flags = args.flags
    tl = None
    if to_light is not None:
        flags |= RN_SKY
        tl = (C.c_float * 3)(*[float(v) for v in to_light])
    counts = (C.c_uint64 * 4)()
    st = Status()
    _check(lib().rn_ao_trace_stats(C.byref(gb), accel.handle, int(samples), float(radius),
                                   C.cast(tl, C.c_void_p) if tl is not None else None, flags, int(tile_stride),
                                   counts, C.byref(st)), st)
    return dict(rays=counts[0], nodes=counts[1], tris=counts[2], sky_rays=counts[3])


class Batch:
    """A prepared batch of views over one accelerator (CUDA tensors only). `views` is a list of
    dicts with keys g (GBuffer), spp, radius and, optionally, ssao=True and sky=True
    (the batch-wide to_light). Outputs are allocated here: batch.outputs[i] holds the view's
    ao (and ss, err, sky, sun). run() replays the captured frame and returns the per-view
    ReconcileResults (error maps are in outputs)."""

    def __init__(self, accel: LinearAccel, views, ss_samples: int = SS_SAMPLES, tolerance: float = TOLERANCE,
                 to_light=None, device_trig: bool = False):
        import torch
        _use_torch_stream()
        self.accel = accel
        self.n = len(views)
        self.outputs = []
        arr = (View * self.n)()
        for k, v in enumerate(views):
            g = v["g"]
            h, w = g.shape
            o = {"ao": torch.empty(h, w, device=g.mask.device)}
            if v.get("ssao", True):
                o["ss"] = torch.empty_like(o["ao"])
                o["err"] = torch.empty_like(o["ao"])
            if to_light is not None:
                o["sky"] = torch.empty_like(o["ao"])
                o["sun"] = torch.empty_like(o["ao"])
            self.outputs.append(o)
            ptr = lambda t: t.data_ptr() if t is not None else None
            arr[k] = View(w, h, int(v["spp"]), float(v["radius"]), g.position.data_ptr(), g.normal.data_ptr(),
                          g.mask.data_ptr(), o["ao"].data_ptr(), ptr(o.get("sky")), ptr(o.get("sun")),
                          ptr(o.get("ss")), ptr(o.get("err")))
        self._views = views                 # keep the G-buffers alive
        flags = (RN_SKY if to_light is not None else 0) | (RN_DEVICE_TRIG if device_trig else 0)
        tl = (C.c_float * 3)(*[float(x) for x in to_light]) if to_light is not None else None
        self._h = C.c_void_p()
        st = Status()
        _check(lib().rn_batch_create(accel.handle, arr, self.n, int(ss_samples), float(tolerance),
                                     C.cast(tl, C.c_void_p) if tl is not None else None, flags, C.byref(self._h),
                                     C.byref(st)), st)
        self.tolerance = tolerance

    def info(self) -> dict:
        t, r = C.c_uint64(), C.c_uint64()
        st = Status()
        _check(lib().rn_batch_info(self._h, C.byref(t), C.byref(r), C.byref(st)), st)
        return dict(tiles=t.value, pixel_samples=r.value)

    def run(self):
        _use_torch_stream()
        res = (ReconcileOut * self.n)()
        st = Status()
        _check(lib().rn_batch_run(self._h, res, C.byref(st)), st)
        return [_result(self.outputs[k].get("err"), res[k]) for k in range(self.n)]

    def close(self):
        if self._h:
            lib().rn_batch_free(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def tc_gemm(P, Q, out_dtype=None, bias=None, relu=False, splits=1):
    """C = P @ Q.T on the tensor cores (CUDA bf16 tensors, K contiguous). FP32 output, or bf16
    when out_dtype is torch.bfloat16; splits > 1 reduces K in slices with FP32 atomics."""
    import torch
    M, K = P.shape
    N = Q.shape[0]
    _use_torch_stream()
    c32 = torch.zeros(M, N, device=P.device) if (out_dtype in (None, torch.float32) or splits > 1) else None
    c16 = torch.empty(M, N, device=P.device, dtype=torch.bfloat16) if out_dtype == torch.bfloat16 else None
    st = Status()
    _check(lib().rn_tc_gemm(C.c_void_p(P.data_ptr()), P.stride(0), C.c_void_p(Q.data_ptr()), Q.stride(0), M, N, K,
                            int(splits), C.c_void_p(c32.data_ptr()) if c32 is not None else None,
                            C.c_void_p(c16.data_ptr()) if c16 is not None else None, N,
                            C.c_void_p(bias.data_ptr()) if bias is not None else None, int(relu), C.byref(st)), st)
    return c16 if c16 is not None else c32


def tc_conv3x3(x0, w, x1=None, bias=None, relu=False, out_dtype=None, upsampled=False):
    """Implicit-GEMM 3x3 convolution (stride 1, zero padding 1) on the tensor cores. x0, x1:
    CUDA bf16 NHWC [B, H, W, C] (channels concatenated); w: bf16 [N, ldw] with column
    tap * Cin + ci, tap = 3 (dy + 1) + (dx + 1). Returns the FP32 (or bf16) output
    [B, H, W, N], and with upsampled=True also its 2x nearest-upsampled bf16 copy."""
    import torch
    B, H, W, c0 = x0.shape
    c1 = x1.shape[3] if x1 is not None else 0
    N = w.shape[0]
    _use_torch_stream()
    bf = out_dtype == torch.bfloat16 or upsampled
    c32 = None if bf else torch.empty(B, H, W, N, device=x0.device)
    c16 = torch.empty(B, H, W, N, device=x0.device, dtype=torch.bfloat16) if bf else None
    up = torch.empty(B, 2 * H, 2 * W, N, device=x0.device, dtype=torch.bfloat16) if upsampled else None
    ptr = lambda t: C.c_void_p(t.data_ptr()) if t is not None else None
    st = Status()
    _check(lib().rn_tc_conv3x3(ptr(x0), c0, ptr(x1), c1, B, H, W, ptr(w), w.stride(0), N, ptr(c32), ptr(c16), ptr(up),
                               ptr(bias), int(relu), C.byref(st)), st)
    out = c16 if bf else c32
    return (out, up) if upsampled else out


class UNet:
    """The learned AO surrogate network for one input shape (see rn_unet_create). Inputs,
    targets and outputs are CUDA float32 tensors: x [B, H, W, 5], y [B, H, W]."""

    def __init__(self, batch: int, height: int, width: int, seed: int = 0, inference: bool = False,
                 explicit: bool = False):
        self._h = C.c_void_p()
        st = Status()
        flags = (1 if inference else 0) | (2 if explicit else 0)
        _check(lib().rn_unet_create(batch, height, width, seed, flags, C.byref(self._h), C.byref(st)), st)
        self.shape = (batch, height, width)
        n = C.c_uint64()
        _check(lib().rn_unet_param_count(self._h, C.byref(n), C.byref(st)), st)
        self.param_count = n.value

    def forward(self, x):
        import torch
        _use_torch_stream()
        out = torch.empty(self.shape, device=x.device)
        st = Status()
        _check(lib().rn_unet_forward(self._h, C.c_void_p(x.data_ptr()), self.shape[0], C.c_void_p(out.data_ptr()),
                                     C.byref(st)), st)
        return out

    def train_step(self, x, y, lr: float) -> float:
        _use_torch_stream()
        loss = C.c_float()
        st = Status()
        _check(lib().rn_unet_train_step(self._h, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), self.shape[0],
                                        float(lr), C.byref(loss), C.byref(st)), st)
        return loss.value

    def _io(self, fn, arr=None):
        out = np.empty(self.param_count, np.float32) if arr is None else np.ascontiguousarray(arr, np.float32)
        if out.size != self.param_count:
            raise ValueError("%d values, expected %d" % (out.size, self.param_count))
        st = Status()
        _check(fn(self._h, C.c_void_p(out.ctypes.data), C.byref(st)), st)
        return out

    def get_params(self):
        return self._io(lib().rn_unet_get_params)

    def set_params(self, p):
        self._io(lib().rn_unet_set_params, p)

    def get_grads(self):
        return self._io(lib().rn_unet_get_grads)

    # data-parallel training: backward on this rank's batch, the gradients exchanged through a
    # flat CUDA tensor, then apply (train_step is backward + apply)
    def backward(self, x, y) -> float:
        _use_torch_stream()
        loss = C.c_float()
        st = Status()
        _check(lib().rn_unet_backward(self._h, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), self.shape[0],
                                      C.byref(loss), C.byref(st)), st)
        return loss.value

    @property
    def grad_count(self) -> int:
        n = C.c_uint64()
        st = Status()
        _check(lib().rn_unet_grad_count(self._h, C.byref(n), C.byref(st)), st)
        return n.value

    def grads_to(self, flat):
        """Copy the gradients into `flat` (a contiguous CUDA float32 tensor of grad_count)."""
        self._flat(flat, 1)

    def grads_from(self, flat):
        """Replace the gradients by `flat` (as grads_to lays them out)."""
        self._flat(flat, 0)

    def _flat(self, flat, to_flat: int):
        import torch
        if not (flat.is_cuda and flat.dtype == torch.float32 and flat.is_contiguous() and flat.numel() == self.grad_count):
            raise ValueError("a contiguous CUDA float32 tensor of %d values is needed" % self.grad_count)
        _use_torch_stream()
        st = Status()
        _check(lib().rn_unet_grads_flat(self._h, C.c_void_p(flat.data_ptr()), int(to_flat), C.byref(st)), st)

    def apply(self, lr: float) -> None:
        _use_torch_stream()
        st = Status()
        _check(lib().rn_unet_apply(self._h, float(lr), C.byref(st)), st)

    def set_clip(self, ratio: float):
        """Adaptive gradient clipping at `ratio` x the running mean norm (0: off)."""
        st = Status()
        _check(lib().rn_unet_set_clip(self._h, float(ratio), C.byref(st)), st)

    def last_grad_norm(self):
        """(global gradient norm of the last train step, clip factor applied)."""
        n, s = C.c_float(), C.c_float()
        st = Status()
        _check(lib().rn_unet_last_grad_norm(self._h, C.byref(n), C.byref(s), C.byref(st)), st)
        return n.value, s.value

    def get_state(self):
        """(weights, first moments, second moments) as one FP32 array, and the step count."""
        out = np.empty(3 * self.param_count, np.float32)
        step = C.c_uint64()
        st = Status()
        _check(lib().rn_unet_get_state(self._h, C.c_void_p(out.ctypes.data), C.byref(step), C.byref(st)), st)
        return out, step.value

    def set_state(self, state, step: int):
        arr = np.ascontiguousarray(state, np.float32)
        if arr.size != 3 * self.param_count:
            raise ValueError("state holds %d values, expected %d" % (arr.size, 3 * self.param_count))
        st = Status()
        _check(lib().rn_unet_set_state(self._h, C.c_void_p(arr.ctypes.data), int(step), C.byref(st)), st)

    def close(self):
        if self._h:
            lib().rn_unet_free(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def surrogate_ao(net: "UNet", g: GBuffer, depth, accel: LinearAccel, spp_full: int, radius: float = 1.0,
                 k: float = 3.0, want_parts: bool = False):
    """One AO frame by the surrogate (rn_surrogate_ao): returns (ao, stats dict) and, with
    want_parts, also dict(ao4, pred, tile_flags). CUDA tensors; `net` has batch 1."""
    import torch
    h, w = g.shape
    dev = g.mask.device
    ao = torch.empty(h, w, device=dev)
    parts = dict(ao4=torch.empty(h, w, device=dev), pred=torch.empty(h, w, device=dev),
                 tile_flags=torch.empty((h + 15) // 16, (w + 15) // 16, device=dev, dtype=torch.uint8)) if want_parts else {}
    args = _Args(g.position, g.normal, g.mask)
    gb = _gbuf(g, args)
    _use_torch_stream()
    ptr = lambda t: C.c_void_p(t.data_ptr()) if t is not None else None
    stt = SurrogateStats()
    st = Status()
    _check(lib().rn_surrogate_ao(net._h, C.byref(gb), ptr(depth), accel.handle, int(spp_full), float(radius), float(k),
                                 ptr(ao), ptr(parts.get("ao4")), ptr(parts.get("pred")), ptr(parts.get("tile_flags")),
                                 C.byref(stt), C.byref(st)), st)
    stats = dict(tiles_covered=stt.tiles_covered, tiles_fallback=stt.tiles_fallback, mean_depth=stt.mean_depth,
                 fallback_fraction=stt.tiles_fallback / max(1, stt.tiles_covered))
    return (ao, stats, parts) if want_parts else (ao, stats)


# The surrogate's layer table, for code that restates the network (tests): (cin, cout) of
# each 3x3 convolution in parameter order.
UNET_CONVS = [(8, 32), (32, 32), (32, 64), (64, 64), (64, 128), (128, 128), (128, 256), (256, 256), (384, 128),
              (128, 128), (192, 64), (64, 64), (96, 32), (32, 32)]


def build_ploc(tris, radius: int = 16):
    """rt::buildPloc on the GPU: (nodes (2n-1, 9) int32, root, rounds)."""
    args = _Args(tris)
    n = int(tris.shape[0])
    nodes = args.out(tris, (max(2 * n - 1, 1), 9), np.int32)
    root, rounds = C.c_int32(), C.c_uint32()
    st = Status()
    _check(lib().rn_ploc_build(args.ptr(tris, np.float32), n, int(radius), args.flags, args.ptr(nodes, np.int32),
                               C.byref(root), C.byref(rounds), C.byref(st)), st)
    return nodes, root.value, rounds.value


def occluded(accel: LinearAccel, rays, t_max):
    """Any-hit for a list of rays (n, 6): uint8 hit flags."""
    args = _Args(rays, t_max)
    n = int(rays.shape[0])
    hit = args.out(rays, (n,), np.uint8)
    st = Status()
    _check(lib().rn_occluded(accel.handle, args.ptr(rays, np.float32), args.ptr(t_max, np.float32), n, args.flags,
                             args.ptr(hit, np.uint8), C.byref(st)), st)
    return hit


def closest(accel: LinearAccel, rays, t_max):
    """rt::closest for a list of rays (n, 6): (triangle index int32, -1 for none; t, -1 for
    none), the nearest hit below t_max with ties to the lowest index."""
    args = _Args(rays, t_max)
    n = int(rays.shape[0])
    tri = args.out(rays, (n,), np.int32)
    t = args.out(rays, (n,), np.float32)
    st = Status()
    _check(lib().rn_closest(accel.handle, args.ptr(rays, np.float32), args.ptr(t_max, np.float32), n, args.flags,
                            args.ptr(tri, np.int32), args.ptr(t, np.float32), C.byref(st)), st)
    return tri, t


def hybrid(g: GBuffer, accel: LinearAccel, eye, to_sun, geo_normal=None):
    """The hybrid pass over a G-buffer: (lit, refl_tri, refl_t), each (h, w); lit 1 / 0 / -1
    (lit, shadowed, uncovered), refl_tri / refl_t the mirror ray's nearest hit (-1: none).
    geo_normal: the surface triangles' normals (h, w, 3) for the offsets and the facing test;
    None uses the G-buffer normals."""
    args = _Args(g.position, g.normal, g.mask, geo_normal)
    gb = _gbuf(g, args)
    h, w = g.shape
    lit = args.out(g.mask, (h, w), np.float32)
    tri = args.out(g.mask, (h, w), np.int32)
    t = args.out(g.mask, (h, w), np.float32)
    e = (C.c_float * 3)(*[float(v) for v in eye])
    l = (C.c_float * 3)(*[float(v) for v in to_sun])
    st = Status()
    _check(lib().rn_hybrid(C.byref(gb), args.ptr(geo_normal, np.float32), accel.handle, C.cast(e, C.c_void_p),
                           C.cast(l, C.c_void_p), args.flags,
                           args.ptr(lit, np.float32), args.ptr(tri, np.int32), args.ptr(t, np.float32), C.byref(st)), st)
    return lit, tri, t


# ---------------------------------------------------------------- path tracer (raw::rt, interface v4)
PT_CONTROLS = dict(drop_lambert_cosine=0x01, mis_weight_one=0x02, aov_drop_specular_indirect=0x04,
                   aov_emission_to_diffuse=0x08, legacy_lobe_v2=0x10)
PT_AOVS = (("radiance", 3, np.float32), ("albedo", 3, np.float32), ("normal", 3, np.float32),
           ("depth", 1, np.float32), ("variance", 1, np.float32), ("triangle", 1, np.int32),
           ("motion", 2, np.float32), ("diffuse", 3, np.float32), ("specular", 3, np.float32),
           ("emission", 3, np.float32), ("diffuse_albedo", 3, np.float32), ("specular_albedo", 3, np.float32),
           ("diffuse_variance", 1, np.float32), ("specular_variance", 1, np.float32))


class PtMaterial(C.Structure):
    _fields_ = [("base_factor", C.c_float), ("roughness", C.c_float), ("metallic", C.c_float),
                ("specular", C.c_float), ("emission", C.c_float * 3)]


class PtSceneDesc(C.Structure):
    _fields_ = [("pos", C.c_void_p), ("nrm", C.c_void_p), ("uv", C.c_void_p), ("nvert", C.c_uint32),
                ("idx", C.c_void_p), ("tri_texture", C.c_void_p), ("ntri", C.c_uint32),
                ("tex_entries", C.c_void_p), ("ntex", C.c_uint32), ("texels", C.c_void_p), ("ntexels", C.c_uint32),
                ("materials", C.c_void_p), ("sun_dir", C.c_float * 3), ("sun_irradiance", C.c_float * 3),
                ("sky", C.c_float * 3)]


class PtDesc(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("spp", C.c_uint32), ("spp_begin", C.c_uint32), ("max_bounces", C.c_uint32),
                ("width", C.c_int32), ("height", C.c_int32), ("camera", C.c_float * 10), ("previous", C.c_float * 10),
                ("jitter", C.c_int32), ("russian_roulette", C.c_int32), ("controls", C.c_uint32)]


class PtOut(C.Structure):
    _fields_ = [(name, C.c_void_p) for name, _, _ in PT_AOVS]


def pt_desc(d: dict) -> PtDesc:
    """A render description (raw::rt::PathTraceDesc) from a dict: seed, spp, spp_begin,
    max_bounces, width, height, camera (10 floats), previous, jitter, russian_roulette and
    controls (names of PT_CONTROLS)."""
    controls = 0
    for k in d.get("controls", ()):
        controls |= PT_CONTROLS[k]
    return PtDesc(int(d.get("seed", 1)), int(d.get("spp", 16)), int(d.get("spp_begin", 0)),
                  int(d.get("max_bounces", 64)), int(d["width"]), int(d["height"]), (C.c_float * 10)(*d["camera"]),
                  (C.c_float * 10)(*d.get("previous", d["camera"])), int(d.get("jitter", True)),
                  int(d.get("russian_roulette", True)), controls)


class PtScene:
    """A path-tracer scene on the GPU (rn_pt_scene_create: raw::rt::finishPtScene). `sc` holds
    numpy arrays: pos (n,3), nrm (n,3), uv (n,2), idx (t,3), tri_tex (t,), tex_entries (k,3),
    texels, materials (k,7: base_factor, roughness, metallic, specular, emission), sun_dir,
    sun_irr, sky."""

    def __init__(self, sc: dict):
        f32 = lambda a: np.ascontiguousarray(a, np.float32)  # noqa: E731
        u32 = lambda a: np.ascontiguousarray(a, np.uint32)  # noqa: E731
        self._keep = dict(pos=f32(sc["pos"]), nrm=f32(sc["nrm"]), uv=f32(sc["uv"]), idx=u32(sc["idx"]),
                          tri_tex=u32(sc["tri_tex"]), tex_entries=u32(sc["tex_entries"]), texels=u32(sc["texels"]))
        mats = np.asarray(sc["materials"], np.float32).reshape(-1, 7)
        self._mats = (PtMaterial * len(mats))(*[PtMaterial(m[0], m[1], m[2], m[3], (C.c_float * 3)(*m[4:7])) for m in mats])
        k = self._keep
        p = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
        desc = PtSceneDesc(p(k["pos"]), p(k["nrm"]), p(k["uv"]), k["pos"].size // 3, p(k["idx"]), p(k["tri_tex"]),
                           k["tri_tex"].size, p(k["tex_entries"]), k["tex_entries"].size // 3, p(k["texels"]),
                           k["texels"].size, C.cast(self._mats, C.c_void_p), (C.c_float * 3)(*sc["sun_dir"]),
                           (C.c_float * 3)(*sc["sun_irr"]), (C.c_float * 3)(*sc["sky"]))
        self._h = C.c_void_p()
        st = Status()
        _check(lib().rn_pt_scene_create(C.byref(desc), C.byref(self._h), C.byref(st)), st)
        self._keep = None

    def info(self) -> dict:
        n, a = C.c_uint32(), C.c_float()
        st = Status()
        _check(lib().rn_pt_scene_info(self._h, C.byref(n), C.byref(a), C.byref(st)), st)
        return dict(emitters=n.value, emitter_area=a.value)

    def close(self) -> None:
        if self._h:
            lib().rn_pt_scene_free(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def path_trace(scene: PtScene, desc: dict, device: bool = False, planes=None):
    """rn_pathtrace: every AOV of raw::rt::pathTraceCpu as (h, w[, k]) arrays (numpy, or CUDA
    tensors with device=True). `planes` limits the outputs to those names."""
    h, w = int(desc["height"]), int(desc["width"])
    names = [n for n, _, _ in PT_AOVS if planes is None or n in planes]
    outs = {}
    if device:
        import torch
        tdt = {np.float32: torch.float32, np.int32: torch.int32}
        for name, k, dt in PT_AOVS:
            if name in names:
                outs[name] = torch.empty((h, w, k) if k > 1 else (h, w), dtype=tdt[dt], device="cuda")
        _use_torch_stream()
        ptr = lambda name: C.c_void_p(outs[name].data_ptr()) if name in outs else None  # noqa: E731
    else:
        for name, k, dt in PT_AOVS:
            if name in names:
                outs[name] = np.zeros((h, w, k) if k > 1 else (h, w), dt)
        ptr = lambda name: outs[name].ctypes.data_as(C.c_void_p) if name in outs else None  # noqa: E731
    o = PtOut(*[ptr(name) for name, _, _ in PT_AOVS])
    d = pt_desc(desc)
    st = Status()
    _check(lib().rn_pathtrace(scene._h, C.byref(d), RN_DEVICE_PTRS if device else 0, C.byref(o), C.byref(st)), st)
    return outs
