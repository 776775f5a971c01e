"""ctypes binding of the AO-path oracle (test infrastructure only).

Loads ``oracle/librn_oracle.so`` (the C restatement in ``rn_oracle.c``) and, where it was
built, ``oracle/_ref/libref_ao.so`` (the reference's own sources). Only the tests, the
smoke check and the benchmark's CPU-baseline leg import this module: it is what results
are compared against, never the thing measured or shipped.

File encodings follow src/core/image.cpp:34-106 of the reference: ``Pf`` PFM with rows
bottom-to-top, the coverage mask as P5 PGM 255/0, and 8-bit previews ``v*255+0.5``.
"""
from __future__ import annotations

import ctypes as C
import hashlib
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "librn_oracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libref_ao.so")

# The CLI's fixed sampling (raw/renderer/render.hpp:25-27) and its default camera
# (raw/tools/cli_params.hpp:16-21).
RT_SAMPLES, SS_SAMPLES, AO_RADIUS, TOLERANCE = 64, 24, 2.0, 0.12
DEFAULT_CAMERA = (4.0, 4.0, 6.0, 0.0, 1.0, 0.0, 0.0, 1.0, 0.0, 0.9)

_F = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_U8 = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
_I32 = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_U64 = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")
_D = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")


def build(with_ref: bool | None = None) -> None:
    """Compile the oracle (and the reference harness when the raw-native tree exists: the
    tree named by RN_REFERENCE_DIR, else the location oracle/Makefile names)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    if with_ref is False:
        return
    extra = ["REF=" + os.environ["RN_REFERENCE_DIR"]] if os.environ.get("RN_REFERENCE_DIR") else []
    jobs = "-j%d" % (os.cpu_count() or 4)
    subprocess.run(["make", "-s", jobs, "-C", HERE, "ref" if with_ref else "ref-if-present"] + extra, check=True)


def reference_dir() -> str | None:
    """The raw-native tree the reference harness was built from (RN_REFERENCE_DIR first), or
    None where no tree is present (the GPU host)."""
    d = os.environ.get("RN_REFERENCE_DIR")
    if not d:
        try:
            d = open(os.path.join(HERE, "_ref", "reference_dir")).read().strip()
        except OSError:
            return None
    return d if os.path.isdir(os.path.join(d, "src", "renderer")) else None


_lib = None
_ref = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build(with_ref=False)
        L = C.CDLL(LIB)
        L.rno_hash01.restype = C.c_float
        L.rno_hash01.argtypes = [C.c_uint32] * 3
        L.rno_intersect.argtypes = [_F, _F, C.POINTER(C.c_float)]
        L.rno_accel_build.restype = C.c_void_p
        L.rno_accel_build.argtypes = [_F, C.c_int]
        L.rno_accel_free.argtypes = [C.c_void_p]
        L.rno_accel_nodes.argtypes = [C.c_void_p]
        L.rno_occluded.argtypes = [C.c_void_p, _F, C.c_float]
        L.rno_occluded_scan.argtypes = [_F, C.c_int, _F, C.c_float]
        L.rno_occluded_scan_batch.argtypes = [_F, C.c_int, _F, _F, C.c_int, _U8, C.c_int]
        L.rno_closest_scan_batch.argtypes = [_F, C.c_int, _F, _F, C.c_int, _I32, _F, C.c_int]
        L.rno_hybrid.argtypes = [C.c_int, C.c_int, _F, _F, C.c_void_p, _U8, _F, C.c_int, _F, _F, _F, _I32, _F,
                                 C.c_int]
        L.rno_trace.argtypes = [C.c_int, C.c_int, _F, _F, _U8, C.c_void_p, _F, C.c_int, C.c_int,
                                C.c_float, C.c_void_p, C.c_int, _F, C.c_void_p, C.c_void_p,
                                C.c_int, C.c_int, C.c_int]
        L.rno_ssao.argtypes = [C.c_int, C.c_int, _F, _F, _U8, C.c_int, C.c_float, _F, C.c_int]
        L.rno_reconcile.argtypes = [C.c_int, C.c_int, _F, _F, _U8, C.c_float, _F,
                                    C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_int),
                                    C.POINTER(C.c_int), C.POINTER(C.c_double)]
        L.rno_test_scene.restype = C.c_int
        L.rno_test_scene.argtypes = [_F, _F, _F]
        L.rno_rasterize.argtypes = [_F, _F, C.c_int, _F, C.c_int, C.c_int, _F, _F, _F, _U8]
        L.rno_rasterize_ex.argtypes = [_F, _F, C.c_int, _F, C.c_int, C.c_int, _F, _F, _F, _U8, _I32]
        L.rno_test_scene_albedo.argtypes = [_F]
        L.rno_view_proj.argtypes = [_F, C.c_int, C.c_int, _F]
        L.rno_shade.argtypes = [C.c_int, C.c_int, _F, _F, _U8, C.c_int, _F, _F, _F, C.c_float, _F, _F]
        L.rno_motion.restype = C.c_int
        L.rno_motion.argtypes = [C.c_int, C.c_int, _F, _U8, _F, _F, _F]
        L.rno_view_gbuffer.argtypes = [C.c_int, C.c_int, _F, _F, _U8, _F, _F, _F, _F]
        L.rno_gtao.argtypes = [C.c_int, C.c_int, _F, _F, _F, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int, _D]
        L.rno_morton_keys.argtypes = [_F, C.c_int, _U64]
        L.rno_ploc_build.restype = C.c_int
        L.rno_ploc_build.argtypes = [_F, C.c_int, C.c_int, _I32, C.POINTER(C.c_uint32)]
        L.rno_tree_hash.restype = C.c_uint64
        L.rno_tree_hash.argtypes = [_I32, C.c_int]
        L.rno_soup.argtypes = [C.c_int, C.c_uint64, _F]
        _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_LIB)


def ref() -> C.CDLL:
    global _ref
    if _ref is None:
        R = C.CDLL(REF_LIB)
        R.ref_render_default.argtypes = [C.c_int, C.c_int, _F, C.c_int, C.c_float, C.c_int, C.c_float,
                                         C.c_int, _F, _F, _U8, _F, _F, _F, _F, _F, _F]
        R.ref_trace.argtypes = [C.c_int, C.c_int, _F, _F, _U8, _F, C.c_int, C.c_int, C.c_float,
                                C.c_void_p, _F, C.c_void_p, C.c_void_p, C.c_int]
        R.ref_ssao.argtypes = [C.c_int, C.c_int, _F, _F, _U8, C.c_int, C.c_float, _F, C.c_int]
        R.ref_reconcile.argtypes = [C.c_int, C.c_int, _F, _F, _U8, C.c_float, _F, _F]
        R.ref_ploc.restype = C.c_int
        R.ref_ploc.argtypes = [_F, C.c_int, C.c_int, _I32, C.POINTER(C.c_uint32)]
        R.ref_closest.argtypes = [_F, C.c_int, _F, _F, C.c_int, _I32, _F]
        R.ref_motion.restype = C.c_int
        R.ref_motion.argtypes = [C.c_int, C.c_int, _F, _U8, _F, _F, _F]
        R.ref_view_gbuffer.argtypes = [C.c_int, C.c_int, _F, _F, _U8, _F, _F, _F, _F]
        R.ref_gtao.argtypes = [C.c_int, C.c_int, _F, _F, _F, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int,
                               _D]
        _ref = R
    return _ref


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


# ---------------------------------------------------------------- scene and G-buffer
def test_scene():
    """The built-in scene (src/scene/scene.cpp:18-32): tris (14, 9), corner normals, light."""
    tris = np.zeros((14, 9), np.float32)
    nrm = np.zeros((14, 9), np.float32)
    light = np.zeros(3, np.float32)
    n = lib().rno_test_scene(tris, nrm, light)
    return tris[:n], nrm[:n], light


def rasterize(tris, nrm, cam, w: int, h: int):
    """G-buffer (depth, position (h,w,3), normal (h,w,3), mask (h,w) u8) of a triangle list."""
    tris, nrm = _f32(tris).reshape(-1, 9), _f32(nrm).reshape(-1, 9)
    depth = np.empty((h, w), np.float32)
    pos = np.empty((h, w, 3), np.float32)
    nr = np.empty((h, w, 3), np.float32)
    mask = np.empty((h, w), np.uint8)
    lib().rno_rasterize(tris, nrm, len(tris), _f32(cam), w, h, depth, pos, nr, mask)
    return depth, pos, nr, mask


# ---------------------------------------------------------------- the three passes
def trace(pos, nrm, mask, tris, spp, radius, to_light=None, accel="bvh", threads=1,
          row0=0, row_stride=1):
    """computeRTAO (to_light None) or computeRTVisibility; returns ao or (ao, sky, sun)."""
    pos, nrm = _f32(pos), _f32(nrm)
    mask = np.ascontiguousarray(mask, np.uint8)
    tris = _f32(tris).reshape(-1, 9)
    h, w = mask.shape
    ao = np.zeros((h, w), np.float32)
    sky = np.zeros((h, w), np.float32) if to_light is not None else None
    sun = np.zeros((h, w), np.float32) if to_light is not None else None
    L = lib()
    handle = L.rno_accel_build(tris, len(tris)) if accel == "bvh" else None
    tl = _f32(to_light) if to_light is not None else None
    try:
        L.rno_trace(w, h, pos, nrm, mask, handle, tris, len(tris), int(spp), float(radius),
                    _ptr(tl), 0, ao, _ptr(sky), _ptr(sun), int(threads), int(row0), int(row_stride))
    finally:
        if handle:
            L.rno_accel_free(handle)
    return ao if to_light is None else (ao, sky, sun)


def occluded_scan(tris, rays, tmax, threads=1):
    """Any-hit by scanning every triangle (the reference's test oracle) for rays (n, 6)."""
    tris = _f32(tris).reshape(-1, 9)
    rays = _f32(rays).reshape(-1, 6)
    hit = np.zeros(len(rays), np.uint8)
    lib().rno_occluded_scan_batch(tris, len(tris), rays, _f32(tmax), len(rays), hit, int(threads))
    return hit


def closest_scan(tris, rays, tmax, threads=1):
    """rt::closest by scanning every triangle (ties to the lowest index) for rays (n, 6):
    (triangle index or -1, t or -1)."""
    tris = _f32(tris).reshape(-1, 9)
    rays = _f32(rays).reshape(-1, 6)
    tri = np.zeros(len(rays), np.int32)
    t = np.zeros(len(rays), np.float32)
    lib().rno_closest_scan_batch(tris, len(tris), rays, _f32(tmax), len(rays), tri, t, int(threads))
    return tri, t


def hybrid(pos, nrm, mask, tris, eye, sun, geo_normal=None, threads=1):
    """The hybrid pass's per-pixel rule over a G-buffer (scans): (lit, refl_tri, refl_t).
    geo_normal: the geometric normals (h, w, 3), or None for the G-buffer normals."""
    mask = np.ascontiguousarray(mask, np.uint8)
    h, w = mask.shape
    tris = _f32(tris).reshape(-1, 9)
    lit = np.zeros((h, w), np.float32)
    tri = np.zeros((h, w), np.int32)
    t = np.zeros((h, w), np.float32)
    ng = _f32(geo_normal) if geo_normal is not None else None
    lib().rno_hybrid(w, h, _f32(pos), _f32(nrm), ng.ctypes.data if ng is not None else None, mask, tris, len(tris),
                     _f32(eye), _f32(sun), lit, tri, t, int(threads))
    return lit, tri, t


def ssao(pos, nrm, mask, samples=SS_SAMPLES, radius=AO_RADIUS, threads=1):
    mask = np.ascontiguousarray(mask, np.uint8)
    h, w = mask.shape
    out = np.zeros((h, w), np.float32)
    lib().rno_ssao(w, h, _f32(pos), _f32(nrm), mask, int(samples), float(radius), out, int(threads))
    return out


def reconcile(approx, truth, mask, tolerance=TOLERANCE):
    """(error map, dict(rmse, maxError, pixels, within, sumSq))."""
    mask = np.ascontiguousarray(mask, np.uint8)
    h, w = mask.shape
    err = np.zeros((h, w), np.float32)
    rmse, mx, s = C.c_float(), C.c_float(), C.c_double()
    n, within = C.c_int(), C.c_int()
    lib().rno_reconcile(w, h, _f32(approx), _f32(truth), mask, float(tolerance), err,
                        C.byref(rmse), C.byref(mx), C.byref(n), C.byref(within), C.byref(s))
    return err, dict(rmse=rmse.value, maxError=mx.value, pixels=n.value, within=bool(within.value),
                     sumSq=s.value)


# ---------------------------------------------------------------- PLOC
def ploc(tris, radius=16):
    """(nodes (2n-1, 9) int32, root, rounds) as rt::buildPloc builds them."""
    tris = _f32(tris).reshape(-1, 9)
    n = len(tris)
    nodes = np.zeros((max(2 * n - 1, 1), 9), np.int32)
    rounds = C.c_uint32()
    root = lib().rno_ploc_build(tris, n, int(radius), nodes, C.byref(rounds))
    return nodes, root, rounds.value


def morton_keys(tris):
    tris = _f32(tris).reshape(-1, 9)
    keys = np.zeros(len(tris), np.uint64)
    lib().rno_morton_keys(tris, len(tris), keys)
    return keys


def tree_hash(nodes) -> str:
    nodes = np.ascontiguousarray(nodes, np.int32)
    return "%016x" % lib().rno_tree_hash(nodes, len(nodes))


def soup(count: int, seed: int):
    tris = np.zeros((count, 9), np.float32)
    lib().rno_soup(count, seed, tris)
    return tris


# ---------------------------------------------------------------- file bytes and digests
def pfm1_bytes(buf) -> bytes:
    buf = np.asarray(buf, np.float32)
    h, w = buf.shape
    return b"Pf\n%d %d\n-1.0\n" % (w, h) + np.ascontiguousarray(buf[::-1]).astype("<f4").tobytes()


def mask_pgm_bytes(mask) -> bytes:
    mask = np.asarray(mask)
    h, w = mask.shape
    return b"P5\n%d %d\n255\n" % (w, h) + np.where(mask != 0, 255, 0).astype(np.uint8).tobytes()


def pgm_bytes(buf) -> bytes:
    buf = np.asarray(buf, np.float32)
    h, w = buf.shape
    v = (np.clip(buf, np.float32(0), np.float32(1)) * np.float32(255.0) + np.float32(0.5)).astype(np.uint8)
    return b"P5\n%d %d\n255\n" % (w, h) + v.tobytes()


def sha256(b: bytes) -> str:
    return hashlib.sha256(b).hexdigest()


# ---------------------------------------------------------------- the whole frame
def test_scene_albedo():
    a = np.zeros((14, 3), np.float32)
    lib().rno_test_scene_albedo(a)
    return a


def rasterize_ex(tris, nrm, cam, w: int, h: int):
    """rasterize plus the triangle each covered pixel shows (-1 elsewhere)."""
    tris = _f32(tris).reshape(-1, 9)
    depth = np.zeros((h, w), np.float32)
    pos = np.zeros((h, w, 3), np.float32)
    nr = np.zeros((h, w, 3), np.float32)
    mask = np.zeros((h, w), np.uint8)
    tri = np.zeros((h, w), np.int32)
    lib().rno_rasterize_ex(tris, _f32(nrm).reshape(-1, 9), len(tris), np.asarray(cam, np.float32), w, h, depth, pos,
                           nr, mask, tri)
    return depth, pos, nr, mask, tri


def view_proj(cam, w: int, h: int):
    vp = np.zeros(16, np.float32)
    lib().rno_view_proj(np.asarray(cam, np.float32), w, h, vp)
    return vp


def shade(nrm, albedo, mask, model, a_or_sky, sun, ldir, li=1.0):
    """(frame clamped, hdr) as shadeV2/shadeHDRV2 (model 2) or shade/shadeHDR (model 1)."""
    mask = np.ascontiguousarray(mask, np.uint8)
    h, w = mask.shape
    frame = np.zeros((h, w, 3), np.float32)
    hdr = np.zeros((h, w, 3), np.float32)
    sun = _f32(sun) if sun is not None else np.zeros((h, w), np.float32)
    lib().rno_shade(w, h, _f32(nrm), _f32(albedo), mask, int(model), _f32(a_or_sky), sun, _f32(ldir), float(li), frame,
                    hdr)
    return frame, hdr


def motion(pos, mask, vp, prev_vp, use_ref=False):
    mask = np.ascontiguousarray(mask, np.uint8)
    h, w = mask.shape
    m = np.zeros((h, w, 2), np.float32)
    valid = (ref().ref_motion if use_ref else lib().rno_motion)(w, h, _f32(pos), mask, _f32(vp), _f32(prev_vp), m)
    return m, valid


def ppm_bytes(frame) -> bytes:
    """frame.ppm of a clamped frame (src/core/image.cpp:9-18)."""
    f = np.asarray(frame, np.float32)
    h, w, _ = f.shape
    v = (np.clip(f, 0.0, 1.0) * np.float32(255.0) + np.float32(0.5)).astype(np.uint8)
    return b"P6\n%d %d\n255\n" % (w, h) + v.tobytes()


def pfm3_bytes(img) -> bytes:
    """frame_hdr.pfm (src/core/image.cpp:40-51): rows bottom to top, little-endian floats."""
    f = np.asarray(img, np.float32)
    h, w, _ = f.shape
    return b"PF\n%d %d\n-1.0\n" % (w, h) + np.ascontiguousarray(f[::-1]).astype("<f4").tobytes()


# ---------------------------------------------------------------- GTAO (raw::post)
def view_gbuffer(pos, nrm, mask, cam, use_ref=False):
    """raw::post::viewGBuffer: (view positions (h,w,3), view normals, view depth (-1 empty))."""
    mask = np.ascontiguousarray(mask, np.uint8)
    h, w = mask.shape
    vp = np.zeros((h, w, 3), np.float32)
    vn = np.zeros((h, w, 3), np.float32)
    vd = np.zeros((h, w), np.float32)
    cam10 = np.ascontiguousarray(cam, np.float32)
    (ref().ref_view_gbuffer if use_ref else lib().rno_view_gbuffer)(w, h, _f32(pos), _f32(nrm), mask, cam10, vp, vn, vd)
    return vp, vn, vd


def gtao(vpos, vnrm, vdepth, fovy, radius=0.5, slices=16, steps=16, use_ref=False):
    """raw::post::gtao (FP64) on a view-space G-buffer; aspect = w / h as a float."""
    h, w = vdepth.shape
    out = np.zeros((h, w), np.float64)
    tan_half = float(np.tan(0.5 * np.float64(np.float32(fovy))))
    aspect = float(np.float32(w) / np.float32(h))
    (ref().ref_gtao if use_ref else lib().rno_gtao)(w, h, _f32(vpos), _f32(vnrm), _f32(vdepth), tan_half, aspect,
                                                   float(radius), int(slices), int(steps), out)
    return out


def render_default(w, h, cam=DEFAULT_CAMERA, spp=RT_SAMPLES, radius=AO_RADIUS, ss_samples=SS_SAMPLES,
                   tolerance=TOLERANCE, threads=1, accel="bvh"):
    """The CLI's frame on the oracle: G-buffer, ao/sky/sun, SSAO, reconcile."""
    tris, nrm9, light = test_scene()
    _, pos, nrm, mask = rasterize(tris, nrm9, cam, w, h)
    ao, sky, sun = trace(pos, nrm, mask, tris, spp, radius, to_light=-light, accel=accel, threads=threads)
    ss = ssao(pos, nrm, mask, ss_samples, radius, threads)
    err, st = reconcile(ss, ao, mask, tolerance)
    return dict(tris=tris, pos=pos, nrm=nrm, mask=mask, ao=ao, sky=sky, sun=sun, ss=ss, err=err, stats=st,
                light=light)


# ---------------------------------------------------------------- path tracer (raw::rt, interface v4)
PT_FLOATS = 64 * 128 * 2 + 128 * 2          # the lobe's energy table (rt_pt_math.hpp:86-90)
PT_CONTROLS = dict(drop_lambert_cosine=1, mis_weight_one=2, aov_drop_specular_indirect=4,
                   aov_emission_to_diffuse=8, legacy_lobe_v2=16)
PT_AOVS = (("radiance", 3, np.float32), ("albedo", 3, np.float32), ("normal", 3, np.float32),
           ("depth", 1, np.float32), ("variance", 1, np.float32), ("triangle", 1, np.int32),
           ("motion", 2, np.float32), ("diffuse", 3, np.float32), ("specular", 3, np.float32),
           ("emission", 3, np.float32), ("diffuse_albedo", 3, np.float32), ("specular_albedo", 3, np.float32),
           ("diffuse_variance", 1, np.float32), ("specular_variance", 1, np.float32))


class PtSceneC(C.Structure):
    _fields_ = [("pos", C.c_void_p), ("nrm", C.c_void_p), ("uv", C.c_void_p), ("nvert", C.c_uint32),
                ("idx", C.c_void_p), ("tri_tex", C.c_void_p), ("ntri", C.c_uint32),
                ("tex_entries", C.c_void_p), ("ntex", C.c_uint32), ("texels", C.c_void_p), ("ntexels", C.c_uint32),
                ("materials", C.c_void_p), ("sun_dir", C.c_float * 3), ("sun_irr", C.c_float * 3),
                ("sky", C.c_float * 3)]


class PtDescC(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("spp", C.c_uint32), ("spp_begin", C.c_uint32), ("max_bounces", C.c_uint32),
                ("width", C.c_int32), ("height", C.c_int32), ("camera", C.c_float * 10), ("previous", C.c_float * 10),
                ("jitter", C.c_int32), ("rr", C.c_int32), ("controls", C.c_uint32)]


class PtOutC(C.Structure):
    _fields_ = [(name, C.c_void_p) for name, _, _ in PT_AOVS]


def pt_scene_struct(sc: dict):
    """A path-tracer scene dict (pos (n,3), nrm (n,3), uv (n,2), idx (t,3) u32, tri_tex (t,) u32,
    tex_entries (k,3) u32, texels u32, materials (k,7), sun_dir, sun_irr, sky) as the C struct;
    returns (struct, the arrays it points into)."""
    keep = dict(pos=_f32(sc["pos"]), nrm=_f32(sc["nrm"]), uv=_f32(sc["uv"]),
                idx=np.ascontiguousarray(sc["idx"], np.uint32), tri_tex=np.ascontiguousarray(sc["tri_tex"], np.uint32),
                tex_entries=np.ascontiguousarray(sc["tex_entries"], np.uint32),
                texels=np.ascontiguousarray(sc["texels"], np.uint32), materials=_f32(sc["materials"]))
    s = PtSceneC(_ptr(keep["pos"]), _ptr(keep["nrm"]), _ptr(keep["uv"]), keep["pos"].size // 3,
                 _ptr(keep["idx"]), _ptr(keep["tri_tex"]), keep["tri_tex"].size, _ptr(keep["tex_entries"]),
                 keep["tex_entries"].size // 3, _ptr(keep["texels"]), keep["texels"].size, _ptr(keep["materials"]),
                 (C.c_float * 3)(*sc["sun_dir"]), (C.c_float * 3)(*sc["sun_irr"]), (C.c_float * 3)(*sc["sky"]))
    return s, keep


def pt_desc_struct(d: dict):
    controls = 0
    for k in d.get("controls", ()):
        controls |= PT_CONTROLS[k]
    return PtDescC(int(d.get("seed", 1)), int(d.get("spp", 16)), int(d.get("spp_begin", 0)),
                   int(d.get("max_bounces", 64)), int(d["width"]), int(d["height"]), (C.c_float * 10)(*d["camera"]),
                   (C.c_float * 10)(*d.get("previous", d["camera"])), int(d.get("jitter", True)),
                   int(d.get("russian_roulette", True)), controls)


def pt_energy_table(threads=None, use_ref=False):
    t = np.zeros(PT_FLOATS, np.float32)
    if use_ref:
        ref().ref_pt_energy_table(t.ctypes.data_as(C.c_void_p))
    else:
        lib().rno_pt_energy_table(t.ctypes.data_as(C.c_void_p), int(threads or os.cpu_count() or 1))
    return t


def pathtrace(scene: dict, desc: dict, threads=None, use_ref=False, table=None):
    """raw::rt::pathTraceCpu of a v2 scene: a dict of every AOV ((h, w[, k]) arrays) and the
    emitter count. use_ref runs the reference's own build (oracle/_ref)."""
    s, keep = pt_scene_struct(scene)
    d = pt_desc_struct(desc)
    h, w = int(desc["height"]), int(desc["width"])
    outs = {name: np.zeros((h, w, k) if k > 1 else (h, w), dt) for name, k, dt in PT_AOVS}
    o = PtOutC(*[_ptr(outs[name]) for name, _, _ in PT_AOVS])
    T = int(threads or os.cpu_count() or 1)
    if use_ref:
        n = ref().ref_pathtrace(C.byref(s), C.byref(d), T, C.byref(o))
    else:
        tab = None if table is None else np.ascontiguousarray(table, np.float32)
        n = lib().rno_pathtrace(C.byref(s), C.byref(d), _ptr(tab), T, C.byref(o))
    outs["emitters"] = n
    return outs


def pt_reference_scene(name: str, emission=1.0, albedo=0.5, material=None, sky=(1.0, 1.0, 1.0)):
    """The reference's own lit scene by name (retro_room, iso_street, dense_block, furnace,
    white_plane) from its build (oracle/_ref): (scene dict, camera 10 floats)."""
    R = ref()
    counts = (C.c_uint32 * 5)()
    mat7 = np.asarray(material if material is not None else (1.0, 0.8, 0.0, 0.5, 0, 0, 0), np.float32)
    sky3 = np.asarray(sky, np.float32)
    args = [name.encode(), C.c_float(emission), C.c_float(albedo), _ptr(mat7), _ptr(sky3), counts]
    assert R.ref_pt_scene(*args, *([None] * 10)) == 0, name
    nv, nt, nk, nx = counts[0], counts[1], counts[2], counts[3]
    sc = dict(pos=np.zeros((nv, 3), np.float32), nrm=np.zeros((nv, 3), np.float32), uv=np.zeros((nv, 2), np.float32),
              idx=np.zeros((nt, 3), np.uint32), tri_tex=np.zeros(nt, np.uint32), tex_entries=np.zeros((nk, 3), np.uint32),
              texels=np.zeros(nx, np.uint32), materials=np.zeros((nk, 7), np.float32))
    light9, cam10 = np.zeros(9, np.float32), np.zeros(10, np.float32)
    R.ref_pt_scene(*args, *[_ptr(sc[k]) for k in ("pos", "nrm", "uv", "idx", "tri_tex", "tex_entries", "texels",
                                                    "materials")], _ptr(light9), _ptr(cam10))
    sc.update(sun_dir=light9[0:3].copy(), sun_irr=light9[3:6].copy(), sky=light9[6:9].copy())
    return sc, cam10
