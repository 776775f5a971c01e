"""GPU parity of the three AO passes against the oracle, through the C ABI.

Bar (the parity rules of the path): the sampler's hash sequence, mask and pixel counts
bit-exact; with the host-libm calibration (the default) RT AO, sky, sun and SSAO are
bit-identical to the oracle, the error map too, RMSE within 1e-6 and the verdict equal.
Where this host's oracle reproduces the reference's x86-64 goldens, the GPU's outputs must
hash to the same SHA-256. Without calibration (RN_DEVICE_TRIG) RT AO stays within 1/spp per
pixel and SSAO within one tap (1/used) of the oracle.
"""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
IDENT = json.load(open(os.path.join(HERE, "golden", "identity.json")))
THREADS = os.cpu_count() or 1


def frame_inputs(O, w, h, cam=None):
    tris, nrm9, light = O.test_scene()
    _, pos, nrm, mask = O.rasterize(tris, nrm9, cam or O.DEFAULT_CAMERA, w, h)
    return tris, light, pos, nrm, mask


def gbuf(rn, pos, nrm, mask, cuda=False):
    if cuda:
        import torch
        return rn.GBuffer(torch.from_numpy(pos).cuda(), torch.from_numpy(nrm).cuda(), torch.from_numpy(mask).cuda())
    return rn.GBuffer(pos, nrm, mask)


# ---------------------------------------------------------------- reconcile
def test_reconcile_two_pixels(rn):
    # tests/test_reconcile.cpp:4-19
    a = np.array([[0.5, 0.8]], np.float32)
    b = np.array([[0.5, 0.4]], np.float32)
    m = np.ones((1, 2), np.uint8)
    r = rn.reconcile(a, b, m, 0.1)
    assert abs(r.error_map[0, 0]) < 1e-6 and abs(r.error_map[0, 1] - 0.4) < 1e-6
    assert abs(r.max_error - 0.4) < 1e-6 and r.pixels == 2 and not r.within_tolerance
    r2 = rn.reconcile(a, a, m, 0.1)
    assert r2.rmse == 0.0 and r2.within_tolerance


@pytest.mark.parametrize("shape", [(1, 1), (3, 7), (17, 33), (512, 512), (1001, 777), (2160, 3840)])
def test_reconcile_matches_oracle(rn, oracle, shape):
    rng = np.random.default_rng(shape[0] * 7 + shape[1])
    h, w = shape
    a = rng.random((h, w), dtype=np.float32)
    t = (np.floor(rng.random((h, w)) * 64) / 64).astype(np.float32)
    m = (rng.random((h, w)) < 0.6).astype(np.uint8)
    err, st = oracle.reconcile(a, t, m, 0.12)
    r = rn.reconcile(a, t, m, 0.12)
    assert np.array_equal(r.error_map, err)
    assert r.pixels == st["pixels"] and r.max_error == np.float32(st["maxError"])
    assert np.float32(r.rmse) == np.float32(st["rmse"])
    assert r.within_tolerance == st["within"]
    # both sums carry rounding (the sequential one more); they agree to ~1e-12 relative
    assert abs(r.sum_sq - st["sumSq"]) <= 1e-10 * max(1.0, st["sumSq"])


def test_reconcile_empty_mask_and_device_pointers(rn):
    import torch
    a = torch.rand(64, 48, device="cuda")
    m = torch.zeros(64, 48, dtype=torch.uint8, device="cuda")
    r = rn.reconcile(a, a * 0.5, m, 0.1)
    torch.cuda.synchronize()
    assert r.pixels == 0 and r.rmse == 0.0 and r.within_tolerance
    assert float(r.error_map.abs().sum()) == 0.0


def test_reconcile_is_deterministic(rn):
    rng = np.random.default_rng(3)
    a = rng.random((777, 1234), dtype=np.float32)
    t = rng.random((777, 1234), dtype=np.float32)
    m = np.ones((777, 1234), np.uint8)
    r1, r2 = rn.reconcile(a, t, m), rn.reconcile(a, t, m)
    assert r1.sum_sq == r2.sum_sq and r1.rmse == r2.rmse


# ---------------------------------------------------------------- SSAO
@pytest.mark.parametrize("size", [(48, 48), (256, 256), (333, 201)])
def test_ssao_bit_exact(rn, oracle, size):
    w, h = size
    _, _, pos, nrm, mask = frame_inputs(oracle, w, h)
    ref = oracle.ssao(pos, nrm, mask, 24, 2.0, THREADS)
    got = rn.compute_ssao(gbuf(rn, pos, nrm, mask), 24, 2.0)
    assert np.array_equal(got, ref), int((got != ref).sum())


def test_ssao_device_pointers_and_ragged_samples(rn, oracle):
    import torch
    _, _, pos, nrm, mask = frame_inputs(oracle, 200, 120, [3, 1.2, -4, 0, 0.5, 0, 0, 1, 0, 1.1])
    for samples, radius in ((1, 2.0), (7, 0.5), (24, 2.0), (40, 3.0), (0, 2.0)):
        ref = oracle.ssao(pos, nrm, mask, samples, radius, THREADS)
        got = rn.compute_ssao(gbuf(rn, pos, nrm, mask, cuda=True), samples, radius)
        torch.cuda.synchronize()
        assert np.array_equal(got.cpu().numpy(), ref), (samples, radius)


def test_ssao_uncalibrated_within_one_tap(rn, oracle):
    _, _, pos, nrm, mask = frame_inputs(oracle, 512, 512)
    ref = oracle.ssao(pos, nrm, mask, 24, 2.0, THREADS)
    got = rn.compute_ssao(gbuf(rn, pos, nrm, mask), 24, 2.0, device_trig=True)
    d = np.abs(got - ref)
    assert d.max() <= 1.0 / 1.0 + 1e-6
    assert (d > 0).mean() < 1e-3


# ---------------------------------------------------------------- RT AO
def test_rtao_small_scene_bit_exact(rn, oracle):
    # tests/test_ray_ao.cpp: 48 x 48, 32 spp, radius 2; and the crease is occluded
    tris, _, pos, nrm, mask = frame_inputs(oracle, 48, 48)
    acc = rn.LinearAccel(tris)
    got = rn.compute_rtao(gbuf(rn, pos, nrm, mask), acc, 32, 2.0)
    ref = oracle.trace(pos, nrm, mask, tris, 32, 2.0, threads=THREADS)
    assert np.array_equal(got, ref)
    cov = mask != 0
    assert 0.0 < got[cov].mean() <= 1.0 and got[cov].min() < 0.95


@pytest.mark.parametrize("spp,radius", [(1, 2.0), (7, 1.0), (64, 2.0), (100, 0.3)])
def test_rt_visibility_bit_exact(rn, oracle, spp, radius):
    tris, light, pos, nrm, mask = frame_inputs(oracle, 160, 128)
    acc = rn.LinearAccel(tris)
    ao, sky, sun = rn.compute_rt_visibility(gbuf(rn, pos, nrm, mask), acc, spp, radius, -light)
    rao, rsky, rsun = oracle.trace(pos, nrm, mask, tris, spp, radius, to_light=-light, threads=THREADS)
    assert np.array_equal(ao, rao), int((ao != rao).sum())
    assert np.array_equal(sky, rsky), int((sky != rsky).sum())
    assert np.array_equal(sun, rsun), int((sun != rsun).sum())


def test_rt_visibility_sun_forced_and_empty_scene(rn, oracle):
    tris, light, pos, nrm, mask = frame_inputs(oracle, 64, 64)
    acc = rn.LinearAccel(tris)
    _, _, sun = rn.compute_rt_visibility(gbuf(rn, pos, nrm, mask), acc, 4, 2.0, -light, sun_forced=True)
    assert (sun == 1.0).all()
    empty = rn.LinearAccel(np.zeros((0, 9), np.float32))
    ao, sky, sun = rn.compute_rt_visibility(gbuf(rn, pos, nrm, mask), empty, 8, 2.0, -light)
    assert (ao == 1.0).all() and (sky == 1.0).all() and (sun == 1.0).all()


def test_rtao_uncalibrated_within_one_sample(rn, oracle):
    tris, light, pos, nrm, mask = frame_inputs(oracle, 256, 256)
    acc = rn.LinearAccel(tris)
    got = rn.compute_rtao(gbuf(rn, pos, nrm, mask), acc, 64, 2.0, device_trig=True)
    ref = oracle.trace(pos, nrm, mask, tris, 64, 2.0, threads=THREADS)
    d = np.abs(got - ref)
    assert d.max() <= 1.0 / 64 + 1e-7
    assert (d == 0).mean() >= 0.999


# ---------------------------------------------------------------- whole AO frame
@pytest.mark.parametrize("case", sorted(IDENT["cases"]))
def test_frame_matches_oracle_and_goldens(rn, oracle, case):
    c = IDENT["cases"][case]
    w, h, cam = c["width"], c["height"], c["camera"]
    tris, light, pos, nrm, mask = frame_inputs(oracle, w, h, cam)
    acc = rn.LinearAccel(tris)
    out = rn.ao_frame(gbuf(rn, pos, nrm, mask), acc, 64, 2.0, 24, 0.12, to_light=-light)
    ao, sky, sun = oracle.trace(pos, nrm, mask, tris, 64, 2.0, to_light=-light, threads=THREADS)
    ss = oracle.ssao(pos, nrm, mask, 24, 2.0, THREADS)
    err, st = oracle.reconcile(ss, ao, mask, 0.12)
    for k, ref in (("ao", ao), ("sky", sky), ("sun", sun), ("ss", ss), ("err", err)):
        assert np.array_equal(out[k], ref), (k, int((out[k] != ref).sum()))
    rec = out["rec"]
    assert rec.pixels == st["pixels"] and rec.max_error == np.float32(st["maxError"])
    assert abs(rec.rmse - st["rmse"]) <= 1e-6 and rec.within_tolerance == st["within"]
    # the reference's own bytes, where this host's oracle reproduces them
    digests = {"ao_rt.pfm": oracle.sha256(oracle.pfm1_bytes(ao)), "ao_ss.pfm": oracle.sha256(oracle.pfm1_bytes(ss)),
               "mask.pgm": oracle.sha256(oracle.mask_pgm_bytes(mask)),
               "ao_error.pgm": oracle.sha256(oracle.pgm_bytes(err))}
    if digests == c["files"]:
        got = {"ao_rt.pfm": oracle.sha256(oracle.pfm1_bytes(out["ao"])),
               "ao_ss.pfm": oracle.sha256(oracle.pfm1_bytes(out["ss"])),
               "mask.pgm": digests["mask.pgm"], "ao_error.pgm": oracle.sha256(oracle.pgm_bytes(out["err"]))}
        assert got == c["files"]
        assert rec.pixels == c["exact"]["pixels"] and rec.within_tolerance == c["exact"]["within"]
        assert np.float32(rec.rmse) == np.float32(c["exact"]["rmse"])


def test_frame_device_pointers_equal_host_path(rn, oracle):
    import torch
    tris, light, pos, nrm, mask = frame_inputs(oracle, 300, 200)
    acc = rn.LinearAccel(torch.from_numpy(tris).cuda())
    a = rn.ao_frame(gbuf(rn, pos, nrm, mask, cuda=True), acc, 16, 2.0, 24, 0.12, to_light=-light)
    torch.cuda.synchronize()
    b = rn.ao_frame(gbuf(rn, pos, nrm, mask), acc, 16, 2.0, 24, 0.12, to_light=-light)
    for k in ("ao", "sky", "sun", "ss", "err"):
        assert np.array_equal(a[k].cpu().numpy(), b[k]), k
    assert a["rec"].sum_sq == b["rec"].sum_sq


def test_4k_256spp_strided_rows_match_oracle(rn, oracle):
    """The full config (3840 x 2160, 256 spp): the GPU frame against the oracle on every
    97th row, plus size-independent properties of the whole frame."""
    w, h = 3840, 2160
    tris, light, pos, nrm, mask = frame_inputs(oracle, w, h)
    assert int(mask.sum()) == 3992795                       # covered pixels of the 4K default view
    acc = rn.LinearAccel(tris)
    out = rn.ao_frame(gbuf(rn, pos, nrm, mask), acc, 256, 2.0, 24, 0.12, to_light=-light)
    ao = np.zeros((h, w), np.float32)
    sky = np.zeros((h, w), np.float32)
    sun = np.zeros((h, w), np.float32)
    import ctypes as C
    L = oracle.lib()
    L.rno_trace(w, h, pos, nrm, mask, None, tris, len(tris), 256, 2.0, C.cast((C.c_float * 3)(*(-light)), C.c_void_p),
                0, ao, sky.ctypes.data_as(C.c_void_p), sun.ctypes.data_as(C.c_void_p), THREADS, 5, 97)
    rows = np.arange(5, h, 97)
    assert np.array_equal(out["ao"][rows], ao[rows])
    assert np.array_equal(out["sky"][rows], sky[rows])
    assert np.array_equal(out["sun"][rows], sun[rows])
    cov = mask != 0
    assert (out["ao"][~cov] == 1).all() and (out["sky"] <= out["ao"]).all()
    q = out["ao"][cov] * 256
    assert np.array_equal(q, np.round(q))                   # k / spp exactly
    assert out["rec"].pixels == 3992795


# ---------------------------------------------------------------- G-buffer and counters
@pytest.mark.parametrize("case", ["default", "default-512", "close-512", "low-512", "wide-1440x900"])
def test_raster_matches_oracle_and_mask_golden(rn, oracle, case):
    import scene as scenes
    c = IDENT["cases"][case]
    w, h, cam = c["width"], c["height"], c["camera"]
    sc = scenes.build_test_scene(cam)
    g, depth = rn.rasterize(sc.tris, sc.normals, sc.camera, w, h, want_depth=True)
    tris, nrm9, _ = oracle.test_scene()
    rd, rp, rnm, rm = oracle.rasterize(tris, nrm9, cam, w, h)
    assert np.array_equal(g.mask, rm)
    assert np.array_equal(g.position, rp) and np.array_equal(g.normal, rnm)
    assert np.array_equal(depth, rd)
    if oracle.sha256(oracle.mask_pgm_bytes(rm)) == c["files"]["mask.pgm"]:
        assert oracle.sha256(oracle.mask_pgm_bytes(g.mask)) == c["files"]["mask.pgm"]


def test_raster_near_clip_and_device_pointers(rn, oracle):
    import torch
    import scene as scenes
    cam = [0.5, 0.6, 0.3, 0.0, 0.5, 0.0, 0.0, 1.0, 0.0, 1.4]    # inside the box's corner: triangles cross the near plane
    sc = scenes.build_test_scene(cam)
    g = rn.rasterize(torch.from_numpy(sc.tris).cuda(), torch.from_numpy(sc.normals).cuda(), cam, 200, 150)
    torch.cuda.synchronize()
    tris, nrm9, _ = oracle.test_scene()
    _, rp, rnm, rm = oracle.rasterize(tris, nrm9, cam, 200, 150)
    assert np.array_equal(g.mask.cpu().numpy(), rm) and np.array_equal(g.position.cpu().numpy(), rp)
    assert np.array_equal(g.normal.cpu().numpy(), rnm)


def test_trace_stats_counts_rays(rn, oracle):
    tris, light, pos, nrm, mask = frame_inputs(oracle, 256, 256)
    acc = rn.LinearAccel(tris)
    st = rn.trace_stats(gbuf(rn, pos, nrm, mask), acc, 16, 2.0, to_light=-light, tile_stride=1)
    assert st["rays"] == int(mask.sum()) * 16
    ao = oracle.trace(pos, nrm, mask, tris, 16, 2.0, threads=THREADS)
    assert st["sky_rays"] == int(round(float((ao[mask != 0] * 16).sum())))
    assert st["nodes"] >= st["rays"] + int(mask.sum()) and st["tris"] > 0   # one walk per ray and per sun ray
