"""Batched multi-view AO and the large synthetic scenes on the GPU.

- A batch (one traversal launch over all views, one SSAO launch, replayed from a CUDA graph)
  gives, per view, exactly what the single-frame call gives on that view.
- On the seeded 744,000-triangle scene, the GPU G-buffer equals the CPU rasterizer bit for
  bit and the traced AO (radius 1.0) equals the oracle's (its SAH BVH) bit for bit.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
THREADS = os.cpu_count() or 1


@pytest.fixture(scope="module")
def big_scene():
    import scene as scenes
    return scenes.build_synthetic_scene(1, 2000, 500)


def _gbuf(rn, sc, cam, w, h):
    import torch
    return rn.rasterize(torch.from_numpy(sc.tris).cuda(), torch.from_numpy(sc.normals).cuda(), cam, w, h)


def test_batch_equals_single_frames(rn):
    import torch
    import scene as scenes
    sc = scenes.build_test_scene()
    acc = rn.LinearAccel(torch.from_numpy(sc.tris).cuda())
    specs = [(256, 256, 16, 2.0, (4, 4, 6, 0, 1, 0, 0, 1, 0, 0.9)), (333, 127, 64, 1.0, (0, 9, 3, 0, 0.5, 0, 0, 1, 0, 0.9)),
             (64, 96, 7, 2.0, (6, 1.5, 2, 0, 1, 0, 0, 1, 0, 0.9)), (200, 150, 32, 0.5, (2, 2.5, 3, 0, 0.8, 0, 0, 1, 0, 0.7))]
    views = [dict(g=_gbuf(rn, sc, cam, w, h), spp=spp, radius=r) for w, h, spp, r, cam in specs]
    b = rn.Batch(acc, views, ss_samples=24, tolerance=0.12, to_light=sc.to_light)
    res = b.run()
    torch.cuda.synchronize()
    for k, v in enumerate(views):
        ref = rn.ao_frame(v["g"], acc, v["spp"], v["radius"], 24, 0.12, to_light=sc.to_light)
        torch.cuda.synchronize()
        for key in ("ao", "sky", "sun", "ss", "err"):
            assert torch.equal(b.outputs[k][key], ref[key]), (k, key)
        assert res[k].pixels == ref["rec"].pixels and res[k].rmse == ref["rec"].rmse
        # the FP64 sum's order follows the SSAO tiling (the batch's 32 x 8 tiles, the single
        # frame's tuned tile height): equal to rounding
        assert abs(res[k].sum_sq - ref["rec"].sum_sq) <= 1e-12 * ref["rec"].sum_sq
        assert res[k].within_tolerance == ref["rec"].within_tolerance
    res2 = b.run()                                      # the graph replays to the same bits
    assert [r.sum_sq for r in res2] == [r.sum_sq for r in res]
    info = b.info()
    assert info["pixel_samples"] == sum(w * h * spp for w, h, spp, _, _ in specs)


def test_big_scene_raster_matches_oracle(rn, oracle, big_scene):
    import scene as scenes
    w, h, _, cam = scenes.orbit_views(1, 64)[5]
    w, h = 320, 240
    g, depth = rn.rasterize(big_scene.tris, big_scene.normals, cam, w, h, want_depth=True)
    rd, rp, rnm, rm = oracle.rasterize(big_scene.tris, big_scene.normals, cam, w, h)
    assert np.array_equal(g.mask, rm) and np.array_equal(depth, rd)
    assert np.array_equal(g.position, rp) and np.array_equal(g.normal, rnm)
    assert 0.2 < rm.mean() < 1.0


def test_big_scene_ao_matches_oracle(rn, oracle, big_scene):
    import scene as scenes
    _, _, _, cam = scenes.orbit_views(1, 64)[11]
    w, h = 192, 128
    g = rn.rasterize(big_scene.tris, big_scene.normals, cam, w, h)
    acc = rn.LinearAccel(big_scene.tris)
    ao, sky, sun = rn.compute_rt_visibility(g, acc, 16, 1.0, big_scene.to_light)
    rao, rsky, rsun = oracle.trace(g.position, g.normal, g.mask, big_scene.tris, 16, 1.0,
                                   to_light=big_scene.to_light, threads=THREADS)
    assert np.array_equal(ao, rao), int((ao != rao).sum())
    assert np.array_equal(sky, rsky), int((sky != rsky).sum())
    assert np.array_equal(sun, rsun), int((sun != rsun).sum())
    cov = g.mask != 0
    assert 0.0 < ao[cov].mean() < 1.0


def test_batched_views_on_big_scene(rn, oracle, big_scene):
    """The batched-views config at a reduced scale: 8 orbit views (resolutions /8, spp as drawn),
    batch == single frames, and every 16th row of the first view == the oracle."""
    import torch
    import scene as scenes
    acc = rn.LinearAccel(torch.from_numpy(big_scene.tris).cuda())
    views = []
    for w, h, spp, cam in scenes.orbit_views(1, 64)[:8]:
        views.append(dict(g=_gbuf(rn, big_scene, cam, w // 8, h // 8), spp=spp, radius=1.0, cam=cam))
    b = rn.Batch(acc, views, ss_samples=24, tolerance=0.12)
    res = b.run()
    for k, v in enumerate(views):
        ref = rn.ao_frame(v["g"], acc, v["spp"], 1.0, 24, 0.12)
        torch.cuda.synchronize()
        assert torch.equal(b.outputs[k]["ao"], ref["ao"]) and torch.equal(b.outputs[k]["ss"], ref["ss"])
        assert abs(res[k].sum_sq - ref["rec"].sum_sq) <= 1e-12 * ref["rec"].sum_sq
    v = views[0]
    g = v["g"]
    pos, nrm, mask = g.position.cpu().numpy(), g.normal.cpu().numpy(), g.mask.cpu().numpy()
    h, w = mask.shape
    import ctypes as C
    ao = np.zeros((h, w), np.float32)
    L = oracle.lib()
    hnd = L.rno_accel_build(np.ascontiguousarray(big_scene.tris), len(big_scene.tris))
    try:
        L.rno_trace(w, h, pos, nrm, mask, hnd, big_scene.tris, len(big_scene.tris), v["spp"], 1.0, None, 0, ao,
                    None, None, THREADS, 0, 16)
    finally:
        L.rno_accel_free(hnd)
    rows = np.arange(0, h, 16)
    assert np.array_equal(b.outputs[0]["ao"].cpu().numpy()[rows], ao[rows])


def test_big_scene_ao_only_walks_match_oracle(rn, oracle, big_scene):
    """AO-only walks start from each warp's frontier; the answer must still be the oracle's."""
    import scene as scenes
    for k, radius in ((3, 1.0), (40, 2.5)):
        _, _, _, cam = scenes.orbit_views(1, 64)[k]
        w, h = 160, 120
        g = rn.rasterize(big_scene.tris, big_scene.normals, cam, w, h)
        acc = rn.LinearAccel(big_scene.tris)
        ao = rn.compute_rtao(g, acc, 32, radius)
        ref = oracle.trace(g.position, g.normal, g.mask, big_scene.tris, 32, radius, threads=THREADS)
        assert np.array_equal(ao, ref), (k, int((ao != ref).sum()))
