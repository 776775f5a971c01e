"""The large 4K head-to-head's scene at full size: the seeded 7.88M-triangle scene (the
batched-views scene generator with 10,000 boxes and 6,000 subdivision-3 icospheres), 3840 x 2160 orbit
views, AO radius 1, the oracle's SAH BVH (the reference's `trace`, src/renderer/ray_ao.cpp:20-63,
whose any-hit answer is the triangle scan's).

- The GPU G-buffer equals the oracle's rasterizer (src/renderer/raster.cpp:92-126) on every
  row, mask bit for bit (pixel count included), position and normal bit for bit.
- The GPU trace equals the oracle bit for bit on every 97th row at 64 spp (the CPU baseline's
  spp), at 4 spp (the surrogate's input, where no per-warp frontier is built) and on every
  389th row at 1024 spp (the head-to-head's truth).
- Size-independent properties of the whole frame: AO is k / spp exactly, 1 off the mask.
"""
import ctypes as C
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
THREADS = os.cpu_count() or 1
W, H, R = 3840, 2160, 1.0


@pytest.fixture(scope="module")
def large(oracle):
    import torch
    import scene as scenes
    sc = scenes.build_synthetic_scene(5, 10000, 6000)
    assert len(sc.tris) == 7880000
    L = oracle.lib()
    hnd = L.rno_accel_build(np.ascontiguousarray(sc.tris), len(sc.tris))
    tris = torch.from_numpy(sc.tris).cuda()
    nrms = torch.from_numpy(sc.normals).cuda()
    yield dict(sc=sc, L=L, hnd=hnd, tris=tris, nrms=nrms)
    L.rno_accel_free(hnd)


def _oracle_rows(large, g, spp, row0, stride):
    pos = np.ascontiguousarray(g.position.cpu().numpy())
    nrm = np.ascontiguousarray(g.normal.cpu().numpy())
    mask = np.ascontiguousarray(g.mask.cpu().numpy())
    ao = np.zeros((H, W), np.float32)
    sc = large["sc"]
    large["L"].rno_trace(W, H, pos, nrm, mask, large["hnd"], sc.tris, len(sc.tris), spp, R, None, 0, ao, None, None,
                         THREADS, row0, stride)
    return ao, mask


@pytest.mark.parametrize("view", [0, 9])
def test_large_view_gbuffer_matches_oracle(rn, oracle, large, view):
    import scene as scenes
    cam = scenes.orbit_views(5, 16)[view][3]
    g, depth = rn.rasterize(large["tris"], large["nrms"], cam, W, H, want_depth=True)
    rd, rp, rnm, rm = oracle.rasterize(large["sc"].tris, large["sc"].normals, cam, W, H)
    mask = g.mask.cpu().numpy()
    assert int(mask.sum()) == int(rm.sum()) and np.array_equal(mask, rm)
    assert np.array_equal(g.position.cpu().numpy(), rp) and np.array_equal(g.normal.cpu().numpy(), rnm)
    assert np.array_equal(depth.cpu().numpy(), rd)
    assert 0.3 < rm.mean() < 1.0


@pytest.mark.parametrize("view,spp,row0,stride", [(0, 64, 5, 97), (9, 64, 41, 97), (0, 4, 13, 97), (9, 1024, 7, 389)])
def test_large_view_trace_matches_oracle_on_strided_rows(rn, large, view, spp, row0, stride):
    import scene as scenes
    cam = scenes.orbit_views(5, 16)[view][3]
    g = rn.rasterize(large["tris"], large["nrms"], cam, W, H)
    acc = rn.LinearAccel(large["tris"])
    ao = rn.compute_rtao(g, acc, spp, R).cpu().numpy()
    ref, mask = _oracle_rows(large, g, spp, row0, stride)
    rows = np.arange(row0, H, stride)
    diff = int((ao[rows] != ref[rows]).sum())
    assert diff == 0, "%d of %d pixels differ from the oracle" % (diff, rows.size * W)
    cov = mask != 0
    assert (ao[~cov] == 1).all()
    q = ao[cov] * spp
    assert np.array_equal(q, np.round(q))                   # k / spp exactly
    assert 0.0 < float(ao[cov].mean()) < 1.0
