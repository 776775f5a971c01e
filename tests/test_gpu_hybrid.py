"""Closest-hit consumers of the AO path's accelerator against the oracle, through the C ABI.

rn_closest is rt::closest (src/renderer/rt_bvh.cpp:125-152): the nearest hit below t_max,
ties to the lowest triangle index. rn_hybrid is the hybrid pass's per-pixel rule
(src/renderer/gpu/rt_hybrid_parity.cpp:38-41, 57-80) over a G-buffer: a sun shadow ray and
a mirror reflection ray per covered pixel. Both use the reference's hit test on the same
operands as the oracle's scans, so the bar is bit-exact: the same triangle, the same t, the
same lit flag.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1


def _soup(seed, n):
    rng = np.random.default_rng(seed)
    c = rng.uniform(-4, 4, (n, 1, 3))
    tris = (c + rng.normal(0, 0.6, (n, 3, 3))).reshape(n, 9).astype(np.float32)
    return tris


def _rays(seed, n, spread=6.0):
    rng = np.random.default_rng(seed)
    o = rng.uniform(-spread, spread, (n, 3))
    d = rng.normal(0, 1, (n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return np.concatenate([o, d], 1).astype(np.float32)


def test_closest_matches_scan_on_a_soup(rn, oracle):
    tris = _soup(1, 3000)
    # exact duplicates at higher indices: equal t, the lower index must win
    tris = np.concatenate([tris, tris[:200]]).astype(np.float32)
    rays = _rays(2, 20000)
    rng = np.random.default_rng(3)
    tmax = np.where(rng.random(len(rays)) < 0.3, rng.uniform(0.5, 4.0, len(rays)), 1e30).astype(np.float32)
    acc = rn.LinearAccel(tris)
    tri, t = rn.closest(acc, rays, tmax)
    rtri, rt = oracle.closest_scan(tris, rays, tmax, threads=THREADS)
    assert np.array_equal(tri, rtri), int((tri != rtri).sum())
    assert np.array_equal(t, rt)
    hits = tri >= 0
    assert 0.2 < hits.mean() < 1.0 and (tri[hits] < 3000).all()
    assert (t[hits] < tmax[hits]).all() and (t[~hits] == -1).all()
    # any hit below t_max is exactly a closest hit below it
    assert np.array_equal(rn.occluded(acc, rays, tmax) != 0, hits)


def test_closest_device_pointers_and_empty_inputs(rn, oracle):
    import torch
    tris = _soup(4, 500)
    rays = _rays(5, 4096)
    tmax = np.full(len(rays), 1e30, np.float32)
    acc = rn.LinearAccel(tris)
    tri, t = rn.closest(acc, rays, tmax)
    dtri, dt = rn.closest(acc, torch.from_numpy(rays).cuda(), torch.from_numpy(tmax).cuda())
    assert np.array_equal(dtri.cpu().numpy(), tri) and np.array_equal(dt.cpu().numpy(), t)
    none = rn.closest(acc, rays[:0], tmax[:0])
    assert none[0].size == 0
    empty = rn.LinearAccel(np.zeros((0, 9), np.float32))
    etri, et = rn.closest(empty, rays, tmax)
    assert (etri == -1).all() and (et == -1).all()


def _hybrid_case(oracle, sc, w, h):
    _, pos, nrm, mask = oracle.rasterize(sc.tris, sc.normals, sc.camera, w, h)
    return pos, nrm, mask, np.asarray(sc.camera[:3], np.float32), sc.to_light


def _check_hybrid(rn, oracle, tris, pos, nrm, mask, eye, sun):
    acc = rn.LinearAccel(tris)
    lit, tri, t = rn.hybrid(rn.GBuffer(pos, nrm, mask), acc, eye, sun)
    rlit, rtri, rt = oracle.hybrid(pos, nrm, mask, tris, eye, sun, threads=THREADS)
    assert np.array_equal(lit, rlit), int((lit != rlit).sum())
    assert np.array_equal(tri, rtri), int((tri != rtri).sum())
    assert np.array_equal(t, rt)
    cov = mask != 0
    assert (lit[~cov] == -1).all() and (tri[~cov] == -1).all()
    return lit, tri, cov


@pytest.mark.parametrize("w,h", [(160, 128), (101, 37)])
def test_hybrid_test_scene_bit_exact(rn, oracle, w, h):
    """160 x 128 and a ragged 101 x 37 (partial 16 x 8 blocks on both edges)."""
    import scene as scenes
    sc = scenes.build_test_scene()
    pos, nrm, mask, eye, sun = _hybrid_case(oracle, sc, w, h)
    lit, tri, cov = _check_hybrid(rn, oracle, sc.tris, pos, nrm, mask, eye, sun)
    # the box shadows part of the plane, and the plane reflects the box
    assert 0.0 < (lit[cov] == 0).mean() < 0.5 and (tri[cov] >= 2).any()


def test_hybrid_synthetic_scene_bit_exact(rn, oracle):
    """A seeded city of boxes and spheres on a 20 x 20 ground grid (about 2,200 triangles),
    320 x 240 from its default view."""
    import scene as scenes
    sc = scenes.build_synthetic_scene(11, 40, 3, grid=20, subdiv=2)
    pos, nrm, mask, eye, sun = _hybrid_case(oracle, sc, 320, 240)
    lit, tri, cov = _check_hybrid(rn, oracle, sc.tris, pos, nrm, mask, eye, sun)
    assert 0.0 < (lit[cov] == 0).mean() < 0.9 and 0.0 < (tri[cov] >= 0).mean()


def test_hybrid_device_pointers_equal_host_path(rn, oracle):
    import torch
    import scene as scenes
    sc = scenes.build_test_scene()
    pos, nrm, mask, eye, sun = _hybrid_case(oracle, sc, 96, 64)
    acc = rn.LinearAccel(sc.tris)
    host = rn.hybrid(rn.GBuffer(pos, nrm, mask), acc, eye, sun)
    g = rn.GBuffer(*(torch.from_numpy(a).cuda() for a in (pos, nrm, mask)))
    dev = rn.hybrid(g, acc, eye, sun)
    for a, b in zip(host, dev):
        assert np.array_equal(a, b.cpu().numpy())
    empty = rn.LinearAccel(np.zeros((0, 9), np.float32))
    lit, tri, _ = rn.hybrid(rn.GBuffer(pos, nrm, mask), empty, eye, sun)
    cov = mask != 0
    assert (lit[cov] == 1).all() and (tri == -1).all()


def test_hybrid_residency_keys_change_no_result(rn, oracle):
    import scene as scenes
    sc = scenes.build_synthetic_scene(12, 30, 2, grid=16, subdiv=2)
    pos, nrm, mask, eye, sun = _hybrid_case(oracle, sc, 128, 96)
    acc = rn.LinearAccel(sc.tris)
    g = rn.GBuffer(pos, nrm, mask)
    saved = rn.tune_get("hybrid_min_blocks")
    try:
        outs = []
        for v in rn.TUNE_KEYS["hybrid_min_blocks"]:
            rn.tune_set("hybrid_min_blocks", v)
            outs.append(rn.hybrid(g, acc, eye, sun))
    finally:
        rn.tune_set("hybrid_min_blocks", saved)
    for o in outs[1:]:
        for a, b in zip(outs[0], o):
            assert np.array_equal(a, b)


def test_closest_ties_on_shared_edges_and_axis_rays(rn, oracle):
    """Rays straight down through the vertices, edges and cells of a triangulated ground grid:
    axis-aligned directions (zero components, infinite inverses) and hits on edges that 2-6
    triangles share at the same t, which the lowest index must win; t_max at or below the hit
    distance leaves no hit."""
    import scene as scenes
    g = scenes.build_synthetic_scene(0, 0, 0, grid=8, half=4.0).tris     # 128 ground triangles, y = 0
    xs = np.linspace(-4.0, 4.0, 17, dtype=np.float32)                    # vertices and edge midpoints
    ox, oz = np.meshgrid(xs, xs, indexing="ij")
    n = ox.size
    down = np.stack([ox.ravel(), np.full(n, 3.0, np.float32), oz.ravel(), np.zeros(n), -np.ones(n), np.zeros(n)], 1)
    slant = down.copy()
    slant[:, 3:] = np.array([0.6, -0.8, 0.0], np.float32)                # exact unit vector, y component -0.8
    slant[:, 0] -= np.float32(2.25)                                      # 3 / 0.8 * 0.6: lands on the same points
    rays = np.concatenate([down, slant]).astype(np.float32)
    for tmax in (np.full(len(rays), 1e30, np.float32), np.full(len(rays), 3.0, np.float32),
                 np.zeros(len(rays), np.float32)):
        acc = rn.LinearAccel(g)
        tri, t = rn.closest(acc, rays, tmax)
        rtri, rt = oracle.closest_scan(g, rays, tmax, threads=THREADS)
        assert np.array_equal(tri, rtri), int((tri != rtri).sum())
        assert np.array_equal(t, rt)
    tri, t = rn.closest(rn.LinearAccel(g), rays, np.full(len(rays), 1e30, np.float32))
    inside = (np.abs(rays[:, 0]) < 4) & (np.abs(rays[:, 2]) < 4)
    assert (tri[:n][inside[:n]] >= 0).all() and (t[:n][inside[:n]] == 3.0).all()


class _XorShift:
    """tests/test_bvh.cpp's generator: xorshift64 (13, 7, 17), 53-bit doubles rounded to float."""

    def __init__(self, seed):
        self.s = seed

    def next(self):
        s = self.s
        s ^= (s << 13) & 0xFFFFFFFFFFFFFFFF
        s ^= s >> 7
        s ^= (s << 17) & 0xFFFFFFFFFFFFFFFF
        self.s = s
        return np.float32((s >> 11) * (1.0 / 9007199254740992.0))

    def vec(self, lo, hi):
        lo, span = np.float32(lo), np.float32(hi) - np.float32(lo)
        return np.array([lo + span * self.next() for _ in range(3)], np.float32)


def _seeded_rays(count, seed):
    """tests/test_bvh.cpp:31-35: origins in [-12, 12)^3, normalized directions from [-1, 1)^3,
    t_max 4 u on every third ray and 1e30 on the rest."""
    r = _XorShift(seed)
    rays = np.empty((count, 6), np.float32)
    tmax = np.empty(count, np.float32)
    for k in range(count):
        o = r.vec(-12.0, 12.0)
        d = r.vec(-1.0, 1.0)
        l = np.sqrt((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2], dtype=np.float32)
        d = d * (np.float32(1.0) / l) if l > 0 else d
        rays[k, :3], rays[k, 3:] = o, d
        tmax[k] = np.float32(1e30) if k % 3 else np.float32(4.0) * r.next()
    return rays, tmax


def test_closest_and_occluded_equal_the_scan_on_seeded_rays(rn, oracle):
    """The reference's BVH check (tests/test_bvh.cpp): 10,000 seeded rays through a
    20,000-triangle soup and 100,000 through the built-in scene; the nearest triangle, its t
    and the occlusion answer all equal the scan's."""
    import scene as scenes
    r = _XorShift(7)
    soup = np.empty((20000, 9), np.float32)
    for i in range(20000):
        c = r.vec(-10.0, 10.0)
        soup[i] = np.concatenate([c + r.vec(-0.6, 0.6), c + r.vec(-0.6, 0.6), c + r.vec(-0.6, 0.6)])
    for tris, count, seed in ((soup, 10000, 11), (scenes.build_test_scene().tris, 100000, 13)):
        rays, tmax = _seeded_rays(count, seed)
        acc = rn.LinearAccel(tris)
        tri, t = rn.closest(acc, rays, tmax)
        rtri, rt = oracle.closest_scan(tris, rays, tmax, threads=THREADS)
        assert np.array_equal(tri, rtri), int((tri != rtri).sum())
        assert np.array_equal(t, rt)
        occ = rn.occluded(acc, rays, tmax)
        assert np.array_equal(occ, oracle.occluded_scan(tris, rays, tmax, threads=THREADS))
        assert 0.01 < (tri >= 0).mean() < 0.95


def test_hybrid_geometric_normals_bit_exact(rn, oracle):
    """Smooth-shaded spheres: the shading normal (the G-buffer's, interpolated) differs from
    the surface triangle's normal, which places the ray origins and decides the facing
    (rt_hybrid_parity.cpp:35-41). The plane of triangle normals comes from the rasterizer's
    per-pixel triangle."""
    import torch
    import scene as scenes
    sc = scenes.build_synthetic_scene(13, 20, 12, grid=12, half=12.0, subdiv=2)
    cam = (14.0, 6.0, 10.0, 0.0, 1.0, 0.0, 0.0, 1.0, 0.0, 0.9)
    _, pos, nrm, mask, ptri = oracle.rasterize_ex(sc.tris, sc.normals, cam, 256, 192)
    t9 = sc.tris[np.maximum(ptri, 0)].reshape(192, 256, 3, 3)
    ng = np.cross(t9[..., 1, :] - t9[..., 0, :], t9[..., 2, :] - t9[..., 0, :]).astype(np.float32)
    ng = (ng * (np.float32(1.0) / np.sqrt((ng * ng).sum(-1, keepdims=True, dtype=np.float32)))).astype(np.float32)
    ng[mask == 0] = 0.0
    eye = np.asarray(cam[:3], np.float32)
    acc = rn.LinearAccel(sc.tris)
    got = rn.hybrid(rn.GBuffer(pos, nrm, mask), acc, eye, sc.to_light, geo_normal=ng)
    ref = oracle.hybrid(pos, nrm, mask, sc.tris, eye, sc.to_light, geo_normal=ng, threads=THREADS)
    for a, b in zip(got, ref):
        assert np.array_equal(a, b), int((a != b).sum())
    # the geometric normals change the answer somewhere: they are not the shading normals
    alt = oracle.hybrid(pos, nrm, mask, sc.tris, eye, sc.to_light, threads=THREADS)
    assert any(not np.array_equal(a, b) for a, b in zip(ref, alt))
    dev = rn.hybrid(rn.GBuffer(*(torch.from_numpy(a).cuda() for a in (pos, nrm, mask))), acc, eye, sc.to_light,
                    geo_normal=torch.from_numpy(ng).cuda())
    for a, b in zip(got, dev):
        assert np.array_equal(a, b.cpu().numpy())
