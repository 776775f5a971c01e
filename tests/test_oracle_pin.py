"""The oracle is pinned before it is trusted: its C restatement must reproduce the
reference's committed SHA-256 goldens (tests/golden/identity.json, taken from the
reference's evidence/identity-golden.json) byte for byte, the reference's exact reconcile
numbers, and the PLOC tree hashes of the reference's GPU evidence. Where the reference's
own sources were compiled here (oracle/_ref), the restatement is also compared with them.

The goldens were made on x86-64 with glibc's libm; a host whose libm rounds cosf, sinf or
tanf differently reproduces the algorithm but not those bytes, and says so by skipping.
"""
import json
import os
import platform

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
IDENT = json.load(open(os.path.join(HERE, "golden", "identity.json")))
PLOC = json.load(open(os.path.join(HERE, "golden", "ploc.json")))
X86 = platform.machine() in ("x86_64", "AMD64")


def _digests(O, r, w, h):
    return {"ao_rt.pfm": O.sha256(O.pfm1_bytes(r["ao"])), "ao_ss.pfm": O.sha256(O.pfm1_bytes(r["ss"])),
            "mask.pgm": O.sha256(O.mask_pgm_bytes(r["mask"])), "ao_error.pgm": O.sha256(O.pgm_bytes(r["err"]))}


@pytest.mark.parametrize("case", sorted(IDENT["cases"]))
def test_oracle_reproduces_reference_goldens(oracle, case):
    c = IDENT["cases"][case]
    r = oracle.render_default(c["width"], c["height"], c["camera"], threads=os.cpu_count() or 1)
    got = _digests(oracle, r, c["width"], c["height"])
    if got != c["files"] and not X86:
        pytest.skip("host libm differs from the x86-64 golden host (%s)" % platform.machine())
    assert got == c["files"]
    assert oracle.sha256(oracle.pfm1_bytes(r["sky"])) == c["sky_sha256"]
    assert oracle.sha256(oracle.pfm1_bytes(r["sun"])) == c["sun_sha256"]
    st = r["stats"]
    assert st["pixels"] == c["exact"]["pixels"]
    assert np.float32(st["rmse"]) == np.float32(c["exact"]["rmse"])
    assert np.float32(st["maxError"]) == np.float32(c["exact"]["maxError"])
    assert st["within"] == c["exact"]["within"]


def test_default_certificate_numbers(oracle):
    # docs/examples/default-certificate.json: pixels 151984, rmse 0.134912357, maxError 0.640625
    c = IDENT["cases"]["default-512"]["exact"]
    assert c["pixels"] == 151984 and "%.9g" % c["rmse"] == "0.134912357" and c["maxError"] == 0.640625
    assert not c["within"]


def test_ploc_soup_tree_hash(oracle):
    s = PLOC["scenes"]["soup"]
    tris = oracle.soup(s["count"], s["seed"])
    nodes, root, rounds = oracle.ploc(tris)
    assert oracle.tree_hash(nodes) == s["tree_hash"]
    assert rounds == s["rounds"]
    assert root == 2 * s["count"] - 2


def test_ploc_test_scene_tree_hash(oracle):
    s = PLOC["scenes"]["test_scene"]
    tris, _, _ = oracle.test_scene()
    nodes, root, rounds = oracle.ploc(tris)
    assert (oracle.tree_hash(nodes), root, rounds) == (s["tree_hash"], s["root"], s["rounds"])


def test_ploc_radius_control_changes_tree(oracle):
    # the reference's false-success control: radius 8 must give another tree
    tris = oracle.soup(2000, 3)
    assert oracle.tree_hash(oracle.ploc(tris, 16)[0]) != oracle.tree_hash(oracle.ploc(tris, 8)[0])


def test_reconcile_two_pixels(oracle):
    # tests/test_reconcile.cpp:4-19
    a = np.array([[0.5, 0.8]], np.float32)
    b = np.array([[0.5, 0.4]], np.float32)
    m = np.ones((1, 2), np.uint8)
    err, st = oracle.reconcile(a, b, m, 0.1)
    assert abs(err[0, 0]) < 1e-6 and abs(err[0, 1] - 0.4) < 1e-6
    assert abs(st["maxError"] - 0.4) < 1e-6 and st["pixels"] == 2 and not st["within"]
    _, st2 = oracle.reconcile(a, a, m, 0.1)
    assert st2["rmse"] == 0.0 and st2["within"]


def test_bvh_equals_scan_on_random_rays(oracle):
    # tests/test_bvh.cpp: seeded rays, the BVH's any-hit answer equals the scan's
    tris = oracle.soup(3000, 11)
    rng = np.random.default_rng(5)
    import ctypes as C
    L = oracle.lib()
    h = L.rno_accel_build(np.ascontiguousarray(tris), len(tris))
    try:
        bad = 0
        for _ in range(4000):
            o = rng.uniform(-14, 14, 3).astype(np.float32)
            d = rng.normal(size=3).astype(np.float32)
            d /= np.float32(np.linalg.norm(d))
            ray = np.concatenate([o, d]).astype(np.float32)
            for tmax in (np.float32(2.0), np.float32(1e30)):
                bad += L.rno_occluded(h, ray, tmax) != L.rno_occluded_scan(np.ascontiguousarray(tris), len(tris), ray, tmax)
        assert bad == 0
    finally:
        L.rno_accel_free(h)


def test_closest_scan_semantics(oracle):
    """The closest scan: a hit exactly where the any-hit scan finds one, the smallest t of the
    hit test below t_max, and duplicates resolved to the lower index."""
    tris = oracle.soup(800, 3)
    tris = np.concatenate([tris, tris[:100]]).astype(np.float32)
    rng = np.random.default_rng(9)
    o = rng.uniform(-14, 14, (3000, 3))
    d = rng.normal(size=(3000, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.concatenate([o, d], 1).astype(np.float32)
    tmax = np.where(rng.random(3000) < 0.5, 3.0, 1e30).astype(np.float32)
    tri, t = oracle.closest_scan(tris, rays, tmax, threads=4)
    hit = oracle.occluded_scan(tris, rays, tmax, threads=4)
    assert np.array_equal(tri >= 0, hit != 0) and 0 < hit.mean() < 1
    assert (tri < 800).all() and (t[tri >= 0] < tmax[tri >= 0]).all()
    import ctypes as C
    tt = C.c_float()
    for i in np.flatnonzero(tri >= 0)[:200]:
        assert oracle.lib().rno_intersect(rays[i].copy(), tris[tri[i]].copy(), C.byref(tt)) and tt.value == t[i]


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(HERE), "oracle", "_ref", "libref_ao.so")),
                    reason="the reference's own sources are not compiled on this host")
def test_closest_scan_equals_reference_closest(oracle):
    """rt::closest of the reference (its PLOC tree, its ordered walk) against the scan."""
    tris = oracle.soup(2000, 17)
    tris = np.concatenate([tris, tris[:150]]).astype(np.float32)
    rng = np.random.default_rng(4)
    o = rng.uniform(-14, 14, (4000, 3))
    d = rng.normal(size=(4000, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.concatenate([o, d], 1).astype(np.float32)
    tmax = np.where(rng.random(4000) < 0.4, rng.uniform(0.5, 5, 4000), 1e30).astype(np.float32)
    tri, t = oracle.closest_scan(tris, rays, tmax, threads=4)
    rtri = np.zeros(4000, np.int32)
    rt = np.zeros(4000, np.float32)
    oracle.ref().ref_closest(tris, len(tris), rays, tmax, 4000, rtri, rt)
    assert np.array_equal(tri, rtri) and np.array_equal(t, rt)


def test_hybrid_rule_restated_in_python(oracle):
    """The oracle's hybrid pass against a scalar float32 restatement of the reference's
    per-pixel rule (src/renderer/gpu/rt_hybrid_parity.cpp:35-41, 57-80; raw/math/vec.hpp
    normalize and dot) on a small G-buffer, with and without separate geometric normals; the
    ray queries scan with the oracle's pinned triangle test."""
    import ctypes as C
    import scene
    f = np.float32
    sc = scene.build_test_scene()
    _, pos, nrm, mask, ptri = oracle.rasterize_ex(sc.tris, sc.normals, sc.camera, 24, 18)
    tris = sc.tris
    t9 = tris[np.maximum(ptri, 0)].reshape(18, 24, 3, 3)
    geo = np.cross(t9[..., 1, :] - t9[..., 0, :], t9[..., 2, :] - t9[..., 0, :]).astype(f)
    geo = geo * (f(1) / np.sqrt((geo * geo).sum(-1, keepdims=True, dtype=f)))
    geo[mask == 0] = 0
    eye = np.asarray(sc.camera[:3], f)
    tt = C.c_float()

    def dot(a, b):
        return f(f(f(a[0] * b[0]) + f(a[1] * b[1])) + f(a[2] * b[2]))

    def normalize(v):
        l = f(np.sqrt(dot(v, v)))
        return (v * (f(1) / l)).astype(f) if l > 0 else v

    def offset(p, ng, d):
        e = f(f(2e-4) * f(f(1) + max(abs(p[0]), max(abs(p[1]), abs(p[2])))))
        return (p + ng * (e if dot(ng, d) > 0 else -e)).astype(f)

    def scan(o, d):
        ray = np.concatenate([o, d]).astype(f)
        best, best_i = f(1e30), -1
        for i in range(len(tris)):
            if oracle.lib().rno_intersect(ray, np.ascontiguousarray(tris[i]), C.byref(tt)) and f(tt.value) < best:
                best, best_i = f(tt.value), i
        return best_i, best

    l = normalize(np.asarray(sc.to_light, f))
    for g in (None, geo):
        lit, tri, t = oracle.hybrid(pos, nrm, mask, tris, eye, sc.to_light, geo_normal=g)
        for y in range(18):
            for x in range(24):
                if not mask[y, x]:
                    assert lit[y, x] == -1 and tri[y, x] == -1
                    continue
                p, n = pos[y, x], nrm[y, x]
                ng = g[y, x] if g is not None else n
                d = normalize((p - eye).astype(f))
                if dot(ng, d) > 0:
                    ng = (ng * f(-1)).astype(f)
                if dot(n, ng) < 0:
                    n = (n * f(-1)).astype(f)
                assert lit[y, x] == (0.0 if scan(offset(p, ng, l), l)[0] >= 0 else 1.0)
                r = (d - n * f(f(2) * dot(d, n))).astype(f)
                i, best = scan(offset(p, ng, r), r)
                assert tri[y, x] == i and t[y, x] == (best if i >= 0 else -1.0)


def test_thread_count_invariance(oracle):
    # tests/test_verify.cpp:40-43: output identical for any thread count
    a = oracle.render_default(128, 96, threads=1)
    b = oracle.render_default(128, 96, threads=5)
    for k in ("ao", "sky", "sun", "ss", "err"):
        assert np.array_equal(a[k], b[k])


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(HERE), "oracle", "_ref", "libref_ao.so")),
                    reason="the reference's own sources are not compiled on this host")
def test_restatement_equals_reference_build(oracle):
    import ctypes as C
    R = oracle.ref()
    rng = np.random.default_rng(1)
    for cam in ([4, 4, 6, 0, 1, 0, 0, 1, 0, 0.9], [3, 1.2, -4, 0, 0.5, 0, 0, 1, 0, 1.1]):
        w, h = 160, 120
        r = oracle.render_default(w, h, cam, spp=13, radius=1.5, threads=4)
        n = w * h
        b = {k: np.zeros(n * (3 if k in ("pos", "nrm") else 1), np.uint8 if k == "mask" else np.float32)
             for k in ("pos", "nrm", "mask", "ao", "sky", "sun", "ss", "err")}
        st = np.zeros(4, np.float32)
        R.ref_render_default(w, h, np.array(cam, np.float32), 13, 1.5, 24, 0.12, 4, b["pos"], b["nrm"], b["mask"],
                             b["ao"], b["sky"], b["sun"], b["ss"], b["err"], st)
        for k in ("ao", "sky", "sun", "ss", "err"):
            assert np.array_equal(r[k].ravel(), b[k]), k
        assert np.array_equal(r["mask"].ravel(), b["mask"])
    tris = oracle.soup(5000, int(rng.integers(1, 1000)))
    nodes, root, rounds = oracle.ploc(tris)
    out = np.zeros((2 * len(tris) - 1, 9), np.int32)
    rr = C.c_uint32()
    assert R.ref_ploc(tris, len(tris), 16, out, C.byref(rr)) == root
    assert np.array_equal(out, nodes) and rr.value == rounds


def test_product_scene_equals_reference_scene(oracle):
    import scene as scenes
    sc = scenes.build_test_scene()
    tris, nrm, light = oracle.test_scene()
    assert np.array_equal(sc.tris, tris) and np.array_equal(sc.normals, nrm) and np.array_equal(sc.light, light)


def test_product_soup_equals_oracle_soup(oracle):
    import scene
    for n, seed in ((20000, 7), (513, 11)):
        assert np.array_equal(scene.soup(n, seed), oracle.soup(n, seed))


def test_synthetic_scenes_are_seeded_and_sized():
    import scene as scenes
    a = scenes.build_synthetic_scene(1, 2000, 500)
    b = scenes.build_synthetic_scene(1, 2000, 500)
    assert a.tris.shape == (744000, 9) and np.array_equal(a.tris, b.tris)
    assert scenes.build_synthetic_scene(7, 200, 50).tris.shape == (146400, 9)
    assert not np.array_equal(a.tris, scenes.build_synthetic_scene(2, 2000, 500).tris)
    v = scenes.orbit_views(1, 64)
    assert len(v) == 64 and {(w, h) for w, h, _, _ in v} <= set(scenes.RESOLUTIONS)
    assert {s for _, _, s, _ in v} <= set(scenes.SPPS)


def test_gtao_restatement_matches_reference_golden(oracle):
    """raw::post::gtao restated in C (FP64) reproduces the reference build's output bytes on
    the built-in scene from both test cameras (tests/golden/gtao.json)."""
    import json
    gold = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "gtao.json")))["cases"]
    tris, nrm9, _ = oracle.test_scene()
    for name, case in gold.items():
        cam = case["camera"]
        _, pos, nrm, mask = oracle.rasterize(tris, nrm9, cam, case["width"], case["height"])
        vp, vn, vd = oracle.view_gbuffer(pos, nrm, mask, cam)
        a = oracle.gtao(vp, vn, vd, cam[9], case["radius"], case["slices"], case["steps"])
        assert int(mask.sum()) == case["covered"]
        assert oracle.sha256(np.ascontiguousarray(a).tobytes()) == case["sha256"], name


@pytest.mark.parametrize("case", sorted(json.load(open(os.path.join(os.path.dirname(__file__), "golden",
                                                                    "identity.json")))["cases"]))
def test_oracle_frame_reproduces_reference_goldens(oracle, case):
    """The shaded frame (shadeV2 / shadeHDRV2 over the G-buffer's albedo and the traced sky
    and sun) reproduces the reference's committed frame.ppm and frame_hdr.pfm SHA-256."""
    c = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "identity.json")))["cases"][case]
    w, h, cam = c["width"], c["height"], c["camera"]
    if w * h > 600 * 600 and platform.machine() != "x86_64":
        pytest.skip("large case: CPU time")
    tris, nrm9, light = oracle.test_scene()
    alb = oracle.test_scene_albedo()
    _, pos, nrm, mask, tri = oracle.rasterize_ex(tris, nrm9, cam, w, h)
    albedo = np.where(mask[..., None] > 0, alb[np.maximum(tri, 0)], 0).astype(np.float32)
    ao, sky, sun = oracle.trace(pos, nrm, mask, tris, oracle.RT_SAMPLES, oracle.AO_RADIUS, to_light=-light,
                                threads=os.cpu_count() or 1)
    frame, hdr = oracle.shade(nrm, albedo, mask, 2, sky, sun, light, 1.0)
    assert oracle.sha256(oracle.ppm_bytes(frame)) == c["frame_files"]["frame.ppm"]
    assert oracle.sha256(oracle.pfm3_bytes(hdr)) == c["frame_files"]["frame_hdr.pfm"]


def test_motion_restatement_equals_reference_build(oracle):
    if not oracle.ref_available():
        pytest.skip("the reference build (oracle/_ref) is absent")
    tris, nrm9, _ = oracle.test_scene()
    cam = oracle.DEFAULT_CAMERA
    prev = (4.3, 3.8, 5.7, 0.0, 1.0, 0.0, 0.0, 1.0, 0.0, 0.9)
    _, pos, nrm, mask = oracle.rasterize(tris, nrm9, cam, 320, 200)
    vp, pv = oracle.view_proj(cam, 320, 200), oracle.view_proj(prev, 320, 200)
    a, na = oracle.motion(pos, mask, vp, pv)
    b, nb = oracle.motion(pos, mask, vp, pv, use_ref=True)
    assert na == nb == int(mask.sum()) and np.array_equal(a, b) and np.abs(a).max() > 0.01
