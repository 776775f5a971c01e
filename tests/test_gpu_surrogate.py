"""The surrogate frame (rn_surrogate_ao) against its restatement in PyTorch ops over the
library's own passes, and the trained network's gain over the method without it.

Gain (ablation): on held-out scenes of the training distribution at 1920 x 1080, against
the 1024-spp trace, the surrogate (4-spp trace + U-Net + fallback) must beat the 4-spp
trace it starts from, a 5 x 5 coverage-aware box filter of that trace (the same input
without the learned part), and plain tracing at 64 spp."""
import os

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
WEIGHTS = os.path.join(ROOT, "raw-native_gb300", "weights", "surrogate_bf16.npz")


def _frame(rn, seed, w, h, boxes=200, spheres=50):
    import torch
    import scene as scenes
    import surrogate as S
    sc = scenes.build_synthetic_scene(seed, boxes, spheres)
    tris, nrms = torch.from_numpy(sc.tris).cuda(), torch.from_numpy(sc.normals).cuda()
    acc = rn.LinearAccel(tris)
    g, depth = rn.rasterize(tris, nrms, S.camera_for(seed), w, h, want_depth=True)
    return g, depth, acc


def _net(rn, h, w):
    import surrogate as S
    net = rn.UNet(1, *S.padded_shape(h, w), inference=True)
    S.load_weights(net, WEIGHTS)
    return net


def test_surrogate_frame_matches_its_restatement(rn):
    import torch
    import surrogate as S
    w, h = 384, 224
    g, depth, acc = _frame(rn, 900123, w, h, 600, 150)
    net = _net(rn, h, w)
    ao, stats, parts = rn.surrogate_ao(net, g, depth, acc, 64, 1.0, 3.0, want_parts=True)
    m = g.mask.bool()
    # the 4-spp input is the library's own 4-spp trace
    ao4 = rn.compute_rtao(g, acc, 4, 1.0)
    assert torch.equal(parts["ao4"], ao4)
    # the network on the same features
    pred = S.predict(net, S.features(g, depth, ao4))
    assert (parts["pred"] - pred).abs().max().item() <= 1e-6
    # the band test: the same tiles up to the summation order of near-threshold tiles
    tiles = S.fallback_tiles(parts["pred"], ao4, g.mask, 4, 3.0)
    assert (tiles != parts["tile_flags"].bool()).float().mean().item() <= 0.01
    assert stats["tiles_fallback"] == int(parts["tile_flags"].sum())
    # the composite: traced pixels on flagged tiles (frame coordinates), prediction elsewhere
    fb = S.tiles_to_pixels(parts["tile_flags"].bool(), h, w) & m
    full = rn.compute_rtao(g, acc, 64, 1.0)
    assert torch.equal(ao[fb], full[fb])
    assert torch.equal(ao[m & ~fb], parts["pred"][m & ~fb])
    assert bool((ao[~m] == 1).all())


def test_surrogate_band_extremes(rn):
    import torch
    w, h = 256, 144
    g, depth, acc = _frame(rn, 900124, w, h)
    net = _net(rn, h, w)
    m = g.mask.bool()
    none, st0 = rn.surrogate_ao(net, g, depth, acc, 32, 1.0, 1e9, want_parts=True)[:2]
    assert st0["tiles_fallback"] == 0 and st0["tiles_covered"] > 0
    full = rn.compute_rtao(g, acc, 32, 1.0)
    _, st1, parts = rn.surrogate_ao(net, g, depth, acc, 32, 1.0, 0.0, want_parts=True)
    # k = 0 flags every covered tile whose means differ at all: nearly all of them
    assert st1["tiles_fallback"] >= 0.9 * st1["tiles_covered"]
    with pytest.raises(rn.RnError):
        rn.surrogate_ao(rn.UNet(2, 144, 256, inference=True), g, depth, acc, 32)   # batch 2
    with pytest.raises(rn.RnError):
        rn.surrogate_ao(_net(rn, 128, 128), g, depth, acc, 32)                     # too small


def test_trained_surrogate_gains_over_the_method_without_it(rn):
    import torch
    import torch.nn.functional as F
    import surrogate as S
    w, h = 1920, 1080
    net = _net(rn, h, w)
    rows = []
    for seed in (900000, 900001, 900002):
        g, depth, acc = _frame(rn, seed, w, h)
        m = g.mask.bool()
        truth = rn.compute_rtao(g, acc, 1024, 1.0)
        ao, stats = rn.surrogate_ao(net, g, depth, acc, 256, 1.0, 3.0)
        ao4 = rn.compute_rtao(g, acc, 4, 1.0)
        mf = m.float()[None, None]
        blur = F.avg_pool2d((ao4 * m.float())[None, None], 5, 1, 2) / F.avg_pool2d(mf, 5, 1, 2).clamp(min=1e-6)
        rows.append(dict(sur=S.rmse(ao, truth, g.mask), ao4=S.rmse(ao4, truth, g.mask),
                         blur=S.rmse(blur[0, 0], truth, g.mask), rt64=S.rmse(rn.compute_rtao(g, acc, 64, 1.0), truth, g.mask),
                         fb=stats["fallback_fraction"]))
    for r in rows:
        assert r["sur"] < 0.25 * r["ao4"], r
        assert r["sur"] < 0.6 * r["blur"], r
        assert r["sur"] < r["rt64"], r
        assert r["fb"] < 0.05, r
