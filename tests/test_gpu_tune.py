"""Launch-shape tuning never changes a result: every value of every key reproduces the
default configuration's traced AO/sky/sun, SSAO and surrogate output bit for bit."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture
def restore_tune(rn):
    saved = rn.tune_all()
    yield
    for k, v in saved.items():
        rn.tune_set(k, v)


def _scene(rn, w, h, n_boxes=300, n_spheres=60):
    import torch
    import scene as scenes
    sc = scenes.build_synthetic_scene(11, n_boxes, n_spheres)
    tris, nrms = torch.from_numpy(sc.tris).cuda(), torch.from_numpy(sc.normals).cuda()
    g = rn.rasterize(tris, nrms, scenes.orbit_views(11, 8)[3][3], w, h)
    return g, rn.LinearAccel(tris), sc.to_light


def test_trace_keys_keep_every_bit(rn, restore_tune):
    g, acc, tl = _scene(rn, 333, 197)
    defaults = {"trace_min_blocks": 3, "trace_packet": 8, "trace_stack": 96, "trace_frontier": 1,
                "trace_frontier_min_spp": 1, "trace_frontier_tail": 0, "trace_pool": 0, "trace_leaf_pass": 1}
    for k, v in defaults.items():
        rn.tune_set(k, v)
    ref_ao = rn.compute_rtao(g, acc, 16, 1.0).clone()
    ref_vis = [t.clone() for t in rn.compute_rt_visibility(g, acc, 16, 1.0, tl)]
    for k in defaults:
        for v in rn.TUNE_KEYS[k]:
            rn.tune_set(k, v)
            assert bool((rn.compute_rtao(g, acc, 16, 1.0) == ref_ao).all()), (k, v)
            vis = rn.compute_rt_visibility(g, acc, 16, 1.0, tl)
            assert all(bool((a == b).all()) for a, b in zip(vis, ref_vis)), (k, v)
        rn.tune_set(k, defaults[k])


@pytest.mark.parametrize("spp", [1, 4, 7, 16, 17])
def test_pooled_walks_keep_every_bit(rn, oracle, restore_tune, spp):
    """AO-only walks from one queue per packet (trace_pool) against one pixel per lane, for
    every refill threshold, packet shape and frontier setting, the queue in pixel order or
    sorted by direction octant (trace_pool_sort), on a ragged frame; and against the oracle."""
    import numpy as np
    g, acc, _ = _scene(rn, 211, 101)
    rn.tune_set("trace_pool", 0)
    ref = rn.compute_rtao(g, acc, spp, 1.0).clone()
    for pool in (16, 24, 32):
        for packet in (4, 8, 16):
            for frontier in (0, 1):
                for sort in (0, 1):
                    rn.tune_set("trace_pool", pool)
                    rn.tune_set("trace_pool_sort", sort)
                    rn.tune_set("trace_packet", packet)
                    rn.tune_set("trace_frontier", frontier)
                    rn.tune_set("trace_frontier_min_spp", 1)
                    got = rn.compute_rtao(g, acc, spp, 1.0)
                    assert bool((got == ref).all()), (pool, sort, packet, frontier, int((got != ref).sum().item()))
    import scene as scenes
    sc = scenes.build_synthetic_scene(11, 300, 60)
    want = oracle.trace(g.position.cpu().numpy(), g.normal.cpu().numpy(), g.mask.cpu().numpy(), sc.tris, spp, 1.0,
                        threads=8)
    assert np.array_equal(ref.cpu().numpy(), want)


def test_ssao_tile_keeps_every_bit(rn, restore_tune):
    import torch
    g, acc, _ = _scene(rn, 333, 197)
    rn.tune_set("ssao_tile_h", 8)
    ref = rn.compute_ssao(g, 24, 1.0).clone()
    truth = rn.compute_rtao(g, acc, 16, 1.0)
    ref_rec = rn.reconcile(ref, truth, g.mask)
    for v in rn.TUNE_KEYS["ssao_tile_h"]:
        rn.tune_set("ssao_tile_h", v)
        assert bool((rn.compute_ssao(g, 24, 1.0) == ref).all()), v
        out = rn.ao_frame(g, acc, 16, 1.0, 24, 0.12)
        assert bool((out["ss"] == ref).all()), v
        assert out["rec"].pixels == ref_rec.pixels and out["rec"].max_error == ref_rec.max_error
        assert abs(out["rec"].sum_sq - ref_rec.sum_sq) <= 1e-10 * ref_rec.sum_sq


def test_conv_tile_keeps_every_bit(rn, restore_tune):
    """The GEMM tile width, the row ring and two tiles per weight box change no output bit,
    on a network whose levels take every convolution kernel (128-pixel rows at levels 0-1)."""
    import torch
    for H, W in ((64, 64), (128, 256)):
        net = rn.UNet(2, H, W, seed=4, inference=True)
        x = torch.rand(2, H, W, 5, device="cuda", generator=torch.Generator(device="cuda").manual_seed(1))
        rn.tune_set("conv_bn_max", 256)
        rn.tune_set("conv_pair", 0)
        ref = net.forward(x).clone()
        for k in ("conv_bn_max", "conv_pair", "conv_halo"):
            for v in rn.TUNE_KEYS[k]:
                rn.tune_set(k, v)
                assert bool((net.forward(x) == ref).all()), (H, W, k, v)
            rn.tune_set(k, {"conv_bn_max": 256, "conv_pair": 0, "conv_halo": 1}[k])


def test_conv_tmem_a_keeps_every_bit(rn, restore_tune):
    """The row-ring convolutions with their A operands kept in TMEM (conv_tmem_a) give the
    same network output bit for bit: the same MMAs in the same order on the same operands,
    only read from TMEM. Frames of several heights (items of 1 to 16 rows, so the TMEM ring
    crosses item boundaries), batch 2. A training step's loss and weight gradients are sums
    by float atomics (split-K weight gradients, per-block loss partials), whose order differs
    from run to run with either setting: they agree within float32 summation noise."""
    import torch
    g = torch.Generator(device="cuda").manual_seed(3)
    for H, W in ((64, 128), (144, 256), (1088, 1920)):
        net = rn.UNet(1 if H > 200 else 2, H, W, seed=5, inference=True)
        x = torch.rand(net.shape[0], H, W, 5, device="cuda", generator=g)
        rn.tune_set("conv_tmem_a", 0)
        ref = net.forward(x).clone()
        rn.tune_set("conv_tmem_a", 1)
        got = net.forward(x)
        assert bool((got == ref).all()), (H, W, int((got != ref).sum().item()))
        net.close()
    trn = rn.UNet(4, 128, 128, seed=6)
    xb = torch.rand(4, 128, 128, 5, device="cuda", generator=g)
    yb = torch.rand(4, 128, 128, device="cuda", generator=g)
    p0 = trn.get_params()
    losses, grads = [], []
    for v in (0, 1):
        rn.tune_set("conv_tmem_a", v)
        trn.set_params(p0)
        losses.append(trn.backward(xb, yb))
        grads.append(trn.get_grads().copy())
    import numpy as np
    assert abs(losses[0] - losses[1]) <= 1e-5 * abs(losses[0])
    scale = float(np.abs(grads[0]).max())
    assert np.allclose(grads[0], grads[1], rtol=1e-3, atol=1e-5 * scale)


def test_conv_fan_keeps_every_bit(rn, restore_tune):
    """The row-ring convolutions in fan-out form (conv_fan: each input row's MMAs add to the
    three output rows that read it, N = 3 x 32 or 3 x 64) give the same network output bit for
    bit: every output row still starts with its first K16 step and adds the other steps in
    the same tap and channel order. Frames of several heights (items of 1 to 16 rows, so the
    accumulator ring wraps inside MMAs and crosses item boundaries), batch 2; also with every
    fan-out layer in 32-channel slices (conv_fan_bn 32)."""
    import torch
    g = torch.Generator(device="cuda").manual_seed(4)
    for H, W in ((64, 128), (144, 256), (1088, 1920)):
        net = rn.UNet(1 if H > 200 else 2, H, W, seed=7, inference=True)
        x = torch.rand(net.shape[0], H, W, 5, device="cuda", generator=g)
        rn.tune_set("conv_fan", 0)
        ref = net.forward(x).clone()
        rn.tune_set("conv_fan", 1)
        for bn in (64, 32):
            rn.tune_set("conv_fan_bn", bn)
            got = net.forward(x)
            assert bool((got == ref).all()), (H, W, bn, int((got != ref).sum().item()))
        rn.tune_set("conv_fan_bn", 64)
        net.close()


@pytest.mark.parametrize("sky", [False, True])
def test_host_frame_keeps_every_bit(rn, restore_tune, sky):
    """rn_ao_frame with pinned host buffers runs without copies: the traversal reads the
    G-buffer from mapped host memory, mirrors it into HBM for the SSAO, and every pass writes
    its image straight into host memory. Every image equals the device-pointer frame's bit for
    bit, with the direct path and with the staged one, on a frame size that leaves ragged
    packets and blocks, twice in a row (the mirror is reused); the reconcile agrees to the FP64
    sum's last bits."""
    import numpy as np
    import torch
    g, acc, tl = _scene(rn, 641, 487)
    to_light = tl if sky else None
    ref = rn.ao_frame(g, acc, 8, 1.0, 24, 0.12, to_light=to_light)
    keys = ("ao", "ss", "err") + (("sky", "sun") if sky else ())
    hg = rn.GBuffer(g.position.cpu().pin_memory().numpy(), g.normal.cpu().pin_memory().numpy(),
                    g.mask.cpu().pin_memory().numpy())
    for direct in rn.TUNE_KEYS["frame_direct"]:
        rn.tune_set("frame_direct", direct)
        for rep in range(2):
            outs = {k: torch.full((487, 641), -7.0).pin_memory().numpy() for k in keys}
            got = rn.ao_frame(hg, acc, 8, 1.0, 24, 0.12, to_light=to_light, outputs=outs)
            for k in keys:
                assert np.array_equal(got[k], ref[k].cpu().numpy()), (direct, rep, k)
            r, q = got["rec"], ref["rec"]
            assert r.pixels == q.pixels and r.max_error == q.max_error, direct
            assert abs(r.sum_sq - q.sum_sq) <= 1e-12 * q.sum_sq, direct
            assert r.rmse == pytest.approx(q.rmse, rel=1e-6) and r.within_tolerance == q.within_tolerance
    # one pageable output (the error map the wrapper allocates) sends the frame down the staged path
    rn.tune_set("frame_direct", 1)
    outs = {k: torch.zeros(487, 641).pin_memory().numpy() for k in keys}
    outs["err"] = None
    got = rn.ao_frame(hg, acc, 8, 1.0, 24, 0.12, to_light=to_light, outputs=outs)
    assert np.array_equal(got["ao"], ref["ao"].cpu().numpy())
    # pageable host buffers take the staged path: the same images
    pg = rn.GBuffer(g.position.cpu().numpy(), g.normal.cpu().numpy(), g.mask.cpu().numpy())
    got = rn.ao_frame(pg, acc, 8, 1.0, 24, 0.12, to_light=to_light)
    for k in keys:
        assert np.array_equal(got[k], ref[k].cpu().numpy()), ("pageable", k)


def test_accel_shape_keeps_every_bit(rn, restore_tune):
    """The traversal accelerator's PLOC radius and leaf size (accel_radius, accel_leaf) change
    the tree, never a traced pixel: the BVH only prunes."""
    import torch
    import scene as scenes
    sc = scenes.build_synthetic_scene(11, 300, 60)
    tris, nrms = torch.from_numpy(sc.tris).cuda(), torch.from_numpy(sc.normals).cuda()
    g = rn.rasterize(tris, nrms, scenes.orbit_views(11, 8)[3][3], 333, 197)
    rn.tune_set("accel_radius", 16)
    rn.tune_set("accel_leaf", 4)
    acc = rn.LinearAccel(tris)
    ref_ao = rn.compute_rtao(g, acc, 16, 1.0).clone()
    ref_vis = [t.clone() for t in rn.compute_rt_visibility(g, acc, 8, 1.0, sc.to_light)]
    for radius, leaf in ((8, 4), (32, 4), (64, 4), (16, 1), (16, 2), (16, 8), (64, 8)):
        rn.tune_set("accel_radius", radius)
        rn.tune_set("accel_leaf", leaf)
        a = rn.LinearAccel(tris)
        assert bool((rn.compute_rtao(g, a, 16, 1.0) == ref_ao).all()), (radius, leaf)
        vis = rn.compute_rt_visibility(g, a, 8, 1.0, sc.to_light)
        assert all(bool((x == y).all()) for x, y in zip(vis, ref_vis)), (radius, leaf)


@pytest.mark.parametrize("leaf", [1, 4, 8])
def test_collapse_block_keeps_every_bit(rn, restore_tune, leaf):
    """The 4-wide collapse in one block (collapse_block) against a launch per level: the same
    node count, leaf triangles and depth, and the same traced frame (AO, sky, sun)."""
    import torch
    import scene as scenes
    sc = scenes.build_synthetic_scene(11, 300, 60)
    tris, nrms = torch.from_numpy(sc.tris).cuda(), torch.from_numpy(sc.normals).cuda()
    g = rn.rasterize(tris, nrms, scenes.orbit_views(11, 8)[3][3], 333, 197)
    rn.tune_set("accel_leaf", leaf)
    rn.tune_set("collapse_block", 0)
    acc = rn.LinearAccel(tris)
    info = acc.info()
    ref = [t.clone() for t in rn.compute_rt_visibility(g, acc, 8, 1.0, sc.to_light)]
    ref_ao = rn.compute_rtao(g, acc, 16, 1.0).clone()
    for v in rn.TUNE_KEYS["collapse_block"][1:]:
        rn.tune_set("collapse_block", v)
        a = rn.LinearAccel(tris)
        assert a.info() == info, (v, a.info(), info)
        assert bool((rn.compute_rtao(g, a, 16, 1.0) == ref_ao).all()), v
        vis = rn.compute_rt_visibility(g, a, 8, 1.0, sc.to_light)
        assert all(bool((x == y).all()) for x, y in zip(vis, ref)), v
    # the reference's 20,000-triangle check soup, one leaf triangle per slot
    soup = torch.from_numpy(scenes.soup(20000, 7)).cuda()
    rn.tune_set("collapse_block", 0)
    i0 = rn.LinearAccel(soup).info()
    rn.tune_set("collapse_block", 65536)
    assert rn.LinearAccel(soup).info() == i0


def test_small_scene_leaf_keeps_every_bit(rn, restore_tune):
    """Scenes under 65,536 triangles take accel_leaf_small: the built-in scene's frame is the
    same for every leaf size."""
    import torch
    import scene as scenes
    sc = scenes.build_test_scene()
    tris, nrms = torch.from_numpy(sc.tris).cuda(), torch.from_numpy(sc.normals).cuda()
    g = rn.rasterize(tris, nrms, sc.camera, 320, 240)
    ref = None
    for leaf in rn.TUNE_KEYS["accel_leaf_small"]:
        rn.tune_set("accel_leaf_small", leaf)
        acc = rn.LinearAccel(tris)
        out = [t.clone() for t in rn.compute_rt_visibility(g, acc, 32, 2.0, sc.to_light)]
        if ref is None:
            ref = out
        assert all(bool((a == b).all()) for a, b in zip(out, ref)), leaf
