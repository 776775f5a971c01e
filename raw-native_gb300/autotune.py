"""Autotuner for the library's launch shapes (rn_tune_* keys): the traversal's packet shape,
stack depth, residency and frontier; the accelerator's shape; the SSAO tile; the convolution
GEMM's tile width; the hybrid pass's residency; the PLOC tail; the path tracer's kernel.

Every candidate is timed with CUDA events on the library's stream over representative
workloads, after a check that it reproduces the default configuration's outputs bit for bit
(the keys change launch shapes, never results). The winners are written as a tune file
("key = value" lines) that rn_tune_load reads; rn_ao.init() loads the package's
tune_sm103.txt when it exists.

  python autotune.py --out tune_sm103.txt [--report report.json] [--quick]
                     [--stages ploc_tail,pt --merge tune_sm103.txt]

--stages runs only the named stages (in the order below); --merge starts from a tune file's
values (applied before the stages run) and writes them back with the stages' picks.

Workloads:
  accel          the traversal accelerator's PLOC radius and leaf size: builds of the
                 7.88M-triangle scene (4K view at 4 and 16 spp) and of the 744k scene
                 (1080p view at 64 spp); the leaf size of scenes under 65,536 triangles
                 on the built-in scene's 4K frame (64 spp, AO + sky + sun)
  trace/model2   the reference's built-in scene and default camera at 3840 x 2160, 64 spp,
                 AO + sky + sun (lighting model 2, radius 2)
  trace/ao       a seeded synthetic scene (2,000 boxes, 500 spheres; 744k triangles),
                 1920 x 1080 orbit view, 64 spp AO only (radius 1)
  trace/large    the 7.88M-triangle scene, one 3840 x 2160 orbit view, 16 spp AO only
                 (the launch shape jointly, then the walk's leaf pass on the same three)
  batch          16 orbit views of the 744k scene in one captured batch (batch_min_blocks)
  ssao           the built-in scene at 4K: SSAO, 24 taps
  conv           the surrogate U-Net: a forward at 1088 x 1920 and a training step on
                 64 crops of 128 x 128 (conv_bn_max, then conv_tmem_a / conv_fan)
  trace/low-spp  the synthetic scene's view at 4, 8, 16 and 32 spp, and a 4K view of the
                 7.88M-triangle scene at 4 and 16 spp (trace_frontier_min_spp)
  trace/tail     the same view at 16, 64 and 256 spp (trace_frontier_tail)
  hybrid         the hybrid pass (shadow + mirror ray per pixel) on the built-in scene and
                 the 744k scene at 4K (hybrid_min_blocks)
  ploc_tail      accelerator builds of the 744k scene, a 1M soup and the 20,000-triangle check
                 soup (the cluster count from which the PLOC rounds run in one block; then the
                 size under which the collapse runs in one block)
  pt             the path tracer on retro_room and iso_street at 1280 x 720, 16 spp (pt_regen,
                 pt_wave, pt_shade_blocks)
The traversal keys are searched jointly (every combination); the others one at a time.
"""
from __future__ import annotations

import argparse
import itertools
import json
import sys
import time

import numpy as np

import rn_ao as rn
import scene as scenes

TRACE_KEYS = ("trace_min_blocks", "trace_packet", "trace_stack", "trace_frontier")


def _time(fn, reps: int) -> float:
    """Mean ms of fn() over reps runs on the current stream, after one warm-up run."""
    import torch
    fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def _apply(cfg: dict) -> None:
    for k, v in cfg.items():
        rn.tune_set(k, v)


def trace_workloads(quick: bool):
    import torch
    out = []
    sc = scenes.build_test_scene()
    tris, nrms = torch.from_numpy(sc.tris).cuda(), torch.from_numpy(sc.normals).cuda()
    w, h = (1920, 1080) if quick else (3840, 2160)
    g = rn.rasterize(tris, nrms, sc.camera, w, h)
    acc = rn.LinearAccel(tris)
    tl = sc.to_light
    out.append(("trace/model2", lambda: rn.compute_rt_visibility(g, acc, 64, 2.0, tl)[0], (g, acc)))
    big = scenes.build_synthetic_scene(7, 500 if quick else 2000, 100 if quick else 500)
    bt, bn = torch.from_numpy(big.tris).cuda(), torch.from_numpy(big.normals).cuda()
    cam = scenes.orbit_views(7, 8)[0][3]
    g2 = rn.rasterize(bt, bn, cam, 1920, 1080)
    acc2 = rn.LinearAccel(bt)
    out.append(("trace/ao", lambda: rn.compute_rtao(g2, acc2, 64, 1.0), (g2, acc2)))
    huge = scenes.build_synthetic_scene(5, 1000 if quick else 10000, 600 if quick else 6000)
    ht, hn = torch.from_numpy(huge.tris).cuda(), torch.from_numpy(huge.normals).cuda()
    g3 = rn.rasterize(ht, hn, scenes.orbit_views(5, 16)[0][3], 1920 if quick else 3840, 1080 if quick else 2160)
    acc3 = rn.LinearAccel(ht)
    out.append(("trace/large", lambda: rn.compute_rtao(g3, acc3, 16, 1.0), (g3, acc3)))
    return out


def tune_trace(quick: bool, reps: int, log):
    defaults = {k: rn.tune_get(k) for k in TRACE_KEYS}
    wls = trace_workloads(quick)
    _apply(defaults)
    ref = [fn().clone() for _, fn, _ in wls]
    rows = []
    for combo in itertools.product(*(rn.TUNE_KEYS[k] for k in TRACE_KEYS)):
        cfg = dict(zip(TRACE_KEYS, combo))
        _apply(cfg)
        same = all(bool((fn() == r).all()) for (_, fn, _), r in zip(wls, ref))
        if not same:
            raise RuntimeError("tuning changed a traced result: %s" % cfg)
        ms = {name: _time(fn, reps) for name, fn, _ in wls}
        rows.append(dict(cfg=cfg, ms=ms))
        log("trace %s  %s" % (cfg, "  ".join("%s %.3f ms" % kv for kv in ms.items())))
    base = next(r for r in rows if r["cfg"] == defaults)["ms"]
    # score: geometric mean of the time ratios to the defaults
    for r in rows:
        r["score"] = float(np.exp(np.mean([np.log(r["ms"][k] / base[k]) for k in base])))
    best = min(rows, key=lambda r: r["score"])
    _apply(best["cfg"])
    return best["cfg"], rows


def tune_walk(quick: bool, reps: int, log):
    """The walk's form on the traversal workloads, after the launch shape: leaf children
    tested inline or in one pass after the slab tests (trace_leaf_pass). Each candidate is
    checked bit for bit; score: geometric mean of the time ratios to the inline form."""
    wls = trace_workloads(quick)
    rn.tune_set("trace_leaf_pass", 0)
    ref = [fn().clone() for _, fn, _ in wls]
    rows = []
    for v in rn.TUNE_KEYS["trace_leaf_pass"]:
        rn.tune_set("trace_leaf_pass", v)
        if not all(bool((fn() == r).all()) for (_, fn, _), r in zip(wls, ref)):
            raise RuntimeError("trace_leaf_pass %d changed a traced result" % v)
        ms = {name: _time(fn, reps) for name, fn, _ in wls}
        rows.append(dict(cfg={"trace_leaf_pass": v}, ms=ms))
        log("trace_leaf_pass %d  %s" % (v, "  ".join("%s %.3f ms" % kv for kv in ms.items())))
    base = rows[0]["ms"]
    for r in rows:
        r["score"] = float(np.exp(np.mean([np.log(r["ms"][k] / base[k]) for k in base])))
    best = min(rows, key=lambda r: r["score"])
    rn.tune_set("trace_leaf_pass", best["cfg"]["trace_leaf_pass"])
    return best["cfg"], rows


def tune_frontier_min_spp(quick: bool, reps: int, log):
    """The spp from which the per-warp frontier pays for its build: AO-only traces of the
    synthetic scene at 4, 8, 16 and 32 spp (1920 x 1080), and of the 7.88M-triangle scene at
    4 and 16 spp (3840 x 2160, radius 1: the surrogate's input trace); the candidate with the
    least total time."""
    import torch
    big = scenes.build_synthetic_scene(7, 500 if quick else 2000, 100 if quick else 500)
    bt, bn = torch.from_numpy(big.tris).cuda(), torch.from_numpy(big.normals).cuda()
    g = rn.rasterize(bt, bn, scenes.orbit_views(7, 8)[0][3], 1920, 1080)
    acc = rn.LinearAccel(bt)
    huge = scenes.build_synthetic_scene(5, 1000 if quick else 10000, 600 if quick else 6000)
    ht, hn = torch.from_numpy(huge.tris).cuda(), torch.from_numpy(huge.normals).cuda()
    gh = rn.rasterize(ht, hn, scenes.orbit_views(5, 16)[0][3], 1920 if quick else 3840, 1080 if quick else 2160)
    acch = rn.LinearAccel(ht)
    rows = []
    for v in rn.TUNE_KEYS["trace_frontier_min_spp"]:
        rn.tune_set("trace_frontier_min_spp", v)
        ms = {"spp%d" % spp: _time(lambda: rn.compute_rtao(g, acc, spp, 1.0), reps) for spp in (4, 8, 16, 32)}
        ms.update({"large_spp%d" % spp: _time(lambda: rn.compute_rtao(gh, acch, spp, 1.0), reps) for spp in (4, 16)})
        rows.append(dict(cfg={"trace_frontier_min_spp": v}, ms=ms, total=sum(ms.values())))
        log("trace_frontier_min_spp %d  %s" % (v, "  ".join("%s %.3f ms" % kv for kv in ms.items())))
    best = min(rows, key=lambda r: r["total"])
    rn.tune_set("trace_frontier_min_spp", best["cfg"]["trace_frontier_min_spp"])
    del acch, gh, ht, hn
    return best["cfg"], rows


def tune_frontier_tail(quick: bool, reps: int, log):
    """Greedy largest-first steps after the level-by-level frontier build (the library takes at
    most spp / 16 of them): AO-only traces of the synthetic scene at 16, 64 and 256 spp, each
    candidate checked bit for bit against no tail; score: geometric mean of the time ratios to
    no tail."""
    import torch
    big = scenes.build_synthetic_scene(7, 500 if quick else 2000, 100 if quick else 500)
    bt, bn = torch.from_numpy(big.tris).cuda(), torch.from_numpy(big.normals).cuda()
    g = rn.rasterize(bt, bn, scenes.orbit_views(7, 8)[0][3], 1920, 1080)
    acc = rn.LinearAccel(bt)
    spps = (16, 64, 256)
    rows, ref = [], None
    for v in rn.TUNE_KEYS["trace_frontier_tail"]:
        rn.tune_set("trace_frontier_tail", v)
        outs = [rn.compute_rtao(g, acc, spp, 1.0).clone() for spp in spps]
        if ref is None:
            ref = outs
        elif not all(bool((a == b).all()) for a, b in zip(outs, ref)):
            raise RuntimeError("trace_frontier_tail %d changed a traced result" % v)
        ms = {"spp%d" % spp: _time(lambda: rn.compute_rtao(g, acc, spp, 1.0), max(2, reps // (1 + spp // 64)))
              for spp in spps}
        rows.append(dict(cfg={"trace_frontier_tail": v}, ms=ms))
        log("trace_frontier_tail %d  %s" % (v, "  ".join("%s %.3f ms" % kv for kv in ms.items())))
    base = rows[0]["ms"]
    for r in rows:
        r["score"] = float(np.exp(np.mean([np.log(r["ms"][k] / base[k]) for k in base])))
    best = min(rows, key=lambda r: r["score"])
    rn.tune_set("trace_frontier_tail", best["cfg"]["trace_frontier_tail"])
    return best["cfg"], rows


def tune_accel(quick: bool, reps: int, log):
    """The traversal accelerator's shape: PLOC search radius x largest leaf, each built for the
    7.88M-triangle scene (4K view, AO radius 1, 4 and 16 spp: the surrogate's input trace and
    a low-spp frame) and the 744k scene (1080p view, 64 spp), every traced image checked bit
    for bit against the default shape; score: geometric mean of the time ratios to the
    default (radius 16, leaves of 4)."""
    import torch
    huge = scenes.build_synthetic_scene(5, 1000 if quick else 10000, 600 if quick else 6000)
    ht, hn = torch.from_numpy(huge.tris).cuda(), torch.from_numpy(huge.normals).cuda()
    gh = rn.rasterize(ht, hn, scenes.orbit_views(5, 16)[0][3], 1920 if quick else 3840, 1080 if quick else 2160)
    big = scenes.build_synthetic_scene(7, 500 if quick else 2000, 100 if quick else 500)
    bt, bn = torch.from_numpy(big.tris).cuda(), torch.from_numpy(big.normals).cuda()
    gb = rn.rasterize(bt, bn, scenes.orbit_views(7, 8)[0][3], 1920, 1080)
    work = (("large_spp4", 0, 4), ("large_spp16", 0, 16), ("ao_spp64", 1, 64))
    rows, ref = [], None
    default = (16, 4)
    combos = [default] + [(r, l) for r in rn.TUNE_KEYS["accel_radius"] for l in rn.TUNE_KEYS["accel_leaf"]
                          if (r, l) != default]
    for radius, leaf in combos:
        rn.tune_set("accel_radius", radius)
        rn.tune_set("accel_leaf", leaf)
        t0 = time.perf_counter()
        accs = (rn.LinearAccel(ht), rn.LinearAccel(bt))
        torch.cuda.synchronize()
        build_s = time.perf_counter() - t0
        geo = (gh, gb)
        outs = [rn.compute_rtao(geo[w], accs[w], spp, 1.0).clone() for _, w, spp in work]
        if ref is None:
            ref = outs
        elif not all(bool((a == b).all()) for a, b in zip(outs, ref)):
            raise RuntimeError("accel_radius %d accel_leaf %d changed a traced result" % (radius, leaf))
        ms = {name: _time(lambda: rn.compute_rtao(geo[w], accs[w], spp, 1.0), reps) for name, w, spp in work}
        rows.append(dict(cfg={"accel_radius": radius, "accel_leaf": leaf}, ms=ms, build_s=build_s))
        log("accel_radius %d accel_leaf %d  build %.2f s  %s" % (radius, leaf, build_s,
                                                                "  ".join("%s %.3f ms" % kv for kv in ms.items())))
        del accs
    base = rows[0]["ms"]
    for r in rows:
        r["score"] = float(np.exp(np.mean([np.log(r["ms"][k] / base[k]) for k in base])))
    best = min(rows, key=lambda r: r["score"])
    for k, v in best["cfg"].items():
        rn.tune_set(k, v)
    # scenes under 65,536 triangles take their own leaf size: the built-in scene's 4K frame
    sc = scenes.build_test_scene()
    st_, sn_ = torch.from_numpy(sc.tris).cuda(), torch.from_numpy(sc.normals).cuda()
    w, h = (1920, 1080) if quick else (3840, 2160)
    gs = rn.rasterize(st_, sn_, sc.camera, w, h)
    ref_small = None
    for leaf in rn.TUNE_KEYS["accel_leaf_small"]:
        rn.tune_set("accel_leaf_small", leaf)
        acc = rn.LinearAccel(st_)
        out = [t.clone() for t in rn.compute_rt_visibility(gs, acc, 64, 2.0, sc.to_light)]
        if ref_small is None:
            ref_small = out
        elif not all(bool((a == b).all()) for a, b in zip(out, ref_small)):
            raise RuntimeError("accel_leaf_small %d changed a traced result" % leaf)
        ms = {"model2": _time(lambda: rn.compute_rt_visibility(gs, acc, 64, 2.0, sc.to_light), reps)}
        rows.append(dict(cfg={"accel_leaf_small": leaf}, ms=ms))
        log("accel_leaf_small %d  model2 %.3f ms" % (leaf, ms["model2"]))
    small = min((r for r in rows if "accel_leaf_small" in r["cfg"]), key=lambda r: r["ms"]["model2"])
    rn.tune_set("accel_leaf_small", small["cfg"]["accel_leaf_small"])
    return dict(best["cfg"], **small["cfg"]), rows


def tune_batch(quick: bool, reps: int, log):
    """Residency of the batched multi-view traversal: 16 orbit views (resolutions and spp as
    drawn) of the 744k scene in one captured batch; every view's AO checked bit for bit."""
    import torch
    sc = scenes.build_synthetic_scene(1, 500 if quick else 2000, 100 if quick else 500)
    tris, nrms = torch.from_numpy(sc.tris).cuda(), torch.from_numpy(sc.normals).cuda()
    acc = rn.LinearAccel(tris)
    views = [dict(g=rn.rasterize(tris, nrms, cam, w, h), spp=spp, radius=1.0)
             for (w, h, spp, cam) in scenes.orbit_views(1, 8 if quick else 16)]
    rows, ref = [], None
    for v in rn.TUNE_KEYS["batch_min_blocks"]:
        rn.tune_set("batch_min_blocks", v)
        b = rn.Batch(acc, views)
        b.run()
        out = [o["ao"].clone() for o in b.outputs]
        if ref is None:
            ref = out
        elif not all(bool((x == y).all()) for x, y in zip(out, ref)):
            raise RuntimeError("batch_min_blocks %d changed a traced result" % v)
        ms = _time(b.run, max(2, reps // 2))
        rows.append(dict(cfg={"batch_min_blocks": v}, ms={"batch": ms}))
        log("batch_min_blocks %d  %.3f ms" % (v, ms))
        del b
    best = min(rows, key=lambda r: r["ms"]["batch"])
    rn.tune_set("batch_min_blocks", best["cfg"]["batch_min_blocks"])
    return best["cfg"], rows


def tune_ssao(quick: bool, reps: int, log):
    import torch
    sc = scenes.build_test_scene()
    tris, nrms = torch.from_numpy(sc.tris).cuda(), torch.from_numpy(sc.normals).cuda()
    w, h = (1920, 1080) if quick else (3840, 2160)
    g = rn.rasterize(tris, nrms, sc.camera, w, h)
    rows = []
    ref = None
    for v in rn.TUNE_KEYS["ssao_tile_h"]:
        rn.tune_set("ssao_tile_h", v)
        ao = rn.compute_ssao(g)
        if ref is None:
            ref = ao.clone()
        elif not bool((ao == ref).all()):
            raise RuntimeError("ssao_tile_h %d changed the SSAO image" % v)
        ms = _time(lambda: rn.compute_ssao(g), reps)
        rows.append(dict(cfg={"ssao_tile_h": v}, ms={"ssao": ms}))
        log("ssao_tile_h %d  %.3f ms" % (v, ms))
    best = min(rows, key=lambda r: r["ms"]["ssao"])
    rn.tune_set("ssao_tile_h", best["cfg"]["ssao_tile_h"])
    return best["cfg"], rows


def tune_hybrid(quick: bool, reps: int, log):
    """Residency of the hybrid pass: the built-in scene from its camera and the 744k scene from
    an orbit view, each candidate's outputs (lit, triangle, t) checked bit for bit; scored by
    the geometric mean of the time ratios to the current setting."""
    import torch
    w, h = (1920, 1080) if quick else (3840, 2160)
    big = scenes.build_synthetic_scene(1, 500 if quick else 2000, 100 if quick else 500)
    wls = []
    for name, sc, cam in (("hybrid/model2", scenes.build_test_scene(), None),
                          ("hybrid/744k", big, scenes.orbit_views(1, 8)[0][3])):
        cam = cam if cam is not None else sc.camera
        tris, nrms = torch.from_numpy(sc.tris).cuda(), torch.from_numpy(sc.normals).cuda()
        g = rn.rasterize(tris, nrms, cam, w, h)
        acc = rn.LinearAccel(tris)
        wls.append((name, lambda g=g, acc=acc, eye=cam[:3], tl=sc.to_light: rn.hybrid(g, acc, eye, tl)))
    current = rn.tune_get("hybrid_min_blocks")
    rows, ref = [], None
    for v in rn.TUNE_KEYS["hybrid_min_blocks"]:
        rn.tune_set("hybrid_min_blocks", v)
        outs = [[o.clone() for o in fn()] for _, fn in wls]
        if ref is None:
            ref = outs
        elif not all(bool((a == b).all()) for out, r in zip(outs, ref) for a, b in zip(out, r)):
            raise RuntimeError("hybrid_min_blocks %d changed a hybrid result" % v)
        ms = {name: _time(fn, reps) for name, fn in wls}
        rows.append(dict(cfg={"hybrid_min_blocks": v}, ms=ms))
        log("hybrid_min_blocks %d  %s" % (v, "  ".join("%s %.3f ms" % kv for kv in ms.items())))
    base = next(r for r in rows if r["cfg"]["hybrid_min_blocks"] == current)["ms"]
    for r in rows:
        r["score"] = float(np.exp(np.mean([np.log(r["ms"][k] / base[k]) for k in base])))
    best = min(rows, key=lambda r: r["score"])
    rn.tune_set("hybrid_min_blocks", best["cfg"]["hybrid_min_blocks"])
    return best["cfg"], rows


def tune_conv(quick: bool, reps: int, log):
    import torch
    H, W = (544, 960) if quick else (1088, 1920)
    inf = rn.UNet(1, H, W, seed=1, inference=True)
    trn = rn.UNet(16 if quick else 64, 128, 128, seed=1)
    g = torch.Generator(device="cuda").manual_seed(0)
    x = torch.rand(1, H, W, 5, device="cuda", generator=g)
    xb = torch.rand(trn.shape[0], 128, 128, 5, device="cuda", generator=g)
    yb = torch.rand(trn.shape[0], 128, 128, device="cuda", generator=g)
    rows = []
    ref = None
    for v in rn.TUNE_KEYS["conv_bn_max"]:
        rn.tune_set("conv_bn_max", v)
        out = inf.forward(x)
        if ref is None:
            ref = out.clone()
        elif not bool((out == ref).all()):
            raise RuntimeError("conv_bn_max %d changed the network's output" % v)
        ms_f = _time(lambda: inf.forward(x), reps)
        ms_t = _time(lambda: trn.train_step(xb, yb, 0.0), max(2, reps // 2))
        rows.append(dict(cfg={"conv_bn_max": v}, ms={"forward": ms_f, "train_step": ms_t}))
        log("conv_bn_max %d  forward %.3f ms  train step %.3f ms" % (v, ms_f, ms_t))
    base = rows[-1]["ms"]
    for r in rows:
        r["score"] = float(np.exp(np.mean([np.log(r["ms"][k] / base[k]) for k in base])))
    best = min(rows, key=lambda r: r["score"])
    rn.tune_set("conv_bn_max", best["cfg"]["conv_bn_max"])
    # then the MMA form of the row-ring layers: row by row with A from shared memory, row by
    # row with A from TMEM, or fanned out (each input row feeding its three output rows)
    rows2, ref2 = [], None
    for cfg in ({"conv_tmem_a": 0, "conv_fan": 0}, {"conv_tmem_a": 1, "conv_fan": 0}, {"conv_tmem_a": 0, "conv_fan": 1}):
        for k, v in cfg.items():
            rn.tune_set(k, v)
        out = inf.forward(x)
        if ref2 is None:
            ref2 = out.clone()
        elif not bool((out == ref2).all()):
            raise RuntimeError("%s changed the network's output" % cfg)
        ms_f = _time(lambda: inf.forward(x), reps)
        ms_t = _time(lambda: trn.train_step(xb, yb, 0.0), max(2, reps // 2))
        rows2.append(dict(cfg=dict(cfg), ms={"forward": ms_f, "train_step": ms_t}))
        log("conv_tmem_a %d conv_fan %d  forward %.3f ms  train step %.3f ms"
            % (cfg["conv_tmem_a"], cfg["conv_fan"], ms_f, ms_t))
    base = rows2[0]["ms"]
    for r in rows2:
        r["score"] = float(np.exp(np.mean([np.log(r["ms"][k] / base[k]) for k in base])))
    best2 = min(rows2, key=lambda r: r["score"])
    for k, v in best2["cfg"].items():
        rn.tune_set(k, v)
    inf.close()
    trn.close()
    return dict(best["cfg"], **best2["cfg"]), rows + rows2


def tune_ploc_tail(quick: bool, reps: int, log):
    """From how many clusters on the PLOC rounds run in one block: builds of the 744k scene,
    a 1M-triangle soup and the reference's 20,000-triangle check soup (the trees checked node
    for node against the first candidate's); scored by the geometric mean of the ratios."""
    import torch
    rng = np.random.default_rng(1)
    n = 200000 if quick else 1000000
    c = rng.uniform(-50, 50, (n, 1, 3)).astype(np.float32)
    soup = (c + rng.uniform(-1, 1, (n, 3, 3)).astype(np.float32)).reshape(-1, 9)
    inputs = [("build/744k", scenes.build_synthetic_scene(1, 500 if quick else 2000, 100 if quick else 500).tris),
              ("build/soup", soup), ("build/20k", scenes.soup(20000, 7))]
    inputs = [(name, torch.from_numpy(np.ascontiguousarray(t)).cuda()) for name, t in inputs]
    current = {"ploc_tail": rn.tune_get("ploc_tail"), "ploc_tail_ctas": rn.tune_get("ploc_tail_ctas")}
    rows, ref = [], None
    current = dict(current, ploc_fused=rn.tune_get("ploc_fused"))
    for tail, ctas, fused in itertools.product(rn.TUNE_KEYS["ploc_tail"], rn.TUNE_KEYS["ploc_tail_ctas"],
                                               rn.TUNE_KEYS["ploc_fused"]):
        if tail == 0 and ctas != 1:
            continue                                   # no tail: the CTA count is unused
        cfg = {"ploc_tail": tail, "ploc_tail_ctas": ctas, "ploc_fused": fused}
        _apply(cfg)
        try:
            trees = [rn.build_ploc(t)[0].cpu() for _, t in inputs]
        except rn.RnError as e:                        # a cluster this device cannot schedule
            log("%s  not launchable: %s" % (cfg, e))
            continue
        if ref is None:
            ref = trees
        elif not all(bool((a == b).all()) for a, b in zip(trees, ref)):
            raise RuntimeError("%s changed a tree" % cfg)
        ms = {name: _time(lambda t=t: rn.LinearAccel(t).close(), reps) for name, t in inputs}
        rows.append(dict(cfg=cfg, ms=ms))
        log("%s  %s" % (cfg, "  ".join("%s %.3f ms" % kv for kv in ms.items())))
    base = next(r for r in rows if r["cfg"] == current)["ms"]
    for r in rows:
        r["score"] = float(np.exp(np.mean([np.log(r["ms"][k] / base[k]) for k in base])))
    best = min(rows, key=lambda r: r["score"])
    _apply(best["cfg"])
    # then the size under which the collapse runs in one block (same node counts required)
    current = rn.tune_get("collapse_block")
    rows2, ref2 = [], None
    for v in rn.TUNE_KEYS["collapse_block"]:
        rn.tune_set("collapse_block", v)
        infos = [rn.LinearAccel(t).info() for _, t in inputs]
        if ref2 is None:
            ref2 = infos
        elif infos != ref2:
            raise RuntimeError("collapse_block %d changed an accelerator: %s" % (v, infos))
        ms = {name: _time(lambda t=t: rn.LinearAccel(t).close(), reps) for name, t in inputs}
        rows2.append(dict(cfg={"collapse_block": v}, ms=ms))
        log("collapse_block %d  %s" % (v, "  ".join("%s %.3f ms" % kv for kv in ms.items())))
    base = next(r for r in rows2 if r["cfg"]["collapse_block"] == current)["ms"]
    for r in rows2:
        r["score"] = float(np.exp(np.mean([np.log(r["ms"][k] / base[k]) for k in base])))
    best2 = min(rows2, key=lambda r: r["score"])
    rn.tune_set("collapse_block", best2["cfg"]["collapse_block"])
    return dict(best["cfg"], **best2["cfg"]), rows + rows2


def tune_pt(quick: bool, reps: int, log):
    """The path tracer's form: one kernel a path (a thread a sample, or persistent threads
    regenerating paths: 4, 8, 16 blocks per SM) or the wavefront form over 64K to 2M path
    slots, and the wavefront shade kernel's register budget: retro_room and iso_street (the reference's lit scenes, from the test fixtures) at
    1280 x 720, 16 spp, every candidate's radiance, variance and diffuse checked bit for bit."""
    import os
    z = np.load(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "tests", "golden",
                             "pt_scenes.npz"))
    wls = []
    for key in ("retro_room", "iso_street"):
        sc = {k.split("/", 1)[1]: z[k] for k in z.files if k.startswith(key + "/")}
        cam = [float(v) for v in sc.pop("camera")]
        s = rn.PtScene(sc)
        d = dict(seed=1, spp=4 if quick else 16, width=320 if quick else 1280, height=180 if quick else 720, camera=cam)
        wls.append(("pt/" + key, s, d))
    keys = ("pt_wave", "pt_regen", "pt_shade_blocks")
    current = {k: rn.tune_get(k) for k in keys}
    cands = [dict(current, pt_wave=0, pt_regen=v) for v in rn.TUNE_KEYS["pt_regen"]]
    cands += [dict(current, pt_wave=v) for v in rn.TUNE_KEYS["pt_wave"] if v >= 64]
    cands += [dict(current, pt_shade_blocks=v) for v in rn.TUNE_KEYS["pt_shade_blocks"]]
    uniq = []
    for c in cands + [dict(current)]:
        if c not in uniq:
            uniq.append(c)
    cands = uniq
    rows, ref = [], None
    for cfg in cands:
        _apply(cfg)
        outs = [rn.path_trace(s, d, device=True, planes=("radiance", "variance", "diffuse")) for _, s, d in wls]
        if ref is None:
            ref = outs
        elif not all(bool((o[k] == r[k]).all()) for o, r in zip(outs, ref) for k in o):
            raise RuntimeError("%s changed a path-traced result" % cfg)
        ms = {name: _time(lambda s=s, d=d: rn.path_trace(s, d, device=True, planes=("radiance",)), max(2, reps // 2))
              for name, s, d in wls}
        rows.append(dict(cfg=dict(cfg), ms=ms))
        log("pt %s  %s" % (cfg, "  ".join("%s %.3f ms" % kv for kv in ms.items())))
    base = next(r for r in rows if r["cfg"] == current)["ms"]
    for r in rows:
        r["score"] = float(np.exp(np.mean([np.log(r["ms"][k] / base[k]) for k in base])))
    best = min(rows, key=lambda r: r["score"])
    _apply(best["cfg"])
    for _, s, _ in wls:
        s.close()
    return best["cfg"], rows


STAGES = {"accel": tune_accel, "trace": tune_trace, "walk": tune_walk, "frontier_min_spp": tune_frontier_min_spp,
          "frontier_tail": tune_frontier_tail, "batch": tune_batch, "ssao": tune_ssao, "conv": tune_conv,
          "hybrid": tune_hybrid, "ploc_tail": tune_ploc_tail, "pt": tune_pt}


def read_tune_file(path: str) -> dict:
    """The "key = value" lines of a tune file ('#' starts a comment), as rn_tune_load reads them."""
    out = {}
    for line in open(path):
        line = line.split("#", 1)[0].strip()
        if not line:
            continue
        k, v = (x.strip() for x in line.split("=", 1))
        if k not in rn.TUNE_KEYS:
            raise ValueError("%s: unknown tune key %r" % (path, k))
        out[k] = int(v)
    return out


def write_tune_file(path: str, cfg: dict, note: str) -> None:
    with open(path, "w") as f:
        f.write("# launch shapes picked by autotune.py: %s\n" % note)
        for k in rn.TUNE_KEYS:
            if k in cfg:
                f.write("%s = %d\n" % (k, cfg[k]))


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--out", required=True, help="tune file to write")
    ap.add_argument("--report", default=None, help="JSON with every candidate's timings")
    ap.add_argument("--quick", action="store_true", help="smaller workloads (a test run)")
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--stages", default=None, help="comma-separated stages to run (default: all): "
                    + ",".join(STAGES))
    ap.add_argument("--merge", default=None, help="tune file whose values apply first and are kept")
    a = ap.parse_args(argv)
    import torch
    rn.init(load_tune=False)
    t0 = time.time()
    log = lambda m: print(m, flush=True)
    cfg, report = {}, {}
    if a.merge:
        cfg.update(read_tune_file(a.merge))
        _apply(cfg)
    names = STAGES if not a.stages else [s.strip() for s in a.stages.split(",") if s.strip()]
    unknown = [s for s in names if s not in STAGES]
    if unknown:
        ap.error("unknown stages %s (known: %s)" % (unknown, ", ".join(STAGES)))
    for name in STAGES:
        if name in names:
            c, report[name] = STAGES[name](a.quick, a.reps, log)
            cfg.update(c)
    dev = torch.cuda.get_device_name(0)
    note = "%s, %d SMs, %s workloads, %.0f s" % (dev, torch.cuda.get_device_properties(0).multi_processor_count,
                                                 "quick" if a.quick else "full", time.time() - t0)
    write_tune_file(a.out, cfg, note)
    log("picked %s" % json.dumps(cfg))
    if a.report:
        json.dump(dict(picked=cfg, note=note, candidates=report), open(a.report, "w"), indent=1)


if __name__ == "__main__":
    sys.exit(main())
