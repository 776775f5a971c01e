#!/usr/bin/env python3
"""Benchmark of the GB300 AO path on the 4K workload.

Workload: the reference's built-in scene and default camera at 3840 x 2160, ray-traced AO at
256 cosine-weighted rays per pixel with lighting model 2's sky and sun visibility (radius 2),
SSAO with 24 taps, and the reconcile (tolerance 0.12): one "step" is one such AO frame, the
three passes of src/renderer/render.cpp:29-54. Inputs are synthetic (the built-in scene,
rasterized on the GPU by this library); no dataset is involved.

  value    AO Grays/s over all ranks, G-buffer resident in HBM, device pointers (the 207 MB
           G-buffer exceeds the 129 MB L2, so no flush is needed between steps)
  e2e      the same metric through the C ABI with pinned host buffers: every step the
           G-buffer crosses from host memory and ao, sky, sun, ss and the error map cross
           back (the library's passes read and write mapped host memory themselves, the
           traversal mirroring the G-buffer into HBM for the SSAO; no copy-engine copy)
  roofline the traversal kernel (trace_kernel): algorithmic bytes per launch = 4-wide node
           fetches x 128 B + leaf-triangle fetches x 48 B, from the library's traversal
           counters over the whole frame, divided by the kernel's CUDA-event time
  cpu_baseline  the oracle (a C restatement of the reference's CPU path) on this host's
           cores, on every 4th row of the same frame
  surrogate_4k  (one GPU) the surrogate-versus-plain-RT head-to-head on the 7.88M-triangle
           scene, measured after the frame's timed region; RN_BENCH_NO_SURROGATE=1 leaves
           this separate report out (for a launch list of the frame alone) and changes
           nothing in the frame's measurement

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
    python bench.py --workload batch|large|surrogate|hybrid|build|pathtrace   (the other workloads)
"""
from __future__ import annotations

import argparse
import csv
import io
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "raw-native_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

W_PX, H_PX, SPP, RADIUS, SS_SAMPLES, TOL = 3840, 2160, 256, 2.0, 24, 0.12
METRIC = "4K AO ms/frame at RMSE<=0.02 vs 1024-spp: surrogate vs plain GPU RT; AO Grays/s"
WORKLOAD = ("plain GPU RT AO frame, built-in scene (14 triangles), default camera, 3840x2160, 256 spp, "
            "sky+sun visibility, SSAO 24 taps, reconcile")


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--cpu-row-stride", type=int, default=4, help="rows of the CPU sample: every n-th")
    p.add_argument("--profile", choices=["frame", "trace", "ssao", "reconcile", "build", "unet", "surrogate",
                                         "pathtrace", "train"],
                   help="run only this pass `--steps` times after `--warmup` (for ncu), print nothing")
    p.add_argument("--spp", type=int, default=SPP, help="samples per pixel (the benchmark uses 256)")
    p.add_argument("--tris", type=int, default=1000000, help="--profile build: soup triangles")
    p.add_argument("--workload", default="4k", choices=["4k", "batch", "large", "surrogate", "hybrid", "build",
                                                        "pathtrace"],
                   help="4k: the benchmark (built-in scene, 3840x2160, 256 spp); batch: 64 orbit views of the "
                        "seeded 744k-triangle scene in one batch; large: 16 4K views of the 7.88M-triangle scene")
    p.add_argument("--views", type=int, default=0, help="batch/large: number of views (default 64 / 16)")
    p.add_argument("--res", default="3840x2160", help="--profile unet: frame size WxH")
    return p.parse_args()


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


# ---------------------------------------------------------------- clocks during the timed region
class Clocks:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.file,
                                         stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        self.file.flush()
        self.file.seek(0)
        rows = [r for r in csv.reader(io.StringIO(self.file.read())) if len(r) >= 9]
        os.unlink(self.file.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "", 1).isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "", 1).isdigit()]
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].strip().lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def measured_peak():
    try:
        mp = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        return float(mp["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def committed_profile():
    """The traversal's figures from the committed ncu summary of the 4K frame (dict, or {}):
    DRAM bytes per launch, issue-active fraction and SIMT efficiency (active threads per
    executed warp instruction / 32)."""
    try:
        return json.load(open(os.path.join(ROOT, "profiles", "trace_kernel_4k_256spp.json")))
    except Exception:
        return {}


# ---------------------------------------------------------------- CPU (oracle) timing
def cpu_frame_sample(row_stride: int, threads: int):
    """The oracle's AO frame on every row_stride-th row: (AO rays traced, seconds)."""
    from oracle import oracle as O
    import numpy as np
    import ctypes as C
    tris, nrm9, light = O.test_scene()
    _, pos, nrm, mask = O.rasterize(tris, nrm9, O.DEFAULT_CAMERA, W_PX, H_PX)
    L = O.lib()
    ao = np.zeros((H_PX, W_PX), np.float32)
    sky = np.zeros_like(ao)
    sun = np.zeros_like(ao)
    tl = (C.c_float * 3)(*(-light))
    acc = L.rno_accel_build(np.ascontiguousarray(tris), len(tris))
    rows = np.arange(0, H_PX, row_stride)
    t0 = time.perf_counter()
    L.rno_trace(W_PX, H_PX, pos, nrm, mask, acc, tris, len(tris), SPP, RADIUS, C.cast(tl, C.c_void_p), 0, ao,
                sky.ctypes.data_as(C.c_void_p), sun.ctypes.data_as(C.c_void_p), threads, 0, row_stride)
    sub = np.ascontiguousarray(mask[rows])
    ss = O.ssao(np.ascontiguousarray(pos[rows]), np.ascontiguousarray(nrm[rows]), sub, SS_SAMPLES, RADIUS, threads)
    O.reconcile(ss, np.ascontiguousarray(ao[rows]), sub, TOL)
    dt = time.perf_counter() - t0
    L.rno_accel_free(acc)
    return int(sub.sum()) * SPP, dt, len(rows)


def frame_config(world: int, covered: int) -> dict:
    """The workload's config, the same dict on both arms (the two lines describe one workload)."""
    return {"workload": WORKLOAD, "width": W_PX, "height": H_PX, "spp": SPP, "radius": RADIUS,
            "ss_samples": SS_SAMPLES, "tolerance": TOL, "covered_px": covered, "ao_rays_per_step": covered * SPP,
            "parallelism": "replicas (one full frame per GPU)" if world > 1 else "single GPU",
            "l2": "inputs larger than L2: 207 MB G-buffer > 129 MB L2, no flush"}


def covered_pixels_cpu() -> int:
    from oracle import oracle as O
    tris, nrm9, _ = O.test_scene()
    return int(O.rasterize(tris, nrm9, O.DEFAULT_CAMERA, W_PX, H_PX)[3].sum())


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    stride = max(args.cpu_row_stride, 1)
    for _ in range(args.warmup):
        cpu_frame_sample(stride * 4, threads)
    rays, secs = 0, 0.0
    for _ in range(args.steps):
        r, dt, nrows = cpu_frame_sample(stride, threads)
        rays += r
        secs += dt
    v = rays / secs / 1e9
    sample = "every %dth row of the 4K frame (%d rows), visibility + SSAO + reconcile, oracle port (SAH BVH)" % (
        stride, nrows)
    print(json.dumps({
        "metric": METRIC, "value": v, "unit": "Grays/s", "impl": "reference", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": secs / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": frame_config(world, covered_pixels_cpu()),
        "cpu_baseline": {"value": v, "unit": "Grays/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": v, "unit": "Grays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


# ---------------------------------------------------------------- GPU
def run_ours(args):
    import numpy as np
    import torch
    import rn_ao as rn
    import scene as scenes

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        pg = dist
    rn.init()
    sc = scenes.build_test_scene()
    tris = torch.from_numpy(sc.tris).cuda()
    nrms = torch.from_numpy(sc.normals).cuda()
    g = rn.rasterize(tris, nrms, sc.camera, W_PX, H_PX)
    t0 = time.perf_counter()
    acc = rn.LinearAccel(tris)
    build_ms = (time.perf_counter() - t0) * 1e3
    covered = int(g.mask.sum().item())
    rays = covered * SPP
    outs = {k: torch.empty(H_PX, W_PX, device="cuda") for k in ("ao", "sky", "sun", "ss", "err")}
    tl = sc.to_light

    def frame():
        return rn.ao_frame(g, acc, SPP, RADIUS, SS_SAMPLES, TOL, to_light=tl, outputs=outs)

    def barrier():
        if pg:
            pg.barrier()

    def max_over_ranks(x: float) -> float:
        if not pg:
            return x
        t = torch.tensor([x], device="cuda")
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        return float(t.item())

    stream = torch.cuda.current_stream()
    # ---- resident: device pointers
    for _ in range(args.warmup):
        frame()
    torch.cuda.synchronize()
    barrier()
    with Clocks(local) as clk:
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            last = frame()
        e1.record(stream)
        torch.cuda.synchronize()
    barrier()
    ms = max_over_ranks(e0.elapsed_time(e1) / args.steps)
    clocks = clk.summary()
    value = world * rays / (ms * 1e-3) / 1e9
    rec = last["rec"]

    # ---- end to end: pinned host buffers through the C ABI
    hpos = g.position.cpu().pin_memory()
    hnrm = g.normal.cpu().pin_memory()
    hmask = g.mask.cpu().pin_memory()
    hg = rn.GBuffer(hpos.numpy(), hnrm.numpy(), hmask.numpy())
    houts = {k: torch.empty(H_PX, W_PX).pin_memory().numpy() for k in ("ao", "sky", "sun", "ss", "err")}
    for _ in range(args.warmup):
        rn.ao_frame(hg, acc, SPP, RADIUS, SS_SAMPLES, TOL, to_light=tl, outputs=houts)
    torch.cuda.synchronize()
    barrier()
    e2, e3 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e2.record(stream)
    for _ in range(args.steps):
        rn.ao_frame(hg, acc, SPP, RADIUS, SS_SAMPLES, TOL, to_light=tl, outputs=houts)
    e3.record(stream)
    torch.cuda.synchronize()
    barrier()
    e2e_ms = max_over_ranks(e2.elapsed_time(e3) / args.steps)
    h2d = hpos.numel() * 4 + hnrm.numel() * 4 + hmask.numel()
    d2h = 5 * H_PX * W_PX * 4 + 24
    same = np.array_equal(houts["ao"], outs["ao"].cpu().numpy()) and np.array_equal(houts["err"], outs["err"].cpu().numpy())

    # ---- roofline of the dominant kernel: the traversal
    stats = rn.trace_stats(g, acc, SPP, RADIUS, to_light=tl, tile_stride=1)
    alg_bytes = stats["nodes"] * 128 + stats["tris"] * 48
    for _ in range(2):
        rn.compute_rt_visibility(g, acc, SPP, RADIUS, tl)
    torch.cuda.synchronize()
    e4, e5 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    nvis = max(3, args.steps // 2)
    e4.record(stream)
    for _ in range(nvis):
        rn.compute_rt_visibility(g, acc, SPP, RADIUS, tl)
    e5.record(stream)
    torch.cuda.synchronize()
    trace_ms = e4.elapsed_time(e5) / nvis
    peak, peak_kind = measured_peak()
    achieved = alg_bytes / (trace_ms * 1e-3) / 1e9
    prof = committed_profile()
    traffic = prof.get("dram_bytes_per_launch")

    if rank != 0:
        return
    cpu = None
    if world == 1:
        r, dt, nrows = cpu_frame_sample(args.cpu_row_stride, os.cpu_count() or 1)
        cpu = {"value": r / dt / 1e9, "unit": "Grays/s", "cores": os.cpu_count() or 1, "kind": "port",
               "sample": "every %dth row of the same 4K frame (%d rows, %.1f s): visibility + SSAO + reconcile, "
                         "oracle port with its SAH BVH" % (args.cpu_row_stride, nrows, dt)}
    out = {
        "metric": METRIC, "value": value, "unit": "Grays/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": frame_config(world, covered),
        "bvh_build_ms": round(build_ms, 3),
        "ms_per_frame": ms,
        "frame_result": {"rmse": rec.rmse, "max_error": rec.max_error, "pixels": rec.pixels,
                         "within_tolerance": rec.within_tolerance},
        "e2e": {"value": world * rays / (e2e_ms * 1e-3) / 1e9, "unit": "Grays/s", "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "matches_resident": bool(same)},
        "gpu_launches": 2 * args.steps,
        "roofline": {"bound": "hbm", "kernel": "trace_kernel", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
                     "limit": "instruction issue: the algorithmic node/triangle bytes are served by L1/L2 "
                              "(the BVH is cache-resident), so frac is cache-served node bandwidth against the "
                              "HBM peak; dram_frac is the HBM share actually used, issue_active the binding limit's "
                              "fraction",
                     "binding_limit": "instruction issue (ncu smsp__issue_active of the same kernel)",
                     "binding_frac": prof.get("issue_active"),
                     "dram_frac": (traffic / (trace_ms * 1e-3) / 1e9 / peak) if traffic else None,
                     "issue_active": prof.get("issue_active"), "simt_efficiency": prof.get("simt_efficiency"),
                     "profile_source": prof.get("source"),
                     "traffic": traffic, "algorithmic_bytes_per_launch": alg_bytes, "launch_ms": trace_ms,
                     "rays_per_launch": stats["rays"], "sky_rays_per_launch": stats["sky_rays"],
                     "walks_per_launch": stats["rays"] + covered,
                     "node_fetches_per_walk": stats["nodes"] / max(1, stats["rays"] + covered),
                     "tri_fetches_per_walk": stats["tris"] / max(1, stats["rays"] + covered)},
        "clocks": clocks,
    }
    if cpu:
        out["cpu_baseline"] = cpu
    if world == 1 and os.path.exists(SURROGATE_WEIGHTS) and not os.environ.get("RN_BENCH_NO_SURROGATE"):
        # the metric's other half: surrogate vs plain GPU RT at 4K on the 7.88M-triangle scene
        out["surrogate_4k"] = surrogate_headtohead(max(2, args.steps // 4), max(1, args.warmup // 3))
    if world == 1 and not os.environ.get("RN_BENCH_NO_EXTRA"):
        # the secondary workloads, short runs after the frame's timed region (each with its own
        # CUDA-event timing; the full runs are `--workload batch|build|pathtrace`)
        short = argparse.Namespace(steps=2, warmup=1, views=0, spp=SPP, workload="batch")
        b = views_report(short)
        out["batch_views"] = {k: b[k] for k in ("value", "unit", "ms_per_step", "ms_per_view", "config", "clocks")}
        out["accel_build"] = {k: v for k, v in build_report(argparse.Namespace(steps=3, warmup=1)).items()
                              if k in ("value", "unit", "ms_per_step", "builds", "config")}
        os.environ["RN_BENCH_NO_CPU"] = "1"
        p = pathtrace_report(argparse.Namespace(steps=2, warmup=1), spp=16)
        out["pathtrace"] = {k: p[k] for k in ("value", "unit", "ms_per_step", "scenes", "config")}
    print(json.dumps(out), flush=True)


def run_profile(args):
    """One pass, repeated, for a profiler: the 4K G-buffer and accelerator are built first.
    unet: the surrogate network's forward on a 3840 x 2160 frame (padded to 2176 x 3840);
    surrogate: one rn_surrogate_ao frame of the 7.88M-triangle scene at 4K (256-spp fallback)."""
    import torch
    import rn_ao as rn
    import scene as scenes
    torch.cuda.set_device(0)
    rn.init()
    if args.profile == "unet":
        import surrogate as S
        fw, fh = (int(v) for v in args.res.split("x"))
        net = rn.UNet(1, *S.padded_shape(fh, fw), inference=True)
        S.load_weights(net, SURROGATE_WEIGHTS)
        x = torch.rand(1, *net.shape[1:], 5, device="cuda")
        for _ in range(args.warmup + args.steps):
            net.forward(x)
        torch.cuda.synchronize()
        return
    if args.profile == "train":
        # surrogate training steps at the training recipe's shape (batch 64 of 128 x 128 crops,
        # Adam): forward, backward (dgrad on the implicit convolution, wgrad on tc_gemm), Adam
        net = rn.UNet(64, 128, 128, seed=1)
        g = torch.Generator(device="cuda").manual_seed(1)
        x = torch.rand(64, 128, 128, 5, device="cuda", generator=g)
        y = torch.rand(64, 128, 128, device="cuda", generator=g)
        for _ in range(args.warmup + args.steps):
            net.train_step(x, y, 1e-3)
        torch.cuda.synchronize()
        return
    if args.profile == "pathtrace":
        # the path tracer on retro_room at --res (default 3840x2160 is too large a capture:
        # pass e.g. --res 320x180) and --spp samples
        fw, fh = (int(v) for v in args.res.split("x"))
        sc, cam = pt_fixture_scene("retro_room")
        s = rn.PtScene(sc)
        d = dict(seed=1, spp=args.spp, width=fw, height=fh, camera=[float(v) for v in cam])
        for _ in range(args.warmup + args.steps):
            rn.path_trace(s, d, device=True)
        torch.cuda.synchronize()
        return
    if args.profile == "surrogate":
        import surrogate as S
        sc = scenes.build_synthetic_scene(5, 10000, 6000)
        tris = torch.from_numpy(sc.tris).cuda()
        g, depth = rn.rasterize(tris, torch.from_numpy(sc.normals).cuda(), scenes.orbit_views(5, 16)[5][3], 3840, 2160,
                                want_depth=True)
        acc = rn.LinearAccel(tris)
        net = rn.UNet(1, *S.padded_shape(2160, 3840), inference=True)
        S.load_weights(net, SURROGATE_WEIGHTS)
        for _ in range(args.warmup + args.steps):
            rn.surrogate_ao(net, g, depth, acc, 256, 1.0, 3.0)
        torch.cuda.synchronize()
        return
    radius = RADIUS
    if args.workload == "4k":
        sc = scenes.build_test_scene()
        cam, w, h = sc.camera, W_PX, H_PX
    else:
        # one 1920x1080 orbit view of the large scene (or of the batched-views scene)
        sc = (scenes.build_synthetic_scene(5, 10000, 6000) if args.workload == "large"
              else scenes.build_synthetic_scene(1, 2000, 500))
        cam, w, h, radius = scenes.orbit_views(5, 16)[0][3], 1920, 1080, 1.0
    tris = torch.from_numpy(sc.tris).cuda()
    g = rn.rasterize(tris, torch.from_numpy(sc.normals).cuda(), cam, w, h)
    acc = rn.LinearAccel(tris)
    if os.environ.get("RN_PRINT_STATS"):
        st = rn.trace_stats(g, acc, args.spp, radius, tile_stride=1)
        print(json.dumps({"workload": args.workload, "spp": args.spp, "radius": radius, **st,
                          "nodes_per_ray": st["nodes"] / max(1, st["rays"]), "tris_per_ray": st["tris"] / max(1, st["rays"]),
                          "accel": acc.info()}), flush=True)
    outs = {k: torch.empty(h, w, device="cuda") for k in ("ao", "sky", "sun", "ss", "err")}
    if args.profile == "build":
        import numpy as np
        rng = np.random.default_rng(1)
        c = rng.uniform(-50, 50, (args.tris, 1, 3)).astype(np.float32)
        t = (c + rng.uniform(-1, 1, (args.tris, 3, 3)).astype(np.float32)).reshape(args.tris, 9)
        soup = torch.from_numpy(np.ascontiguousarray(t)).cuda()
    tl = sc.to_light if args.workload == "4k" else None
    fn = {"frame": lambda: rn.ao_frame(g, acc, args.spp, radius, SS_SAMPLES, TOL, to_light=tl, outputs=outs),
          "trace": lambda: rn.compute_rt_visibility(g, acc, args.spp, radius, tl),
          "ssao": lambda: rn.compute_ssao(g, SS_SAMPLES, radius),
          "reconcile": lambda: rn.reconcile(outs["ss"], outs["ao"], g.mask, TOL),
          "build": lambda: rn.LinearAccel(soup)}[args.profile]
    for _ in range(args.warmup + args.steps):
        fn()
    torch.cuda.synchronize()


def run_views(args):
    """The batched-views and large-scene workloads: one batch frame = every view's AO (radius 1),
    SSAO and reconcile, from one traversal launch and one SSAO launch (a CUDA graph)."""
    print(json.dumps(views_report(args)), flush=True)


def views_report(args) -> dict:
    import numpy as np
    import torch
    import rn_ao as rn
    import scene as scenes
    torch.cuda.set_device(0)
    rn.init()
    if args.workload == "batch":
        sc = scenes.build_synthetic_scene(1, 2000, 500)
        specs = scenes.orbit_views(1, args.views or 64)
        name = "batched views: seeded 744k-triangle scene, %d orbit views, resolutions/spp as drawn, radius 1" % len(specs)
    else:
        sc = scenes.build_synthetic_scene(5, 10000, 6000)
        n = args.views or 16
        specs = [(3840, 2160, args.spp if args.spp != SPP else 64, cam)
                 for (_, _, _, cam) in scenes.orbit_views(5, n)]
        name = "large: seeded 7.88M-triangle scene, %d 4K orbit views, %d spp, radius 1" % (n, specs[0][2])
    tris = torch.from_numpy(sc.tris).cuda()
    nrms = torch.from_numpy(sc.normals).cuda()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    acc = rn.LinearAccel(tris)
    build_ms = (time.perf_counter() - t0) * 1e3
    views = []
    for w, h, spp, cam in specs:
        views.append(dict(g=rn.rasterize(tris, nrms, cam, w, h), spp=spp, radius=1.0))
    covered_rays = sum(int(v["g"].mask.sum().item()) * v["spp"] for v in views)
    b = rn.Batch(acc, views, ss_samples=SS_SAMPLES, tolerance=TOL)
    for _ in range(args.warmup):
        b.run()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    with Clocks(0) as clk:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            res = b.run()
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    info = acc.info()
    out = {"metric": METRIC, "value": covered_rays / (ms * 1e-3) / 1e9, "unit": "Grays/s", "n_gpus": 1,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "config": {"workload": name, "triangles": int(len(sc.tris)), "views": len(views),
                      "ao_rays_per_step": covered_rays, "bvh_build_ms": round(build_ms, 1),
                      "bvh_wide_nodes": info["wide_nodes"], "ploc_rounds": info["ploc_rounds"]},
           "ms_per_view": ms / len(views),
           "rmse_mean": float(np.mean([r.rmse for r in res])), "clocks": clk.summary(),
           "gpu_launches": 2 * args.steps}
    return out


# the network trained on mixed-density scenes (the 200-box recipe's network is
# weights/surrogate_bf16.npz; RN_SURROGATE_WEIGHTS selects another file)
SURROGATE_WEIGHTS = os.path.join(PKG, "weights", "surrogate_mixed_bf16.npz")


def equal_rmse_spp(rmse_at, bar: float = 0.02, lo: int = 1, hi: int = 1024):
    """The smallest integer spp whose RMSE meets `bar` on every view: rmse_at(spp) returns the
    worst view's RMSE. Powers of two first (the last failing one and the first passing one
    bracket the answer), then bisection on the integers between them. Returns (spp, the
    evaluated {spp: worst RMSE})."""
    seen = {}

    def worst(s):
        if s not in seen:
            seen[s] = rmse_at(s)
        return seen[s]

    p = lo
    while p < hi and worst(p) > bar:
        p *= 2
    p = min(p, hi)
    if worst(p) > bar:
        return p, seen
    a, b = max(lo, p // 2), p           # worst(a) > bar unless a == p; worst(b) <= bar
    if a == b or worst(a) <= bar:
        return a, seen
    while b - a > 1:
        m = (a + b) // 2
        if worst(m) <= bar:
            b = m
        else:
            a = m
    return b, seen


def cpu_large_sample(frames, tris, spp: int, row_stride: int, threads: int):
    """The oracle (its SAH BVH, a restatement of the reference's trace) at `spp` on every
    row_stride-th row of each view's G-buffer (read back from the GPU; the GPU rasterizer
    equals the oracle's): (AO rays traced, seconds of tracing, seconds of BVH build, rows)."""
    from oracle import oracle as O
    import numpy as np
    L = O.lib()
    t0 = time.perf_counter()
    hnd = L.rno_accel_build(np.ascontiguousarray(tris), len(tris))
    build_s = time.perf_counter() - t0
    rays, secs, nrows = 0, 0.0, 0
    try:
        for k, f in enumerate(frames):
            g = f["g"]
            pos = np.ascontiguousarray(g.position.cpu().numpy())
            nrm = np.ascontiguousarray(g.normal.cpu().numpy())
            mask = np.ascontiguousarray(g.mask.cpu().numpy())
            h, w = mask.shape
            ao = np.zeros((h, w), np.float32)
            row0 = (7 * k) % row_stride
            t0 = time.perf_counter()
            L.rno_trace(w, h, pos, nrm, mask, hnd, tris, len(tris), spp, 1.0, None, 0, ao, None, None, threads,
                        row0, row_stride)
            secs += time.perf_counter() - t0
            rows = np.arange(row0, h, row_stride)
            rays += int(mask[rows].sum()) * spp
            nrows += len(rows)
    finally:
        L.rno_accel_free(hnd)
    return rays, secs, build_s, nrows


def surrogate_headtohead(steps: int, warmup: int, n_views: int = 16, weights: str = None, cpu_views: int = 4):
    """The 4K head-to-head: orbit views at 3840 x 2160 of the seeded 7.88M-triangle scene, AO
    radius 1. Truth: the 1024-spp trace of each view. Plain GPU RT runs at the smallest integer
    spp whose RMSE against the truth is <= 0.02 on every view (powers of two, then bisection:
    equal_rmse_spp); the surrogate (rn_surrogate_ao: 4-spp trace + U-Net + fallback tiles traced
    at that same spp) runs on the same views. Both are timed per frame with CUDA events,
    G-buffers resident. The CPU baseline is the oracle at 64 spp on the host's cores, on every
    97th row of the first `cpu_views` views, extrapolated to a frame (cpu_views 0: none)."""
    import numpy as np
    import torch
    import rn_ao as rn
    import scene as scenes
    import surrogate as S
    weights = weights or os.environ.get("RN_SURROGATE_WEIGHTS") or SURROGATE_WEIGHTS
    sc = scenes.build_synthetic_scene(5, 10000, 6000)
    tris, nrms = torch.from_numpy(sc.tris).cuda(), torch.from_numpy(sc.normals).cuda()
    acc = rn.LinearAccel(tris)
    W, H, R = 3840, 2160, 1.0
    net = rn.UNet(1, *S.padded_shape(H, W), inference=True)
    meta = S.load_weights(net, weights)
    frames = []
    for (_, _, _, cam) in scenes.orbit_views(5, n_views):
        g, depth = rn.rasterize(tris, nrms, cam, W, H, want_depth=True)
        truth = rn.compute_rtao(g, acc, S.SPP_TARGET, R)
        frames.append(dict(g=g, depth=depth, truth=truth, covered=int(g.mask.sum().item())))

    def worst_rmse(spp):
        return max(S.rmse(rn.compute_rtao(f["g"], acc, spp, R), f["truth"], f["g"].mask) for f in frames)

    spp_rt, searched = equal_rmse_spp(worst_rmse, 0.02, 16, 1024)
    stream = torch.cuda.current_stream()

    def timed(fn, reps):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            out = fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps, out

    rt_ms, sur_ms, sur_rmse, fb, t4_ms, net_ms = [], [], [], [], [], []
    x = torch.zeros(1, *net.shape[1:], 5, device="cuda")
    with Clocks(0) as clk:
        for f in frames:
            ms, _ = timed(lambda: rn.compute_rtao(f["g"], acc, spp_rt, R), steps)
            rt_ms.append(ms)
            ms, (ao, st) = timed(lambda: rn.surrogate_ao(net, f["g"], f["depth"], acc, spp_rt, R, 3.0), steps)
            sur_ms.append(ms)
            sur_rmse.append(S.rmse(ao, f["truth"], f["g"].mask))
            fb.append(st["fallback_fraction"])
            t4_ms.append(timed(lambda: rn.compute_rtao(f["g"], acc, S.SPP_IN, R), steps)[0])
        net_ms.append(timed(lambda: net.forward(x), steps)[0])
    rays_rt = sum(f["covered"] for f in frames) * spp_rt
    cpu = None
    if cpu_views > 0:
        stride, cpu_spp = 97, 64
        cr, cs, cb, nrows = cpu_large_sample(frames[:cpu_views], sc.tris, cpu_spp, stride, os.cpu_count() or 1)
        rate = cr / cs
        px = float(np.mean([f["covered"] for f in frames]))
        cpu = {"value": rate / 1e9, "unit": "Grays/s", "cores": os.cpu_count() or 1, "kind": "port", "spp": cpu_spp,
               "ms_per_frame_extrapolated": px * cpu_spp / rate * 1e3,
               "ms_per_frame_at_plain_rt_spp_extrapolated": px * spp_rt / rate * 1e3,
               "bvh_build_s": cb,
               "sample": "every %dth row of %d of the %d 4K views (%d rows, %.2f s of tracing, %.1f M AO rays): AO "
                         "at %d spp, radius 1, oracle port (SAH BVH, built once in %.1f s, not counted); per-frame "
                         "figures extrapolated from the rate by the views' mean covered pixels"
                         % (stride, len(frames[:cpu_views]), len(frames), nrows, cs, cr / 1e6, cpu_spp, cb)}
    return {
        "workload": "surrogate vs plain GPU RT: seeded 7.88M-triangle scene, %d orbit views at 3840x2160, radius 1, "
                    "truth 1024 spp" % n_views,
        "triangles": int(len(sc.tris)), "views": n_views, "weights": os.path.relpath(weights, ROOT),
        "trained": {k: meta.get(k) for k in ("steps", "batch", "lr", "data_digest")},
        "training_scenes": (meta.get("data") or {}).get("density", "fixed"),
        "plain_rt": {"spp": spp_rt, "spp_rule": "smallest integer spp with RMSE <= 0.02 on every view "
                                                "(powers of two, then bisection)",
                     "ms_per_frame": float(np.mean(rt_ms)),
                     "grays_per_s": rays_rt / (sum(rt_ms) * 1e-3) / 1e9,
                     "rmse_by_spp_max_over_views": {int(k): v for k, v in sorted(searched.items())}},
        "surrogate": {"ms_per_frame": float(np.mean(sur_ms)), "rmse_max_over_views": max(sur_rmse),
                      "rmse_mean": float(np.mean(sur_rmse)), "fallback_fraction_mean": float(np.mean(fb)),
                      "spp_input": S.SPP_IN, "fallback_spp": spp_rt, "trace4_ms": float(np.mean(t4_ms)),
                      "network_ms": float(np.mean(net_ms))},
        "speedup_vs_plain_rt": float(np.mean(rt_ms) / np.mean(sur_ms)),
        "surrogate_meets_rmse": bool(max(sur_rmse) <= 0.02),
        "clocks": clk.summary(),
        **({"cpu_baseline": cpu} if cpu else {}),
    }


def run_surrogate(args):
    import torch
    import rn_ao as rn
    torch.cuda.set_device(0)
    rn.init()
    r = surrogate_headtohead(args.steps, args.warmup, args.views or 16)
    out = {"metric": METRIC, "value": r["surrogate"]["ms_per_frame"], "unit": "ms/frame (surrogate)", "n_gpus": 1,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["surrogate"]["ms_per_frame"],
           "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "bf16 network, f32 trace",
           "data": "synthetic", "config": {"workload": r.pop("workload"), "views": r["views"]}, **r}
    print(json.dumps(out), flush=True)


def run_hybrid(args):
    """The closest-hit consumers: the hybrid pass (a sun shadow ray and a mirror reflection ray
    per covered pixel, rn_hybrid) on 3840x2160 views of the built-in scene and of the seeded
    7.88M-triangle scene, G-buffers resident; and rn_closest on the reflection rays of the
    first large view (the same rays as a flat list). Timed per frame with CUDA events."""
    import numpy as np
    import torch
    import rn_ao as rn
    import scene as scenes
    torch.cuda.set_device(0)
    rn.init()
    stream = torch.cuda.current_stream()

    def timed(fn):
        for _ in range(max(3, args.warmup)):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / args.steps

    W, H = 3840, 2160
    out = {"metric": "hybrid shadow + reflection rays per second", "unit": "G rays/s", "n_gpus": 1,
           "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32", "data": "synthetic", "scenes": []}
    with Clocks(0) as clk:
        for name, sc, views in (("built-in scene (14 triangles)", scenes.build_test_scene(), None),
                                ("seeded 7.88M-triangle scene", scenes.build_synthetic_scene(5, 10000, 6000), 4)):
            tris, nrms = torch.from_numpy(sc.tris).cuda(), torch.from_numpy(sc.normals).cuda()
            acc = rn.LinearAccel(tris)
            cams = [sc.camera] if views is None else [v[3] for v in scenes.orbit_views(5, views)]
            ms, rays = [], 0
            for cam in cams:
                g = rn.rasterize(tris, nrms, cam, W, H)
                eye = cam[:3]
                ms.append(timed(lambda: rn.hybrid(g, acc, eye, sc.to_light)))
                lit, tri, _ = rn.hybrid(g, acc, eye, sc.to_light)
                rays += 2 * int(g.mask.sum().item())
                cov = g.mask != 0
                shadowed = float((lit[cov] == 0).float().mean().item())
                reflected = float((tri[cov] >= 0).float().mean().item())
            row = {"scene": name, "views": len(cams), "ms_per_frame": float(np.mean(ms)),
                   "grays_per_s": rays / (sum(ms) * 1e-3) / 1e9, "shadowed_fraction_last_view": shadowed,
                   "reflected_fraction_last_view": reflected}
            if views is not None:
                # the last view's reflection rays as a flat list through rn_closest
                pos, nrm = g.position.reshape(-1, 3), g.normal.reshape(-1, 3)
                keep = g.mask.reshape(-1) != 0
                p, n = pos[keep], nrm[keep]
                d = torch.nn.functional.normalize(p - torch.tensor(eye, device="cuda"), dim=1)
                n = torch.where(((n * d).sum(1, keepdim=True) > 0), -n, n)
                r = d - n * (2 * (d * n).sum(1, keepdim=True))
                rays6 = torch.cat([p + n * 1e-3, r], 1).contiguous()
                tmax = torch.full((len(rays6),), 1e30, device="cuda")
                cms = timed(lambda: rn.closest(acc, rays6, tmax))
                row["closest"] = {"rays": len(rays6), "ms": cms, "grays_per_s": len(rays6) / (cms * 1e-3) / 1e9}
            out["scenes"].append(row)
    big = out["scenes"][-1]
    out.update(value=big["grays_per_s"], ms_per_step=big["ms_per_frame"], clocks=clk.summary(),
               config={"workload": "hybrid pass, 3840x2160, seeded 7.88M-triangle scene, 4 orbit views",
                       "inputs": "G-buffers resident in HBM (64 MB per view with its outputs)"})
    print(json.dumps(out), flush=True)


def run_build(args):
    print(json.dumps(build_report(args)), flush=True)


def build_report(args) -> dict:
    """The accelerator build (rn_accel_build: PLOC on the GPU, then the collapse to 4-wide
    nodes) from device-resident triangles: the 7.88M-triangle and 744k-triangle seeded scenes,
    a 1M-triangle random soup and the reference's 20,000-triangle PLOC check soup. Each build is timed with CUDA events around the call (it
    ends with a stream synchronize), device allocations included."""
    import numpy as np
    import torch
    import rn_ao as rn
    import scene as scenes
    torch.cuda.set_device(0)
    rn.init()
    stream = torch.cuda.current_stream()
    rng = np.random.default_rng(1)
    c = rng.uniform(-50, 50, (1000000, 1, 3)).astype(np.float32)
    soup = (c + rng.uniform(-1, 1, (1000000, 3, 3)).astype(np.float32)).reshape(-1, 9)
    cases = (("seeded 7.88M-triangle scene", scenes.build_synthetic_scene(5, 10000, 6000).tris),
             ("seeded 744k-triangle scene", scenes.build_synthetic_scene(1, 2000, 500).tris),
             ("1M-triangle random soup", soup),
             ("rt::soup(20000, 7), the reference's PLOC evidence input", scenes.soup(20000, 7)))
    out = {"metric": "accelerator build rate", "unit": "M triangles/s", "n_gpus": 1, "steps": args.steps,
           "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32 boxes, u32 codes", "data": "synthetic", "builds": []}
    with Clocks(0) as clk:
        for name, tris in cases:
            t = torch.from_numpy(np.ascontiguousarray(tris)).cuda()
            for _ in range(max(1, args.warmup)):
                rn.LinearAccel(t).close()
            ms = []
            for _ in range(args.steps):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                acc = rn.LinearAccel(t)
                e1.record(stream)
                torch.cuda.synchronize()
                ms.append(e0.elapsed_time(e1))
                info = acc.info()
                acc.close()
            n = len(tris)
            out["builds"].append({"input": name, "triangles": n, "ms_per_build": float(np.median(ms)),
                                  "mtris_per_s": n / (float(np.median(ms)) * 1e-3) / 1e6, **info})
    big = out["builds"][0]
    out.update(value=big["mtris_per_s"], ms_per_step=big["ms_per_build"], clocks=clk.summary(),
               config={"workload": "accelerator build, seeded 7.88M-triangle scene (median of the timed builds)",
                       "inputs": "triangles resident in HBM (284 MB, larger than L2)"})
    return out


def pt_fixture_scene(key: str):
    """A lit scene of the reference's path tracer from tests/golden/pt_scenes.npz (made by the
    reference's own scene builders): (scene dict, camera)."""
    import numpy as np
    z = np.load(os.path.join(ROOT, "tests", "golden", "pt_scenes.npz"))
    sc = {k.split("/", 1)[1]: z[k] for k in z.files if k.startswith(key + "/")}
    cam = sc.pop("camera")
    return sc, cam


def run_pathtrace(args):
    print(json.dumps(pathtrace_report(args)), flush=True)


def pathtrace_report(args, spp: int = 64) -> dict:
    """The path tracer (rn_pathtrace, interface v4): retro_room (the reference's lit room: sun
    through the open end, a ceiling lamp, textured brick, tile, plank and brass) and iso_street
    at 1920 x 1080, 64 spp, 64 bounces with Russian roulette, every AOV (the frame the reference
    times its own GPU path tracer on: docs/rt-interface-v4.md:36-40); timed per frame with CUDA
    events, outputs in HBM. The CPU baseline is the oracle (a restatement of raw::rt::pathTraceCpu,
    bit-identical to the reference build) on the host's cores, on the same frame at 4 spp.
    Metric: path samples per second."""
    import torch
    import rn_ao as rn
    torch.cuda.set_device(0)
    rn.init()
    stream = torch.cuda.current_stream()
    W, H, SPPS = 1920, 1080, spp
    out = {"metric": "path-traced samples per second (interface v4, every AOV)", "unit": "M samples/s",
           "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32", "data": "synthetic: the reference's own lit scenes", "scenes": []}
    with Clocks(0) as clk:
        for key in ("retro_room", "iso_street"):
            sc, cam = pt_fixture_scene(key)
            s = rn.PtScene(sc)
            d = dict(seed=1, spp=SPPS, width=W, height=H, camera=[float(v) for v in cam])
            for _ in range(max(1, args.warmup)):
                o = rn.path_trace(s, d, device=True)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(args.steps):
                o = rn.path_trace(s, d, device=True)
            e1.record(stream)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / args.steps
            row = {"scene": key, "width": W, "height": H, "spp": SPPS, "ms_per_frame": ms,
                   "msamples_per_s": W * H * SPPS / (ms * 1e-3) / 1e6, "emitters": s.info()["emitters"],
                   "radiance_mean": float(o["radiance"].mean().item())}
            if not os.environ.get("RN_BENCH_NO_CPU"):
                from oracle import oracle as O
                # the same frame at 4 of the 64 samples: a bounded CPU sample of the same work
                dd = dict(d, spp=4)
                t0 = time.perf_counter()
                O.pathtrace(sc, dd, threads=os.cpu_count() or 1)
                dt = time.perf_counter() - t0
                row["cpu_baseline"] = {"value": W * H * 4 / dt / 1e6, "unit": "M samples/s", "cores": os.cpu_count() or 1,
                                       "kind": "port", "sample": "the same %dx%d frame at 4 spp (%.1f s), oracle "
                                       "restatement of pathTraceCpu, all host threads" % (W, H, dt)}
            if key == "retro_room" and SPPS == 64:
                # context only (other hardware and API, one run): the reference's GPU path tracer
                row["reference_gpu_context"] = {"ms_per_frame": 1638.0, "msamples_per_s": W * H * 64 / 1.638 / 1e6,
                                                "hardware": "RTX 4090, D3D12 (WGSL), interface v4",
                                                "source": "docs/rt-interface-v4.md:38-39"}
            out["scenes"].append(row)
            s.close()
    first = out["scenes"][0]
    out.update(value=first["msamples_per_s"], ms_per_step=first["ms_per_frame"], clocks=clk.summary(),
               config={"workload": "path tracer, retro_room at %dx%d, %d spp, 64 bounces (Russian roulette)" % (W, H, SPPS),
                       "outputs": "every AOV in HBM"}, gpu_launches=2 * args.steps)
    return out


def main():
    args = parse()
    if args.workload == "pathtrace":
        run_pathtrace(args)
        return
    if args.workload == "build":
        run_build(args)
        return
    if args.workload == "hybrid":
        run_hybrid(args)
        return
    if args.workload == "surrogate" and not args.profile:
        run_surrogate(args)
        return
    if args.workload != "4k" and not args.profile:
        run_views(args)
        return
    if args.profile:
        run_profile(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
