"""The whole frame on the GPU (rn_render_frame, raw::renderWithParams): against the
reference's committed golden SHA-256 of frame.ppm, frame_hdr.pfm and the AO outputs on the
CLI cases, and plane by plane against the oracle (albedo, motion under a moving camera,
lighting model 1, no ray-traced pass). Every plane must be bit-identical, so the
GPU-versus-CPU comparison of raw-gpu-cert/1 (src/renderer/gpu_reconcile.cpp:62-101, with the
bounds of raw/cert/gpu_tolerance.hpp) verifies with zero error."""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "identity.json")))["cases"]
SMALL = [k for k, c in sorted(GOLD.items()) if c["width"] * c["height"] <= 512 * 512]


def _scene(oracle):
    tris, nrm9, light = oracle.test_scene()
    return tris, nrm9, oracle.test_scene_albedo(), light


@pytest.mark.parametrize("case", SMALL)
def test_frame_matches_reference_goldens(rn, oracle, case):
    c = GOLD[case]
    tris, nrm9, alb, light = _scene(oracle)
    f = rn.render_frame(tris, nrm9, alb, c["camera"], c["width"], c["height"], light=(light, 1.0))
    assert oracle.sha256(oracle.ppm_bytes(f["frame"])) == c["frame_files"]["frame.ppm"]
    assert oracle.sha256(oracle.pfm3_bytes(f["hdr"])) == c["frame_files"]["frame_hdr.pfm"]
    assert oracle.sha256(oracle.pfm1_bytes(f["ao_rt"])) == c["files"]["ao_rt.pfm"]
    assert oracle.sha256(oracle.pfm1_bytes(f["ao_ss"])) == c["files"]["ao_ss.pfm"]
    assert oracle.sha256(oracle.mask_pgm_bytes(f["mask"])) == c["files"]["mask.pgm"]
    assert oracle.sha256(oracle.pgm_bytes(f["error_map"])) == c["files"]["ao_error.pgm"]
    ex = c["exact"]
    assert f["rec"].pixels == ex["pixels"] and abs(f["rec"].rmse - ex["rmse"]) <= 1e-6 * ex["rmse"]
    assert f["rec"].within_tolerance == ex["within"]
    assert f["motion_valid"] == f["motion_total"] == ex["pixels"]          # a static frame
    assert not f["motion"].any()


def _cpu_frame(oracle, cam, prev_cam, w, h, model=2, rtao=True):
    tris, nrm9, alb, light = _scene(oracle)
    depth, pos, nrm, mask, tri = oracle.rasterize_ex(tris, nrm9, cam, w, h)
    albedo = np.where(mask[..., None] > 0, alb[np.maximum(tri, 0)], 0).astype(np.float32)
    if rtao:
        ao, sky, sun = oracle.trace(pos, nrm, mask, tris, 64, 2.0, to_light=-light, threads=os.cpu_count() or 1)
    ss = oracle.ssao(pos, nrm, mask, 24, 2.0, os.cpu_count() or 1)
    if model == 2:
        frame, hdr = oracle.shade(nrm, albedo, mask, 2, sky, sun, light, 1.0)
    else:
        frame, hdr = oracle.shade(nrm, albedo, mask, 1, ao if rtao else ss, None, light, 1.0)
    vp = oracle.view_proj(cam, w, h)
    pv = oracle.view_proj(prev_cam, w, h) if prev_cam is not None else vp
    mot, valid = oracle.motion(pos, mask, vp, pv)
    return dict(depth=depth, position=pos, normal=nrm, mask=mask, albedo=albedo, ao_ss=ss, frame=frame, hdr=hdr,
                motion=mot, valid=valid, pv=pv, **(dict(ao_rt=ao) if rtao else {}))


def _gpu_cpu_channels(g, c):
    """raw::reconcileGpuCpu's channel RMSEs (gpu_reconcile.cpp:69-96) over pixels both cover."""
    both = (g["mask"] > 0) & (c["mask"] > 0)
    mismatch = int(((g["mask"] > 0) != (c["mask"] > 0)).sum())
    d = c["depth"][both]
    r = {"depth_rel": (g["depth"][both] - d) / np.where(np.abs(d) > 1e-6, d, 1.0)}
    for k in ("position", "normal", "motion", "frame"):
        r[k] = (g[k][both] - c[k][both]).ravel()
    r["ao_ss"] = g["ao_ss"][both] - c["ao_ss"][both]
    if "ao_rt" in c:
        r["ao_rt"] = g["ao_rt"][both] - c["ao_rt"][both]
    rmse = {k: float(np.sqrt(np.mean(v.astype(np.float64) ** 2))) for k, v in r.items()}
    return rmse, mismatch


BOUNDS = {"depth_rel": 1e-4, "position": 1e-3, "normal": 1e-3, "motion": 1e-4, "ao_ss": 0.01, "ao_rt": 0.01,
          "frame": 0.01}


@pytest.mark.parametrize("model,rtao", [(2, True), (1, True), (1, False)])
def test_frame_planes_equal_the_oracle_with_motion(rn, oracle, model, rtao):
    cam = (4.0, 4.0, 6.0, 0.0, 1.0, 0.0, 0.0, 1.0, 0.0, 0.9)
    prev = (4.3, 3.8, 5.7, 0.0, 1.0, 0.0, 0.0, 1.0, 0.0, 0.9)
    w, h = 301, 203
    cpu = _cpu_frame(oracle, cam, prev, w, h, model, rtao)
    tris, nrm9, alb, light = _scene(oracle)
    g = rn.render_frame(tris, nrm9, alb, cam, w, h, light=(light, 1.0), prev_view_proj=cpu["pv"], rtao=rtao,
                        lighting=model)
    for k in ("depth", "position", "normal", "mask", "albedo", "ao_ss", "frame", "hdr", "motion") + (("ao_rt",) if rtao else ()):
        assert np.array_equal(g[k], cpu[k]), k
    assert g["motion_valid"] == cpu["valid"] and g["motion_total"] == int(cpu["mask"].sum())
    assert np.abs(g["motion"]).max() > 0.01
    rmse, mismatch = _gpu_cpu_channels(g, cpu)
    assert mismatch == 0 and all(v == 0.0 for v in rmse.values()), rmse
    assert all(rmse[k] <= BOUNDS[k] for k in rmse)
    if not rtao:
        assert g["rec"].pixels == 0 and not g["error_map"].any()


def test_frame_device_pointers_and_light_defaults(rn, oracle):
    import torch
    tris, nrm9, alb, light = _scene(oracle)
    cam = (4.0, 4.0, 6.0, 0.0, 1.0, 0.0, 0.0, 1.0, 0.0, 0.9)
    host = rn.render_frame(tris, nrm9, alb, cam, 160, 120, light=(light, 1.0), spp=16)
    dev = rn.render_frame(torch.from_numpy(tris).cuda(), torch.from_numpy(nrm9).cuda(), torch.from_numpy(alb).cuda(),
                          cam, 160, 120, light=(light, 1.0), spp=16)
    torch.cuda.synchronize()
    for k in ("frame", "hdr", "ao_rt", "sky", "sun", "albedo", "mask"):
        assert np.array_equal(dev[k].cpu().numpy(), host[k]), k
    nolight = rn.render_frame(tris, nrm9, alb, cam, 160, 120, spp=16)     # the (0,-1,0), 1 default light
    assert not np.array_equal(nolight["frame"], host["frame"])
    with pytest.raises(rn.RnError):
        rn.render_frame(tris, nrm9, alb, cam, 0, 120)
