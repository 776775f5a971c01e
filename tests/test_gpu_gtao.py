"""GTAO on the GPU (rn_gtao) against the oracle's FP64 restatement of raw::post::gtao, under
the reference's own parity rule for its GPU pass: |gpu - cpu| <= 1e-3 on all but 0.1 % of
pixels (raw/renderer/post_parity.hpp:15-19); and GTAO judged by the traced AO (1024 spp,
radius 0.5) with the bounds of the reference's evidence: mean |difference| <= 0.05 and 95th
percentile <= 0.15 over pixels at least 8 from the border. On the near camera, where more
than 2,000 of those pixels are occluded (the evidence's coverage bound), a control
(visibility 1 everywhere) must fail the same bounds; from the CLI camera the scene has too
little occlusion (about 1,960 pixels) for the control to mean anything."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CAMERAS = {"test_scene": (4.0, 4.0, 6.0, 0.0, 1.0, 0.0, 0.0, 1.0, 0.0, 0.9),
           "near": (1.8, 3.2, 2.4, 0.8, 0.2, 1.0, 0.0, 1.0, 0.0, 0.9)}


def _gbuffer(oracle, cam, w, h):
    tris, nrm9, _ = oracle.test_scene()
    _, pos, nrm, mask = oracle.rasterize(tris, nrm9, cam, w, h)
    return tris, pos, nrm, mask


@pytest.mark.parametrize("name", sorted(CAMERAS))
@pytest.mark.parametrize("size", [(256, 256), (320, 200)])
def test_gtao_parity_with_the_oracle(rn, oracle, name, size):
    cam = CAMERAS[name]
    w, h = size
    _, pos, nrm, mask = _gbuffer(oracle, cam, w, h)
    g = rn.GBuffer(pos, nrm, mask)
    got = rn.gtao(g, cam)
    vp, vn, vd = oracle.view_gbuffer(pos, nrm, mask, cam)
    want = oracle.gtao(vp, vn, vd, cam[9])
    d = np.abs(got.astype(np.float64) - want)
    assert bool((got[mask == 0] == 1.0).all())
    assert (d > 1e-3).sum() <= 1e-3 * mask.sum(), (int((d > 1e-3).sum()), float(d.max()))


def test_gtao_judged_by_the_traced_ao(rn, oracle):
    import torch
    for name, cam in CAMERAS.items():
        tris, pos, nrm, mask = _gbuffer(oracle, cam, 256, 256)
        g = rn.GBuffer(pos, nrm, mask)
        a = rn.gtao(g, cam)
        acc = rn.LinearAccel(tris)
        ref = rn.compute_rtao(g, acc, 1024, 0.5)
        inner = np.zeros_like(mask, dtype=bool)
        inner[8:248, 8:248] = True
        sel = inner & (mask > 0)
        d = np.abs(a - ref)[sel]
        ctl = np.abs(1.0 - ref)[sel]
        assert d.mean() <= 0.05 and np.percentile(d, 95) <= 0.15, (name, d.mean(), np.percentile(d, 95))
        if name == "near":
            assert (ref[sel] < 0.9).sum() >= 2000                                   # coverage
            assert not (ctl.mean() <= 0.05 and np.percentile(ctl, 95) <= 0.15)      # the control fails
        rec = rn.reconcile(a, ref, mask, 0.12, error_map=False)
        assert rec.pixels == int(mask.sum()) and rec.rmse > 0
