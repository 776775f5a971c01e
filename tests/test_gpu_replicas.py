"""A frame split into row bands, the bands run one after another on this GPU as the ranks
of a multi-GPU job would run them: the bands' traced and SSAO pixels are the whole frame's,
and the reconcile combined from the bands' parts has the whole frame's pixels, maximum and
RMSE (and so its verdict)."""
import pytest

import replicas

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("world", [2, 3])
def test_row_bands_reproduce_the_frame(rn, world):
    import torch
    import scene as scenes
    sc = scenes.build_test_scene()
    tris, nrms = torch.from_numpy(sc.tris).cuda(), torch.from_numpy(sc.normals).cuda()
    g = rn.rasterize(tris, nrms, sc.camera, 301, 203)
    acc = rn.LinearAccel(tris)
    whole = rn.ao_frame(g, acc, 32, 2.0, 24, 0.12, to_light=sc.to_light)
    parts = []
    for r in range(world):
        out, part = replicas.band_frame(g, acc, r, world, 32, 2.0, 24, 0.12, to_light=sc.to_light)
        y0, y1 = out["rows"]
        for k in ("ao", "sky", "sun", "ss"):
            assert bool((out[k][y0:y1] == whole[k][y0:y1]).all()), (r, k)
        parts.append(part)
    c = replicas.combine_reconcile(parts, 0.12)
    rec = whole["rec"]
    assert c.pixels == rec.pixels and c.max_error == rec.max_error
    assert c.rmse == rec.rmse and c.within_tolerance == rec.within_tolerance
    assert abs(c.sum_sq - rec.sum_sq) <= 1e-10 * rec.sum_sq
