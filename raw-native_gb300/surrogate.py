"""The learned AO surrogate around the U-Net (rn_ao.UNet): training data from the GPU
oracle, training, inference and the ray-traced fallback.

Inputs per pixel (5 channels): view depth normalised by the AO radius (relative to the mean
depth of the image's covered pixels, clamped to +-8), the world normal, and the 4-spp traced
AO; uncovered pixels carry depth 0, normal 0 and AO 1. Target: the 1024-spp traced AO. The
4 samples of the input are the first 4 of the target's sequence (the sampler has no frame
seed), as the traced oracle defines them.

Fallback: the frame is cut into 16 x 16 tiles; where the prediction's tile mean leaves the
band mean(ao4) +- k * sigma (sigma = the 4-spp estimate's standard error over the tile's
covered pixels, at least 0.5 / sqrt(4 n)), the tile is re-traced at full spp and the traced
values replace the prediction there.
"""
from __future__ import annotations

import dataclasses
import hashlib
import json
import time

import numpy as np

import rn_ao as rn
import scene as scenes

RADIUS = 1.0
TILE = 16


def features(g, depth, ao4, radius: float = RADIUS):
    """(H, W, 5) float32 CUDA features of a G-buffer, its depth and a 4-spp AO image."""
    import torch
    m = g.mask.bool()
    d = torch.where(m, depth, torch.zeros_like(depth))
    mean = d[m].mean() if bool(m.any()) else torch.tensor(0.0, device=d.device)
    f = torch.zeros(*g.mask.shape, 5, device=g.mask.device)
    f[..., 0] = torch.where(m, ((depth - mean) / radius).clamp(-8, 8), torch.zeros_like(depth))
    f[..., 1:4] = torch.where(m[..., None], g.normal, torch.zeros_like(g.normal))
    f[..., 4] = torch.where(m, ao4, torch.ones_like(ao4))
    return f.contiguous()


def render_view(tris, nrms, acc, cam, w, h, spps=(4, 1024), radius=RADIUS):
    """G-buffer, depth and traced AO at each spp of `spps` for one view (CUDA tensors)."""
    g, depth = rn.rasterize(tris, nrms, cam, w, h, want_depth=True)
    aos = [rn.compute_rtao(g, acc, s, radius) for s in spps]
    return g, depth, aos


@dataclasses.dataclass
class Dataset:
    x: object          # [N, 128, 128, 5]
    y: object          # [N, 128, 128]
    manifest: dict

    @property
    def digest(self) -> str:
        return hashlib.sha256(json.dumps(self.manifest, sort_keys=True).encode()).hexdigest()[:16]


def generate_dataset(n_seeds: int, seed0: int = 1000, view: int = 512, crop: int = 128, n_boxes: int = 200,
                     n_spheres: int = 50, spp_in: int = 4, spp_target: int = 1024, log=None) -> Dataset:
    """Crops of (features, 1024-spp AO) from one orbit view of each training scene (seeds
    seed0 .. seed0 + n_seeds - 1), every crop x crop tile of a view x view render."""
    import torch
    xs, ys = [], []
    t0 = time.time()
    for k in range(n_seeds):
        sd = seed0 + k
        sc = scenes.build_synthetic_scene(sd, n_boxes, n_spheres)
        tris = torch.from_numpy(sc.tris).cuda()
        nrms = torch.from_numpy(sc.normals).cuda()
        acc = rn.LinearAccel(tris)
        _, _, _, cam = scenes.orbit_views(sd, 8)[sd % 8]
        g, depth, (ao4, ao_t) = render_view(tris, nrms, acc, cam, view, view, (spp_in, spp_target))
        f = features(g, depth, ao4)
        for yy in range(0, view, crop):
            for xx in range(0, view, crop):
                xs.append(f[yy:yy + crop, xx:xx + crop].clone())
                ys.append(ao_t[yy:yy + crop, xx:xx + crop].clone())
        acc.close()
        if log and (k + 1) % max(1, n_seeds // 10) == 0:
            log("data: %d/%d scenes, %.1f s" % (k + 1, n_seeds, time.time() - t0))
    x = torch.stack(xs).contiguous()
    y = torch.stack(ys).contiguous()
    return Dataset(x, y, dict(seeds=[seed0, seed0 + n_seeds], view=view, crop=crop, boxes=n_boxes, spheres=n_spheres,
                              spp_in=spp_in, spp_target=spp_target, radius=RADIUS, crops=int(x.shape[0])))


def train(net, data: Dataset, steps: int, batch: int = 64, lr: float = 1e-3, seed: int = 0, log=None, log_every=500):
    """Adam on the MSE for `steps` mini-batches drawn with a seeded permutation."""
    import torch
    gen = torch.Generator(device="cuda").manual_seed(seed)
    n = data.x.shape[0]
    losses = []
    t0 = time.time()
    perm = torch.randperm(n, device="cuda", generator=gen)
    pos = 0
    for step in range(steps):
        if pos + batch > n:
            perm = torch.randperm(n, device="cuda", generator=gen)
            pos = 0
        idx = perm[pos:pos + batch]
        pos += batch
        loss = net.train_step(data.x[idx].contiguous(), data.y[idx].contiguous(), lr)
        losses.append(loss)
        if log and (step + 1) % log_every == 0:
            log("train: step %d loss %.5f (%.1f s)" % (step + 1, float(np.mean(losses[-log_every:])), time.time() - t0))
    return losses


def pad16(t, value=0.0):
    """Pad an (H, W[, C]) tensor at the bottom/right to multiples of 16."""
    import torch.nn.functional as F
    h, w = t.shape[:2]
    ph, pw = (-h) % 16, (-w) % 16
    if not ph and not pw:
        return t
    if t.dim() == 3:
        return F.pad(t.permute(2, 0, 1), (0, pw, 0, ph), value=value).permute(1, 2, 0).contiguous()
    return F.pad(t, (0, pw, 0, ph), value=value).contiguous()


def predict(net, f):
    """The network's AO for one (H, W, 5) feature image (net created for the padded size)."""
    h, w = f.shape[:2]
    out = net.forward(pad16(f)[None].contiguous())
    return out[0, :h, :w]


def fallback_tiles(pred, ao4, mask, spp_in: int = 4, k: float = 3.0, tile: int = TILE):
    """Boolean (ceil(H/tile), ceil(W/tile)) map of the tiles to re-trace at full spp."""
    import torch
    import torch.nn.functional as F
    m = mask.float()
    h, w = m.shape
    ph, pw = (-h) % tile, (-w) % tile
    pad = lambda t: F.pad(t[None, None], (0, pw, 0, ph))
    cnt = F.avg_pool2d(pad(m), tile) * tile * tile
    sp = F.avg_pool2d(pad(pred * m), tile) * tile * tile
    s4 = F.avg_pool2d(pad(ao4 * m), tile) * tile * tile
    v4 = F.avg_pool2d(pad(ao4 * (1 - ao4) * m), tile) * tile * tile
    n = cnt.clamp(min=1)
    sigma = torch.sqrt(torch.clamp(v4 / n, min=0) / spp_in / n).clamp(min=0.5 / torch.sqrt(spp_in * n))
    dev = (sp / n - s4 / n).abs()
    return ((dev > k * sigma) & (cnt > 0))[0, 0]


def tiles_to_pixels(tiles, h, w, tile: int = TILE):
    import torch
    return tiles.repeat_interleave(tile, 0).repeat_interleave(tile, 1)[:h, :w]


def surrogate_frame(net, g, depth, acc, spp_full: int, radius: float = RADIUS, k: float = 3.0):
    """The surrogate's AO for one frame: 4-spp trace, network, fallback tiles re-traced at
    spp_full. Returns (ao, fallback tile fraction, ao4)."""
    import torch
    ao4 = rn.compute_rtao(g, acc, 4, radius)
    pred = predict(net, features(g, depth, ao4, radius))
    tiles = fallback_tiles(pred, ao4, g.mask, 4, k)
    fb = tiles_to_pixels(tiles, *g.mask.shape) & g.mask.bool()
    out = torch.where(g.mask.bool(), pred, torch.ones_like(pred))
    if bool(fb.any()):
        sub = rn.GBuffer(g.position, g.normal, (fb).to(torch.uint8).contiguous())
        traced = rn.compute_rtao(sub, acc, spp_full, radius)
        out = torch.where(fb, traced, out)
    covered_tiles = int((tiles_to_pixels(torch.ones_like(tiles), *g.mask.shape) & g.mask.bool()).any())
    frac = float(tiles.float().sum() / max(1, int(tiles.numel())))
    return out, frac, ao4


def rmse(a, b, mask):
    import torch
    m = mask.bool()
    return float(torch.sqrt(((a - b)[m] ** 2).mean())) if bool(m.any()) else 0.0


def checkpoint(net, path: str, step: int, seed: int, data: Dataset, extra=None):
    """Weights with step, seed and the data manifest's digest (npz)."""
    np.savez_compressed(path, params=net.get_params(), step=step, seed=seed, data_digest=data.digest,
                        manifest=json.dumps(data.manifest), extra=json.dumps(extra or {}))


def load_checkpoint(net, path: str) -> dict:
    z = np.load(path, allow_pickle=False)
    net.set_params(z["params"])
    return dict(step=int(z["step"]), seed=int(z["seed"]), data_digest=str(z["data_digest"]))
