"""The learned AO surrogate around the U-Net (rn_ao.UNet): training data rendered by the GPU
ray-traced oracle, training, inference, and the ray-traced fallback on 16 x 16 tiles.

Inputs per pixel (5 channels): view depth over the AO radius, taken relative to the mean depth
of the frame's covered pixels, clamped to +-32 and scaled by 1/8; the world normal; and the
4-spp traced AO. Uncovered pixels carry depth 0, normal 0 and AO 1. Target: the 1024-spp
traced AO (uncovered pixels 1). The traced sampler hash01(x, y, s) has no frame or view seed,
so the 4 input samples of a pixel are the first 4 of its 1024-sample target sequence, and
every view of a pixel position draws the same sequence.

Fallback: the frame is cut into 16 x 16 tiles. Where the prediction's tile mean leaves the
band mean(ao4) +- k sigma, with sigma the standard error of the tile's 4-spp mean
(sqrt(sum p(1-p) / 4) / n over its n covered pixels, at least 0.5 / sqrt(4 n)), the tile is
traced at the full spp and the traced values replace the prediction there.

Command line (one GPU):
  python surrogate.py train --out DIR [--seeds 2000 --crops 20000 --steps 20000 ...]
  python surrogate.py eval --ckpt FILE [--seeds 200 ...]
Data-parallel training on N GPUs of one node (each rank renders the same crops from the same
seeds, takes its share of every step's N x batch crops, and the ranks average their
gradients with one NCCL all-reduce per step; rank 0 writes the files):
  python -m torch.distributed.run --nproc-per-node N --master-addr 127.0.0.1 surrogate.py train --out DIR
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import dataclasses
import hashlib
import json
import os
import sys
import time

import numpy as np

import rn_ao as rn
import scene as scenes

RADIUS = 1.0
TILE = 16
SPP_IN = 4
SPP_TARGET = 1024
TRAIN_SEED0 = 1000            # training scenes: seeds 1000 .. 1000 + n - 1
EVAL_SEED0 = 900000           # held-out scenes: seeds 900000 .. 900000 + n - 1
SCENE_BOXES, SCENE_SPHERES = 200, 50
VIEW_W, VIEW_H = 1920, 1080
CROP = 128


def camera_for(seed: int):
    """The orbit camera a scene seed is viewed from."""
    return scenes.orbit_views(seed, 8)[seed % 8][3]


def features(g, depth, ao4, radius: float = RADIUS):
    """(H, W, 5) float32 CUDA features of a G-buffer, its depth and a 4-spp AO image."""
    import torch
    m = g.mask.bool()
    # the covered pixels' mean depth, summed in FP64 and rounded to FP32 (as rn_surrogate_ao)
    mean = (depth[m].double().sum() / m.sum()).float() if bool(m.any()) else torch.zeros((), device=depth.device)
    f = torch.zeros(*g.mask.shape, 5, device=g.mask.device)
    f[..., 0] = torch.where(m, ((depth - mean) / radius).clamp(-32, 32) * 0.125, torch.zeros_like(depth))
    f[..., 1:4] = torch.where(m[..., None], g.normal, torch.zeros_like(g.normal))
    f[..., 4] = torch.where(m, ao4, torch.ones_like(ao4))
    return f.contiguous()


def masked_trace(g, acc, spp: int, pixel_mask, radius: float = RADIUS):
    """Traced AO over the pixels of `pixel_mask` & coverage (1 elsewhere); frame coordinates
    keep each pixel's own sample sequence."""
    import torch
    sub = rn.GBuffer(g.position, g.normal, (g.mask.bool() & pixel_mask).to(torch.uint8).contiguous())
    return rn.compute_rtao(sub, acc, spp, radius)


def scene_counts(seed: int, density: str):
    """(boxes, spheres) of a training or evaluation scene. "fixed": 200 and 50 (146,400
    triangles). "mixed": each drawn log-uniformly per seed, boxes in [200, 10000] and spheres
    in [50, 6000], from the sparse scenes up to the density of the 7.88M-triangle scene."""
    if density == "fixed":
        return SCENE_BOXES, SCENE_SPHERES
    if density != "mixed":
        raise ValueError("density %r" % density)
    rng = np.random.Generator(np.random.PCG64(seed ^ 0xD3))
    b = int(round(np.exp(rng.uniform(np.log(200.0), np.log(10000.0)))))
    s = int(round(np.exp(rng.uniform(np.log(50.0), np.log(6000.0)))))
    return b, s


class SceneSource:
    """Seeded scenes built on host threads, at most `ahead` of them ahead of their use."""

    def __init__(self, seeds, density: str = "fixed", workers: int = 8, ahead: int = 16):
        self.seeds, self.density, self.workers, self.ahead = list(seeds), density, workers, ahead

    def _build(self, seed):
        b, s = scene_counts(seed, self.density)
        return scenes.build_synthetic_scene(seed, b, s)

    def __iter__(self):
        import collections
        with cf.ThreadPoolExecutor(self.workers) as pool:
            pending = collections.deque()
            it = iter(self.seeds)
            for sd in it:
                pending.append((sd, pool.submit(self._build, sd)))
                if len(pending) >= self.ahead:
                    break
            while pending:
                sd, f = pending.popleft()
                nxt = next(it, None)
                if nxt is not None:
                    pending.append((nxt, pool.submit(self._build, nxt)))
                yield sd, f.result()


@dataclasses.dataclass
class Dataset:
    x: object          # [N, CROP, CROP, 5] float32 CUDA
    y: object          # [N, CROP, CROP] float32 CUDA
    manifest: dict

    @property
    def digest(self) -> str:
        return hashlib.sha256(json.dumps(self.manifest, sort_keys=True).encode()).hexdigest()[:16]


def generate_dataset(n_seeds: int, n_crops: int, seed0: int = TRAIN_SEED0, log=print, density: str = "fixed") -> Dataset:
    """n_crops random CROP x CROP crops, spread evenly over n_seeds scenes (one 1920 x 1080
    orbit view each): features from the 4-spp trace, target from the 1024-spp trace, both
    traced only inside the crops."""
    import torch
    per = -(-n_crops // n_seeds)
    xs = torch.empty(n_seeds * per, CROP, CROP, 5, device="cuda")
    ys = torch.empty(n_seeds * per, CROP, CROP, device="cuda")
    k = 0
    t0 = time.time()
    for i, (sd, sc) in enumerate(SceneSource(range(seed0, seed0 + n_seeds), density)):
        tris = torch.from_numpy(sc.tris).cuda()
        nrms = torch.from_numpy(sc.normals).cuda()
        acc = rn.LinearAccel(tris)
        g, depth = rn.rasterize(tris, nrms, camera_for(sd), VIEW_W, VIEW_H, want_depth=True)
        rng = np.random.Generator(np.random.PCG64(sd ^ 0xC409))
        ys0 = rng.integers(0, VIEW_H - CROP + 1, per)
        xs0 = rng.integers(0, VIEW_W - CROP + 1, per)
        sel = torch.zeros(VIEW_H, VIEW_W, dtype=torch.bool, device="cuda")
        for y0, x0 in zip(ys0, xs0):
            sel[y0:y0 + CROP, x0:x0 + CROP] = True
        ao4 = masked_trace(g, acc, SPP_IN, sel)
        aot = masked_trace(g, acc, SPP_TARGET, sel)
        f = features(g, depth, ao4)
        for y0, x0 in zip(ys0, xs0):
            xs[k] = f[y0:y0 + CROP, x0:x0 + CROP]
            ys[k] = aot[y0:y0 + CROP, x0:x0 + CROP]
            k += 1
        acc.close()
        if log and (i + 1) % max(1, n_seeds // 10) == 0:
            log("data: %d/%d scenes, %d crops, %.1f s" % (i + 1, n_seeds, k, time.time() - t0))
    man = dict(seeds=[seed0, seed0 + n_seeds], view=[VIEW_W, VIEW_H], crop=CROP, crops=k, density=density,
               boxes=SCENE_BOXES if density == "fixed" else [200, 10000],
               spheres=SCENE_SPHERES if density == "fixed" else [50, 6000], spp_in=SPP_IN, spp_target=SPP_TARGET, radius=RADIUS, crop_rng="PCG64(seed^0xC409)")
    return Dataset(xs[:k], ys[:k], man)


def init_head(net, target_mean: float, head_scale: float = 0.1):
    """Start the sigmoid head at the data's mean AO: bias logit(mean), head weights scaled
    down. With the head at 0.5 against targets near 1, the first Adam steps drive every ReLU
    of the last level negative and the network collapses to a constant."""
    p = net.get_params()
    m = min(max(target_mean, 1e-3), 1 - 1e-3)
    p[-33:-1] *= head_scale
    p[-1] = np.log(m / (1 - m))
    net.set_params(p)


def lr_at(step: int, total: int, peak: float, warmup: int = 100) -> float:
    """Linear warm-up over `warmup` steps, then cosine decay to zero at `total`."""
    if step < warmup:
        return peak * (step + 1) / warmup
    return 0.5 * peak * (1.0 + np.cos(np.pi * min(1.0, (step - warmup) / max(1, total - warmup))))


def train(net, data: Dataset, steps: int, batch: int = 64, lr: float = 1e-3, seed: int = 0, log=print,
          log_every: int = 500, start: int = 0, total: int = 0, pg=None):
    """Adam on the MSE for `steps` mini-batches of a seeded shuffle, learning rate from lr_at
    over `total` steps (0: constant lr); returns the losses. With a process group of several
    ranks (one GPU each, the same data and seed on every rank), each step takes world x batch
    crops, rank r its r-th run of `batch`, and the gradients are averaged over the ranks
    before the shared Adam step (replicas.dp_train_step)."""
    import torch
    import replicas
    world = pg.get_world_size() if pg is not None and pg.is_initialized() else 1
    rank = pg.get_rank() if world > 1 else 0
    gen = torch.Generator(device="cuda").manual_seed(seed)
    n = data.x.shape[0]
    losses = []
    t0 = time.time()
    flat = torch.empty(net.grad_count, device="cuda") if world > 1 else None
    perm, pos = torch.randperm(n, device="cuda", generator=gen), 0
    for step in range(start, start + steps):
        if pos + world * batch > n:
            perm, pos = torch.randperm(n, device="cuda", generator=gen), 0
        idx = replicas.batch_indices(perm, pos, batch, rank, world)
        pos += world * batch
        step_lr = lr_at(step, total, lr) if total else lr
        if world > 1:
            losses.append(replicas.dp_train_step(net, data.x[idx].contiguous(), data.y[idx].contiguous(), step_lr,
                                                 flat, pg))
        else:
            losses.append(net.train_step(data.x[idx].contiguous(), data.y[idx].contiguous(), step_lr))
        if log and (step + 1) % log_every == 0:
            gn, sc = net.last_grad_norm()
            log("train: step %d loss %.6f lr %.2e |g| %.3e clip %.3f (%.1f s)" % (
                step + 1, float(np.mean(losses[-log_every:])), step_lr, gn, sc, time.time() - t0))
    return losses


def padded_shape(h: int, w: int):
    """The network input shape for an h x w frame: multiples of 16, and (H/8)(W/8) a multiple
    of 128 (the deepest level's GEMM rows)."""
    H, W = -(-h // 16) * 16, -(-w // 16) * 16
    while ((H // 8) * (W // 8)) % 128:
        H += 16
    return H, W


def pad_to(t, H: int, W: int, value: float = 0.0):
    import torch.nn.functional as F
    h, w = t.shape[:2]
    if (h, w) == (H, W):
        return t.contiguous()
    if t.dim() == 3:
        return F.pad(t.permute(2, 0, 1), (0, W - w, 0, H - h), value=value).permute(1, 2, 0).contiguous()
    return F.pad(t, (0, W - w, 0, H - h), value=value).contiguous()


def predict(net, f):
    """The network's AO for one (h, w, 5) feature image; `net` was created for its padded shape."""
    h, w = f.shape[:2]
    _, H, W = net.shape
    x = pad_to(f, H, W)
    if (H, W) != (h, w):               # the padding reads as uncovered pixels (AO 1)
        x[h:, :, 4] = 1.0
        x[:h, w:, 4] = 1.0
    return net.forward(x[None])[0, :h, :w]


def tile_sum(t, tile: int = TILE):
    """Sums of an (h, w) float tensor over tile x tile tiles (the last row/column of tiles
    padded with zeros)."""
    import torch.nn.functional as F
    h, w = t.shape
    return F.avg_pool2d(F.pad(t[None, None], (0, (-w) % tile, 0, (-h) % tile)), tile)[0, 0] * (tile * tile)


def fallback_tiles(pred, ao4, mask, spp_in: int = SPP_IN, k: float = 3.0, tile: int = TILE):
    """(ceil(h/tile), ceil(w/tile)) bool map of the tiles whose predicted mean leaves the
    confidence band around the 4-spp mean."""
    import torch
    m = mask.float()
    tsum = lambda t: tile_sum(t, tile)
    cnt = tsum(m)
    n = cnt.clamp(min=1)
    mean_p = tsum(pred * m) / n
    mean_4 = tsum(ao4 * m) / n
    var = tsum(ao4 * (1 - ao4) * m).clamp(min=0)
    sigma = torch.maximum(torch.sqrt(var / spp_in) / n, 0.5 / torch.sqrt(spp_in * n))
    return ((mean_p - mean_4).abs() > k * sigma) & (cnt > 0)


def tiles_to_pixels(tiles, h: int, w: int, tile: int = TILE):
    return tiles.repeat_interleave(tile, 0).repeat_interleave(tile, 1)[:h, :w]


def surrogate_ao(net, g, depth, acc, spp_full: int, radius: float = RADIUS, k: float = 3.0, ao4=None):
    """The surrogate's AO for one frame: a 4-spp trace, the network, and the fallback tiles
    traced at spp_full. Returns (ao, fallback tile fraction of covered tiles)."""
    import torch
    if ao4 is None:
        ao4 = rn.compute_rtao(g, acc, SPP_IN, radius)
    pred = predict(net, features(g, depth, ao4, radius))
    tiles = fallback_tiles(pred, ao4, g.mask, SPP_IN, k)
    h, w = g.mask.shape
    m = g.mask.bool()
    out = torch.where(m, pred, torch.ones_like(pred))
    fb = tiles_to_pixels(tiles, h, w) & m
    if bool(fb.any()):
        out = torch.where(fb, masked_trace(g, acc, spp_full, fb, radius), out)
    n_cov = int((tile_sum(m.float()) > 0).sum())
    return out, float(tiles.sum()) / max(1, n_cov)


def rmse(a, b, mask) -> float:
    m = mask.bool()
    return float(((a - b)[m].double() ** 2).mean().sqrt()) if bool(m.any()) else 0.0


def save_checkpoint(net, path: str, seed: int, data_manifest: dict, extra=None):
    """Master weights, Adam moments, step, seed and the data manifest with its digest."""
    state, step = net.get_state()
    digest = hashlib.sha256(json.dumps(data_manifest, sort_keys=True).encode()).hexdigest()[:16]
    np.savez_compressed(path, state=state, step=step, seed=seed, data_digest=digest,
                        manifest=json.dumps(data_manifest, sort_keys=True), extra=json.dumps(extra or {}))


def save_weights(net, path: str, meta: dict):
    """Inference weights only, rounded to BF16 (the values the GEMMs read), as uint16."""
    p = net.get_params()
    bits = p.view(np.uint32)
    r = ((bits + 0x7FFF + ((bits >> 16) & 1)) >> 16).astype(np.uint16)      # round to nearest even
    np.savez_compressed(path, bf16=r, meta=json.dumps(meta, sort_keys=True))


def load_weights(net, path: str) -> dict:
    z = np.load(path, allow_pickle=False)
    if "state" in z:
        net.set_state(z["state"], int(z["step"]))
        return dict(step=int(z["step"]), seed=int(z["seed"]), data_digest=str(z["data_digest"]))
    p = (z["bf16"].astype(np.uint32) << 16).view(np.float32)
    net.set_params(p)
    return json.loads(str(z["meta"]))


# ------------------------------------------------------------------ evaluation
def eval_frame(net, sc, cam, w: int, h: int, spps=(16, 32, 64, 128, 256), k: float = 3.0, spp_full: int = 256):
    """RMSE against the 1024-spp trace of: the 4-spp trace, the network alone, the network
    with fallback, and plain tracing at each of `spps`; plus the fallback fraction."""
    import torch
    tris = torch.from_numpy(sc.tris).cuda()
    nrms = torch.from_numpy(sc.normals).cuda()
    acc = rn.LinearAccel(tris)
    g, depth = rn.rasterize(tris, nrms, cam, w, h, want_depth=True)
    truth = rn.compute_rtao(g, acc, SPP_TARGET, RADIUS)
    ao4 = rn.compute_rtao(g, acc, SPP_IN, RADIUS)
    pred = predict(net, features(g, depth, ao4))
    out, frac = surrogate_ao(net, g, depth, acc, spp_full, k=k, ao4=ao4)
    r = dict(covered=int(g.mask.sum()), rmse_ao4=rmse(ao4, truth, g.mask), rmse_net=rmse(pred, truth, g.mask),
             rmse_surrogate=rmse(out, truth, g.mask), fallback_fraction=frac)
    for s in spps:
        r["rmse_rt%d" % s] = rmse(rn.compute_rtao(g, acc, s, RADIUS), truth, g.mask)
    acc.close()
    return r


def evaluate(net, n_seeds: int, seed0: int = EVAL_SEED0, w: int = VIEW_W, h: int = VIEW_H, log=print,
             density: str = "fixed", **kw):
    rows = []
    for sd, sc in SceneSource(range(seed0, seed0 + n_seeds), density):
        rows.append(dict(seed=sd, **eval_frame(net, sc, camera_for(sd), w, h, **kw)))
        if log and len(rows) % max(1, n_seeds // 10) == 0:
            log("eval: %d/%d  net %.4f  surrogate %.4f  fallback %.3f" % (
                len(rows), n_seeds, np.mean([r["rmse_net"] for r in rows]),
                np.mean([r["rmse_surrogate"] for r in rows]), np.mean([r["fallback_fraction"] for r in rows])))
    keys = [k for k in rows[0] if k.startswith("rmse") or k == "fallback_fraction"]
    summary = {k: float(np.mean([r[k] for r in rows])) for k in keys}
    summary["frames"] = len(rows)
    return summary, rows


# ------------------------------------------------------------------ command line
def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    sub = ap.add_subparsers(dest="cmd", required=True)
    t = sub.add_parser("train")
    t.add_argument("--out", required=True)
    t.add_argument("--seeds", type=int, default=2000)
    t.add_argument("--crops", type=int, default=20000)
    t.add_argument("--steps", type=int, default=20000)
    t.add_argument("--batch", type=int, default=64)
    t.add_argument("--lr", type=float, default=1e-3)
    t.add_argument("--init-seed", type=int, default=0)
    t.add_argument("--clip", type=float, default=2.0)
    t.add_argument("--ckpt-every", type=int, default=5000)
    t.add_argument("--eval-seeds", type=int, default=0)
    t.add_argument("--density", choices=["fixed", "mixed"], default="fixed",
                   help="training scenes: 200 boxes + 50 spheres, or counts drawn per seed up to the large scene's")
    e = sub.add_parser("eval")
    e.add_argument("--ckpt", required=True)
    e.add_argument("--seeds", type=int, default=200)
    e.add_argument("--out", default=None)
    e.add_argument("--density", choices=["fixed", "mixed"], default="fixed")
    a = ap.parse_args(argv)
    import torch
    import replicas
    rank, world, local = replicas.rank_env()
    pg = None
    if world > 1:
        # data-parallel training under torchrun: one GPU per rank, NCCL for the gradients
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
        pg = dist
    rn.init()
    if a.cmd == "train":
        os.makedirs(a.out, exist_ok=True)
        log_f = open(os.path.join(a.out, "train.log" if rank == 0 else "train.rank%d.log" % rank), "a")

        def log(msg):
            if rank == 0:
                print(msg, flush=True)
            log_f.write(msg + "\n")
            log_f.flush()
        t0 = time.time()
        data = generate_dataset(a.seeds, a.crops, log=log, density=a.density)
        torch.cuda.synchronize()
        log("data: %d crops in %.1f s, digest %s" % (data.x.shape[0], time.time() - t0, data.digest))
        net = rn.UNet(a.batch, CROP, CROP, seed=a.init_seed)
        init_head(net, float(data.y.mean()))
        net.set_clip(a.clip)
        done = 0
        t1 = time.time()
        while done < a.steps:
            n = min(a.ckpt_every, a.steps - done)
            train(net, data, n, a.batch, a.lr, seed=a.init_seed + done, log=log, start=done, total=a.steps, pg=pg)
            done += n
            if rank == 0:
                save_checkpoint(net, os.path.join(a.out, "surrogate_ckpt.npz"), a.init_seed, data.manifest)
        train_s = time.time() - t1
        log("train: %d steps in %.1f s (%.2f ms/step)" % (a.steps, train_s, 1e3 * train_s / max(1, a.steps)))
        meta = dict(data=data.manifest, data_digest=data.digest, steps=a.steps, batch=a.batch, lr=a.lr,
                    schedule="warmup 100, cosine", clip=a.clip, init_seed=a.init_seed, train_seconds=round(train_s, 1),
                    ranks=world)
        if rank != 0:
            return 0
        save_weights(net, os.path.join(a.out, "surrogate_bf16.npz"), meta)
        del data
        if a.eval_seeds:
            inf = rn.UNet(1, *padded_shape(VIEW_H, VIEW_W), inference=True)
            load_weights(inf, os.path.join(a.out, "surrogate_bf16.npz"))
            summary, rows = evaluate(inf, a.eval_seeds, log=log)
            log("eval: " + json.dumps(summary))
            json.dump(dict(summary=summary, rows=rows, meta=meta), open(os.path.join(a.out, "eval.json"), "w"), indent=1)
    else:
        inf = rn.UNet(1, *padded_shape(VIEW_H, VIEW_W), inference=True)
        meta = load_weights(inf, a.ckpt)
        summary, rows = evaluate(inf, a.seeds, density=a.density)
        print(json.dumps(summary))
        if a.out:
            json.dump(dict(summary=summary, rows=rows, meta=meta), open(a.out, "w"), indent=1)


if __name__ == "__main__":
    sys.exit(main())
