"""Several GPUs, one process each: how the AO path splits over ranks and how the ranks'
results combine. Pixels, tiles and views are independent, so no data-path collective is
needed: every rank builds its own BVH from the identical FP32 triangle list (the build is
deterministic), works on its own share, and the host combines the shares.

  - a frame splits by row band: rank r traces and shades rows [y0, y1) of the frame in frame
    coordinates (the sampler hashes frame x, y), reading the whole G-buffer so SSAO's
    6-pixel neighbourhood crosses band edges; its reconcile covers its rows only;
  - a set of views splits round-robin by view;
  - surrogate training splits each step's crops by rank (data parallel): every rank runs the
    backward pass on its crops, the gradients are averaged with one all-reduce of a flat
    tensor, and every rank takes the same Adam step;
  - the reconcile's parts (FP64 sum of squared errors, covered pixels, max error) combine on
    the host in rank order, and the RMSE and verdict follow as raw::reconcile derives them
    (src/cert/reconcile.cpp:17-20): rmse = (float)sqrt(sum / n), within = rmse <= tolerance.

Timing over ranks takes the maximum (the job ends with its slowest rank).
"""
from __future__ import annotations

import dataclasses
import math
import os

import numpy as np


def rank_env():
    """(rank, world size, local rank) from the launcher's environment (1 rank without one)."""
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def row_band(h: int, rank: int, world: int):
    """Rows [y0, y1) of an h-row frame for `rank`: contiguous bands, sizes differing by <= 1."""
    if not (0 <= rank < world):
        raise ValueError("rank %d of %d" % (rank, world))
    base, extra = divmod(h, world)
    y0 = rank * base + min(rank, extra)
    return y0, y0 + base + (1 if rank < extra else 0)


def shard_views(views, rank: int, world: int):
    """The views of `rank`: every world-th view starting at rank (uneven sizes spread out)."""
    if not (0 <= rank < world):
        raise ValueError("rank %d of %d" % (rank, world))
    return list(views)[rank::world]


@dataclasses.dataclass
class ReconcilePart:
    sum_sq: float      # FP64 sum of squared errors over the part's covered pixels
    pixels: int
    max_error: float

    def as_array(self):
        return np.array([self.sum_sq, float(self.pixels), self.max_error], np.float64)

    @staticmethod
    def from_array(a) -> "ReconcilePart":
        return ReconcilePart(float(a[0]), int(round(float(a[1]))), float(a[2]))


@dataclasses.dataclass
class Combined:
    rmse: float
    max_error: float
    pixels: int
    within_tolerance: bool
    sum_sq: float


def combine_reconcile(parts, tolerance: float) -> Combined:
    """The whole frame's reconcile from its parts, summed in the order given (rank order).

    With no masked pixel at all the rmse is 0 and the verdict is rmse <= tolerance, i.e. true,
    as src/cert/reconcile.cpp:18-19 decides it (the certificate turns pixels == 0 into
    "unverifiable" on its own, src/cert/certificate_from.cpp)."""
    total, n, mx = 0.0, 0, 0.0
    for p in parts:
        total += p.sum_sq
        n += p.pixels
        mx = max(mx, p.max_error)
    rmse = float(np.float32(math.sqrt(total / n))) if n else 0.0
    return Combined(rmse, float(np.float32(mx)), n, bool(rmse <= np.float32(tolerance)), total)


def gather_parts(part: ReconcilePart, pg=None, device=None):
    """Every rank's part, in rank order (all ranks receive all)."""
    if pg is None or not pg.is_initialized() or pg.get_world_size() == 1:
        return [part]
    import torch
    t = torch.from_numpy(part.as_array())
    if device is not None:
        t = t.to(device)
    out = [torch.zeros_like(t) for _ in range(pg.get_world_size())]
    pg.all_gather(out, t)
    return [ReconcilePart.from_array(o.cpu().numpy()) for o in out]


def max_over_ranks(x: float, pg=None, device=None) -> float:
    if pg is None or not pg.is_initialized() or pg.get_world_size() == 1:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def batch_indices(perm, pos: int, batch: int, rank: int, world: int):
    """This rank's crops of one data-parallel step: the step takes world x batch consecutive
    entries of the shared permutation from `pos` and rank r the r-th run of `batch` (every
    rank holds the same permutation, drawn from the same seed)."""
    if not (0 <= rank < world):
        raise ValueError("rank %d of %d" % (rank, world))
    return perm[pos + rank * batch: pos + (rank + 1) * batch]


def allreduce_mean_(t, pg=None):
    """In place: the mean of `t` over the ranks (a sum all-reduce, then / world)."""
    if pg is None or not pg.is_initialized() or pg.get_world_size() == 1:
        return t
    pg.all_reduce(t)
    t /= pg.get_world_size()
    return t


def dp_train_step(net, x, y, lr: float, flat, pg=None) -> float:
    """One data-parallel step of the surrogate network: backward on this rank's batch, the
    gradients averaged over the ranks (all-reduce of one flat CUDA tensor), then the same
    clipped Adam update on every rank, so the replicas stay identical. Returns the mean of
    the ranks' batch losses."""
    import torch
    loss = net.backward(x, y)
    if pg is None or not pg.is_initialized() or pg.get_world_size() == 1:
        net.apply(lr)
        return loss
    net.grads_to(flat)
    allreduce_mean_(flat, pg)
    net.grads_from(flat)
    net.apply(lr)
    lt = torch.tensor([loss], dtype=torch.float64, device=flat.device)
    allreduce_mean_(lt, pg)
    return float(lt.item())


def band_frame(g, accel, rank: int, world: int, samples: int, radius: float, ss_samples: int, tolerance: float,
               to_light=None):
    """One rank's band of an AO frame on its GPU: traced AO (and sky/sun) and SSAO for rows
    [y0, y1) (other rows are left at 1 / unwritten), and the reconcile part of those rows.
    Returns (outputs dict, ReconcilePart)."""
    import torch
    import rn_ao as rn
    h, w = g.shape
    y0, y1 = row_band(h, rank, world)
    band = torch.zeros(h, w, dtype=torch.bool, device=g.mask.device)
    band[y0:y1] = True
    gb = rn.GBuffer(g.position, g.normal, (g.mask.bool() & band).to(torch.uint8).contiguous())
    if to_light is not None:
        ao, sky, sun = rn.compute_rt_visibility(gb, accel, samples, radius, to_light)
    else:
        ao, sky, sun = rn.compute_rtao(gb, accel, samples, radius), None, None
    ss = rn.compute_ssao(g, ss_samples, radius)           # the whole G-buffer: neighbours cross bands
    rec = rn.reconcile(ss[y0:y1].contiguous(), ao[y0:y1].contiguous(), g.mask[y0:y1].contiguous(), tolerance,
                       error_map=False)
    return dict(ao=ao, sky=sky, sun=sun, ss=ss, rows=(y0, y1)), ReconcilePart(rec.sum_sq, rec.pixels, rec.max_error)
