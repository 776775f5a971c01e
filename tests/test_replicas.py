"""Several ranks, one GPU each (host-side logic, on CPU): row bands and view shards cover
their frame / view list exactly once, and a frame's reconcile combined from per-rank parts
(gathered over a 2-rank gloo group) gives the whole frame's pixels, maximum and RMSE."""
import os
import socket

import numpy as np
import pytest

import replicas


@pytest.mark.parametrize("h,world", [(1, 1), (7, 2), (2160, 3), (1080, 8), (5, 8)])
def test_row_bands_partition_the_frame(h, world):
    rows = []
    for r in range(world):
        y0, y1 = replicas.row_band(h, r, world)
        assert 0 <= y0 <= y1 <= h
        rows.extend(range(y0, y1))
    assert rows == list(range(h))
    sizes = [np.subtract(*replicas.row_band(h, r, world)[::-1]) for r in range(world)]
    assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        replicas.row_band(h, world, world)


def test_view_shards_partition_the_views():
    views = list(range(64))
    for world in (1, 2, 3, 8):
        got = sorted(v for r in range(world) for v in replicas.shard_views(views, r, world))
        assert got == views


def _synthetic(h=37, w=53, seed=3):
    rng = np.random.default_rng(seed)
    a = rng.random((h, w), np.float32)
    t = rng.random((h, w), np.float32)
    m = (rng.random((h, w)) < 0.7).astype(np.uint8)
    return a, t, m


def test_combined_parts_equal_the_whole_frame(oracle):
    a, t, m = _synthetic()
    _, whole = oracle.reconcile(a, t, m, 0.3)
    for world in (1, 2, 5):
        parts = []
        for r in range(world):
            y0, y1 = replicas.row_band(a.shape[0], r, world)
            _, d = oracle.reconcile(a[y0:y1], t[y0:y1], m[y0:y1], 0.3)
            parts.append(replicas.ReconcilePart(d["sumSq"], d["pixels"], d["maxError"]))
        c = replicas.combine_reconcile(parts, 0.3)
        assert c.pixels == whole["pixels"] and c.max_error == whole["maxError"]
        assert c.rmse == whole["rmse"] and c.within_tolerance == whole["within"]
        assert abs(c.sum_sq - whole["sumSq"]) <= 1e-12 * whole["sumSq"]
    empty = replicas.combine_reconcile([replicas.ReconcilePart(0.0, 0, 0.0)] * 2, 0.3)
    assert empty.pixels == 0 and empty.rmse == 0.0 and empty.within_tolerance


def test_combined_verdict_equals_oracle_on_empty_partial_and_full_masks(oracle):
    """src/cert/reconcile.cpp:18-19: with no masked pixel rmse is 0 and the verdict is true."""
    a, t, m = _synthetic()
    masks = {"empty": np.zeros_like(m), "partial": m, "full": np.ones_like(m)}
    for name, mk in masks.items():
        for tol in (0.0, 0.05, 0.3):
            _, whole = oracle.reconcile(a, t, mk, tol)
            parts = []
            for r in range(3):
                y0, y1 = replicas.row_band(a.shape[0], r, 3)
                _, d = oracle.reconcile(a[y0:y1], t[y0:y1], np.ascontiguousarray(mk[y0:y1]), tol)
                parts.append(replicas.ReconcilePart(d["sumSq"], d["pixels"], d["maxError"]))
            c = replicas.combine_reconcile(parts, tol)
            assert c.pixels == whole["pixels"], name
            assert c.rmse == whole["rmse"] and c.within_tolerance == whole["within"], (name, tol, c, whole)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, q):
    import sys
    import torch.distributed as dist
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for p in (root, os.path.join(root, "raw-native_gb300")):
        sys.path.insert(0, p)
    import replicas as R
    from oracle import oracle as O
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        a, t, m = _synthetic()
        y0, y1 = R.row_band(a.shape[0], rank, world)
        _, d = O.reconcile(a[y0:y1], t[y0:y1], m[y0:y1], 0.3)
        parts = R.gather_parts(R.ReconcilePart(d["sumSq"], d["pixels"], d["maxError"]), dist)
        c = R.combine_reconcile(parts, 0.3)
        slowest = R.max_over_ranks(10.0 + rank, dist)
        q.put((rank, c.rmse, c.pixels, c.max_error, c.sum_sq, slowest, [p.pixels for p in parts]))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_combine_a_banded_reconcile(oracle):
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    a, t, m = _synthetic()
    _, whole = oracle.reconcile(a, t, m, 0.3)
    for rank, rmse, pixels, mx, ssum, slowest, per_rank in results:
        assert rmse == whole["rmse"] and pixels == whole["pixels"] and mx == whole["maxError"]
        assert slowest == 11.0
        assert sum(per_rank) == whole["pixels"]
    assert results[0][4] == results[1][4]              # every rank combined the same sum


def test_data_parallel_batches_partition_each_step():
    import torch
    perm = torch.randperm(1000, generator=torch.Generator().manual_seed(1))
    for world in (1, 2, 4):
        pos = 0
        for _ in range(3):
            got = torch.cat([replicas.batch_indices(perm, pos, 16, r, world) for r in range(world)])
            assert torch.equal(got, perm[pos:pos + 16 * world])
            pos += 16 * world
    with pytest.raises(ValueError):
        replicas.batch_indices(perm, 0, 16, 2, 2)


def _dp_rank_main(rank, world, port, q):
    import sys
    import torch
    import torch.distributed as dist
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for p in (root, os.path.join(root, "raw-native_gb300")):
        sys.path.insert(0, p)
    import replicas as R
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # each rank's "gradients" (a stand-in flat tensor); the mean over the ranks reaches all
        g = torch.arange(6, dtype=torch.float32) * (rank + 1)
        R.allreduce_mean_(g, dist)
        q.put((rank, g.tolist()))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_average_gradients():
    """The data-parallel gradient exchange (one all-reduce of a flat tensor, / world) gives
    every rank the same mean."""
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_dp_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    want = [1.5 * i for i in range(6)]
    assert results[0] == want and results[1] == want
