"""GPU PLOC builder and traversal against the oracle.

The binary tree must equal rt::buildPloc node for node (tree hash, root, rounds), as the
reference's own GPU build does (evidence/rt-r2-bvh-gpu-d3d12-rtx4090.json); the 4-wide
accelerator built from it must answer every any-hit query exactly as the scan of every
triangle does (tests/test_bvh.cpp's criterion).
"""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
PLOC = json.load(open(os.path.join(HERE, "golden", "ploc.json")))


def test_soup_tree_hash(rn, oracle):
    s = PLOC["scenes"]["soup"]
    tris = oracle.soup(s["count"], s["seed"])
    nodes, root, rounds = rn.build_ploc(tris)
    assert oracle.tree_hash(nodes) == s["tree_hash"]
    assert rounds == s["rounds"] and root == 2 * s["count"] - 2


def test_test_scene_tree(rn, oracle):
    s = PLOC["scenes"]["test_scene"]
    tris, _, _ = oracle.test_scene()
    nodes, root, rounds = rn.build_ploc(tris)
    assert (oracle.tree_hash(nodes), root, rounds) == (s["tree_hash"], s["root"], s["rounds"])


@pytest.mark.parametrize("n,seed", [(1, 1), (2, 2), (3, 3), (5, 4), (17, 5), (1000, 6), (4097, 7), (65536, 8),
                                    (300001, 9)])
def test_ploc_equals_oracle(rn, oracle, n, seed):
    tris = oracle.soup(n, seed)
    nodes, root, rounds = rn.build_ploc(tris)
    rn_nodes, rroot, rrounds = oracle.ploc(tris)
    assert root == rroot and rounds == rrounds
    assert np.array_equal(nodes, rn_nodes), int((nodes != rn_nodes).any(axis=1).sum())


@pytest.mark.parametrize("tail,ctas", [(4096, 1), (32768, 1), (262144, 1), (4096, 4), (65536, 8), (262144, 8),
                                       (262144, 16)])
@pytest.mark.parametrize("n,seed,radius", [(2, 2, 16), (17, 5, 16), (4097, 7, 16), (65536, 8, 16), (300001, 9, 16),
                                           (20000, 7, 8), (5000, 12, 32)])
def test_ploc_tail_in_one_launch_equals_oracle(rn, oracle, tail, ctas, n, seed, radius):
    """The last rounds in one block or one thread-block cluster (ploc_tail, ploc_tail_ctas)
    build the same tree, node for node."""
    old = rn.tune_get("ploc_tail"), rn.tune_get("ploc_tail_ctas")
    rn.tune_set("ploc_tail", tail)
    rn.tune_set("ploc_tail_ctas", ctas)
    try:
        tris = oracle.soup(n, seed)
        nodes, root, rounds = rn.build_ploc(tris, radius)
        rn_nodes, rroot, rrounds = oracle.ploc(tris, radius)
        assert root == rroot and rounds == rrounds
        assert np.array_equal(nodes, rn_nodes), int((nodes != rn_nodes).any(axis=1).sum())
    finally:
        rn.tune_set("ploc_tail", old[0])
        rn.tune_set("ploc_tail_ctas", old[1])


@pytest.mark.parametrize("tail", [0, 4096, 32768])
@pytest.mark.parametrize("n,seed,radius", [(2, 2, 16), (17, 5, 16), (4097, 7, 16), (65536, 8, 16), (300001, 9, 16),
                                           (20000, 7, 8), (5000, 12, 32), (1000000, 3, 8)])
def test_ploc_fused_rounds_equal_oracle(rn, oracle, tail, n, seed, radius):
    """A round's prefix sum, scatter and commit in one launch (ploc_fused: tiles by ticket,
    decoupled look-back) build the same tree, node for node, with and without the tail, twice
    in a row (the look-back words of the first build must not pass for the second's)."""
    old = rn.tune_get("ploc_tail"), rn.tune_get("ploc_fused")
    rn.tune_set("ploc_tail", tail)
    rn.tune_set("ploc_fused", 1)
    try:
        tris = oracle.soup(n, seed)
        rn_nodes, rroot, rrounds = oracle.ploc(tris, radius)
        for _ in range(2):
            nodes, root, rounds = rn.build_ploc(tris, radius)
            assert root == rroot and rounds == rrounds
            assert np.array_equal(nodes, rn_nodes), int((nodes != rn_nodes).any(axis=1).sum())
    finally:
        rn.tune_set("ploc_tail", old[0])
        rn.tune_set("ploc_fused", old[1])


def test_ploc_radius_8_differs(rn, oracle):
    tris = oracle.soup(5000, 12)
    a = rn.build_ploc(tris, 16)[0]
    b = rn.build_ploc(tris, 8)[0]
    assert oracle.tree_hash(a) != oracle.tree_hash(b)
    assert np.array_equal(b, oracle.ploc(tris, 8)[0])


def test_ploc_duplicate_centroids(rn, oracle):
    # many triangles with one centroid: equal Morton codes, order by index
    t = np.tile(np.array([[0, 0, 0, 1, 0, 0, 0, 1, 0]], np.float32), (300, 1))
    t[::3] += np.float32(0.25)
    nodes, root, rounds = rn.build_ploc(t)
    r = oracle.ploc(t)
    assert np.array_equal(nodes, r[0]) and (root, rounds) == (r[1], r[2])


def random_rays(rng, n, lo=-14.0, hi=14.0):
    o = rng.uniform(lo, hi, (n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True).astype(np.float32)
    return np.ascontiguousarray(np.concatenate([o, d], axis=1), np.float32)


@pytest.mark.parametrize("scene", ["test", "soup"])
def test_any_hit_equals_scan(rn, oracle, scene):
    rng = np.random.default_rng(42)
    tris = oracle.test_scene()[0] if scene == "test" else oracle.soup(20000, 7)
    acc = rn.LinearAccel(tris)
    n = 20000
    rays = random_rays(rng, n, -6, 6) if scene == "test" else random_rays(rng, n)
    tmax = np.where(rng.random(n) < 0.5, np.float32(1e30), rng.uniform(0.1, 8.0, n)).astype(np.float32)
    got = rn.occluded(acc, rays, tmax)
    ref = oracle.occluded_scan(tris, rays, tmax, threads=os.cpu_count() or 1)
    assert np.array_equal(got, ref), int((got != ref).sum())
    assert 0.05 * n < ref.sum() < n


def test_accel_info(rn, oracle):
    """The accelerator of a 20,000-triangle soup with the default shape (PLOC radius 16, leaves
    of at most 4 triangles): the PLOC round count and the 4-wide node count."""
    saved = {k: rn.tune_get(k) for k in ("accel_radius", "accel_leaf")}
    try:
        rn.tune_set("accel_radius", 16)
        rn.tune_set("accel_leaf", 4)
        tris = oracle.soup(20000, 7)
        acc = rn.LinearAccel(tris)
        info = acc.info()
        assert info["leaf_tris"] == 20000 and info["ploc_rounds"] == 40
        assert 20000 // 4 // 4 <= info["wide_nodes"] < 20000
    finally:
        for k, v in saved.items():
            rn.tune_set(k, v)
