"""The path tracer's oracle pinned (CPU): rno_pathtrace, the C restatement of
raw::rt::pathTraceCpu (interface v4, v2 scenes), against the reference's own outputs.

- The lobe's energy table equals the reference's, byte for byte (its SHA-256 in
  tests/golden/pt.json, made from the reference build by tests/golden/make_golden_pt.py).
- On the reference's lit scenes (tests/golden/pt_scenes.npz, made by the reference's own
  scene builders) every AOV of every golden case equals the reference's bytes: radiance,
  albedo, normal, depth, variance, triangle, motion, and the split radiance with its albedos
  and variances.
- Where the reference build is present (oracle/_ref), the oracle also equals it on a seeded
  synthetic scene with emissive, metallic and rough triangles, and on the 100,760-triangle
  dense_block.
"""
import hashlib
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = json.load(open(os.path.join(HERE, "golden", "pt.json")))
SCENES = np.load(os.path.join(HERE, "golden", "pt_scenes.npz"))


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def scene(key):
    sc = {k.split("/", 1)[1]: SCENES[k] for k in SCENES.files if k.startswith(key + "/")}
    cam = sc.pop("camera")
    return sc, cam


@pytest.fixture(scope="module")
def table(oracle):
    return oracle.pt_energy_table()


def test_energy_table_equals_the_reference(table):
    assert sha(table) == GOLD["energy_table_sha256"]
    assert table.dtype == np.float32 and table.size == 64 * 128 * 2 + 128 * 2


@pytest.mark.parametrize("case", sorted(GOLD["cases"]))
def test_oracle_equals_reference_outputs(oracle, table, case):
    c = GOLD["cases"][case]
    sc, _ = scene(c["scene"])
    out = oracle.pathtrace(sc, c["desc"], table=table)
    assert out["emitters"] == c["emitters"]
    bad = [k for k, h in c["sha256"].items() if sha(out[k]) != h]
    assert not bad, bad


def synthetic_scene(seed=5, boxes=40):
    """A seeded room of boxes: emissive ceiling quads, metals, rough and smooth dielectrics,
    a checkerboard texture (power-of-two sizes), smooth normals on a few boxes."""
    rng = np.random.default_rng(seed)
    pos, nrm, uv, idx, tex = [], [], [], [], []

    def quad(a, b, c, d, t, n=None):
        base = len(pos)
        for p in (a, b, c, d):
            pos.append(p)
        e1, e2 = np.subtract(b, a), np.subtract(d, a)
        nn = np.cross(e1, e2)
        nn = nn / np.linalg.norm(nn)
        for k in range(4):
            nrm.append(nn if n is None else n[k])
        uv.extend([(0, 0), (1, 0), (1, 1), (0, 1)])
        idx.extend([(base, base + 1, base + 2), (base, base + 2, base + 3)])
        tex.extend([t, t])

    s = 6.0
    quad((-s, 0, -s), (-s, 0, s), (s, 0, s), (s, 0, -s), 0)                       # floor (checkerboard)
    quad((-s, 4, -s), (s, 4, -s), (s, 4, s), (-s, 4, s), 1)                       # ceiling
    quad((-1, 3.99, -1), (1, 3.99, -1), (1, 3.99, 1), (-1, 3.99, 1), 2)          # lamp, facing down
    quad((-s, 0, -s), (s, 0, -s), (s, 4, -s), (-s, 4, -s), 1)                     # back wall
    for i in range(boxes):
        c = rng.uniform(-4.5, 4.5, 2)
        h = rng.uniform(0.3, 2.0)
        r = rng.uniform(0.2, 0.7)
        t = int(rng.integers(3, 6))
        x0, x1, z0, z1 = c[0] - r, c[0] + r, c[1] - r, c[1] + r
        quad((x0, h, z0), (x0, h, z1), (x1, h, z1), (x1, h, z0), t)
        quad((x0, 0, z0), (x1, 0, z0), (x1, h, z0), (x0, h, z0), t)
        quad((x0, 0, z1), (x0, h, z1), (x1, h, z1), (x1, 0, z1), t)
        quad((x0, 0, z0), (x0, h, z0), (x0, h, z1), (x0, 0, z1), t)
        quad((x1, 0, z0), (x1, 0, z1), (x1, h, z1), (x1, h, z0), t)
    board = np.array([0xff3050a0 if ((x // 4 + y // 4) % 2) else 0xffe0e0e0 for y in range(16) for x in range(16)],
                       np.uint32)
    white = np.full(16, 0xffffffff, np.uint32)
    rough = np.array([(0xff000000 | int(v)) for v in rng.integers(0, 2 ** 24, 64)], np.uint32)
    texels = np.concatenate([board, white, white, rough, white, rough])
    entries = np.array([(0, 16, 16), (256, 4, 4), (272, 4, 4), (288, 8, 8), (352, 4, 4), (368, 8, 8)], np.uint32)
    materials = np.array([(1.0, 0.7, 0.0, 0.5, 0, 0, 0),          # checkerboard floor
                          (0.8, 0.9, 0.0, 0.3, 0, 0, 0),          # walls
                          (1.0, 1.0, 0.0, 0.0, 8.0, 7.0, 6.0),    # lamp
                          (1.0, 0.3, 1.0, 1.0, 0, 0, 0),          # rough metal
                          (1.0, 0.08, 0.0, 1.0, 0, 0, 0),         # glossy dielectric
                          (0.9, 0.6, 0.3, 0.7, 0, 0, 0)], np.float32)
    return dict(pos=np.array(pos, np.float32), nrm=np.array(nrm, np.float32), uv=np.array(uv, np.float32),
                idx=np.array(idx, np.uint32), tri_tex=np.array(tex, np.uint32), tex_entries=entries, texels=texels,
                materials=materials, sun_dir=np.array([0.3, 0.9, 0.2], np.float32),
                sun_irr=np.array([2.0, 1.9, 1.7], np.float32), sky=np.array([0.2, 0.25, 0.3], np.float32))


SYNTH_CAMERA = (0.0, 2.5, 5.5, 0.0, 1.0, -1.0, 0.0, 1.0, 0.0, 1.1)


def _has_ref(oracle):
    try:
        oracle.ref()
        return True
    except OSError:
        return False


@pytest.mark.parametrize("controls", [[], ["legacy_lobe_v2"], ["aov_emission_to_diffuse", "mis_weight_one"]])
def test_oracle_equals_reference_on_a_synthetic_scene(oracle, table, controls):
    if not _has_ref(oracle):
        pytest.skip("the reference build (oracle/_ref) is not on this host")
    sc = synthetic_scene()
    d = dict(seed=(11 << 32) | 3, spp=6, width=56, height=40, camera=SYNTH_CAMERA, controls=controls)
    a = oracle.pathtrace(sc, d, use_ref=True)
    b = oracle.pathtrace(sc, d, table=table)
    assert a["emitters"] == b["emitters"] == 2
    for k, _, _ in oracle.PT_AOVS:
        assert np.array_equal(a[k], b[k]), k


def test_oracle_equals_reference_on_dense_block(oracle, table):
    if not _has_ref(oracle):
        pytest.skip("the reference build (oracle/_ref) is not on this host")
    sc, cam = oracle.pt_reference_scene("dense_block")
    d = dict(seed=1, spp=2, width=40, height=30, camera=cam)
    a = oracle.pathtrace(sc, d, use_ref=True)
    b = oracle.pathtrace(sc, d, table=table)
    for k, _, _ in oracle.PT_AOVS:
        assert np.array_equal(a[k], b[k]), k
