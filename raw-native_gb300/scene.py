"""Scenes the AO path renders: the reference's built-in test scene and the seeded synthetic
scenes of the large workloads.

build_test_scene() restates raw::buildTestScene (src/scene/scene.cpp:4-32): a 10 x 10 plane
(2 triangles) and a 2 x 2 x 2 box centred at (0, 1, 0) (12 triangles), in the order
raw::LinearAccel::build flattens them (src/renderer/accel.cpp:13-25), with per-corner
normals for the rasterizer and the light direction normalize(-0.4, -1, -0.3).
"""
from __future__ import annotations

import dataclasses

import numpy as np

F = np.float32

# raw/tools/cli_params.hpp:16-21: the CLI's default view.
DEFAULT_CAMERA = (4.0, 4.0, 6.0, 0.0, 1.0, 0.0, 0.0, 1.0, 0.0, 0.9)


@dataclasses.dataclass
class Scene:
    tris: np.ndarray       # (n, 9) float32: corners a, b, c
    normals: np.ndarray    # (n, 9) float32: the corners' vertex normals
    light: np.ndarray      # (3,) float32: lights[0].dir (towards the scene)
    camera: tuple          # eye(3), target(3), up(3), fovy

    @property
    def to_light(self) -> np.ndarray:
        """lights[0].dir * -1 (src/renderer/render.cpp:33)."""
        return (-self.light).astype(F)


def _normalize(v) -> np.ndarray:
    """raw::normalize in float32, operation by operation (raw/math/vec.hpp:15-16)."""
    x, y, z = F(v[0]), F(v[1]), F(v[2])
    l = np.sqrt(F(F(F(x * x) + F(y * y)) + F(z * z)))
    if not l > 0:
        return np.array([x, y, z], F)
    inv = F(F(1.0) / l)
    return np.array([F(x * inv), F(y * inv), F(z * inv)], F)


def _quad(tris, nrms, a, b, c, d, n):
    for t in ((a, b, c), (a, c, d)):
        tris.append(np.array(t, F).reshape(9))
        nrms.append(np.array([n, n, n], F).reshape(9))


def build_test_scene(camera=DEFAULT_CAMERA) -> Scene:
    tris, nrms = [], []
    _quad(tris, nrms, (-5, 0, -5), (5, 0, -5), (5, 0, 5), (-5, 0, 5), (0, 1, 0))
    c, h = (0.0, 1.0, 0.0), 1.0
    p0 = (c[0] - h, c[1] - h, c[2] - h)
    p1 = (c[0] + h, c[1] + h, c[2] + h)
    _quad(tris, nrms, (p0[0], p0[1], p1[2]), (p1[0], p0[1], p1[2]), (p1[0], p1[1], p1[2]), (p0[0], p1[1], p1[2]), (0, 0, 1))
    _quad(tris, nrms, (p1[0], p0[1], p0[2]), (p0[0], p0[1], p0[2]), (p0[0], p1[1], p0[2]), (p1[0], p1[1], p0[2]), (0, 0, -1))
    _quad(tris, nrms, (p0[0], p1[1], p1[2]), (p1[0], p1[1], p1[2]), (p1[0], p1[1], p0[2]), (p0[0], p1[1], p0[2]), (0, 1, 0))
    _quad(tris, nrms, (p0[0], p0[1], p0[2]), (p1[0], p0[1], p0[2]), (p1[0], p0[1], p1[2]), (p0[0], p0[1], p1[2]), (0, -1, 0))
    _quad(tris, nrms, (p1[0], p0[1], p1[2]), (p1[0], p0[1], p0[2]), (p1[0], p1[1], p0[2]), (p1[0], p1[1], p1[2]), (1, 0, 0))
    _quad(tris, nrms, (p0[0], p0[1], p0[2]), (p0[0], p0[1], p1[2]), (p0[0], p1[1], p1[2]), (p0[0], p1[1], p0[2]), (-1, 0, 0))
    return Scene(np.ascontiguousarray(np.stack(tris)), np.ascontiguousarray(np.stack(nrms)),
                 _normalize((-0.4, -1.0, -0.3)), tuple(camera))


# ------------------------------------------------------------------ seeded synthetic scenes
# The large workloads use scenes this project generates (the reference has none): a ground
# grid, yawed boxes and subdivided icospheres resting on it, placed by a seeded PCG64.
#   build_synthetic_scene(seed, 2000, 500)    ~744,000 triangles (batched views)
#   build_synthetic_scene(seed, 200, 50)      146,400 triangles (surrogate training scenes)
#   build_synthetic_scene(seed, 10000, 6000)  ~7,880,000 triangles (4K head-to-head)

def _soup_hash(x: int) -> int:
    x ^= x >> 16
    x = (x * 0x7FEB352D) & 0xFFFFFFFF
    x ^= x >> 15
    x = (x * 0x846CA68B) & 0xFFFFFFFF
    return x ^ (x >> 16)


def soup(count: int, seed: int) -> np.ndarray:
    """raw::rt::soup (src/renderer/rt_scenes.cpp:52-63), the reference's PLOC check input:
    `count` triangles, each a centre uniform in [-12, 12)^3 plus three corners within +-1 of
    it, all drawn from one integer-hash sequence. (count, 9) float32."""
    r = (seed * 2654435761 + 1) & 0xFFFFFFFF
    u = np.empty(12 * count, np.float64)
    for k in range(12 * count):
        r = _soup_hash((r + 0x9E3779B9) & 0xFFFFFFFF)
        u[k] = r >> 8
    v = (u / 16777216.0).astype(np.float32).reshape(count, 4, 3)   # exact: 24-bit integers / 2^24
    c = np.float32(24.0) * v[:, 0] - np.float32(12.0)
    corners = c[:, None, :] + (np.float32(2.0) * v[:, 1:] - np.float32(1.0))
    return np.ascontiguousarray(corners.reshape(count, 9), np.float32)


def _icosphere(subdiv: int):
    """Unit icosphere: 20 * 4^subdiv triangles (vertices, faces), outward winding."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = np.array([(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
                  (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)], np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array([(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
                  (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5),
                  (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)], np.int64)
    verts = list(map(tuple, v))
    for _ in range(subdiv):
        cache = {}

        def mid(a, b):
            key = (min(a, b), max(a, b))
            if key not in cache:
                m = (np.array(verts[a]) + np.array(verts[b])) / 2.0
                verts.append(tuple(m / np.linalg.norm(m)))
                cache[key] = len(verts) - 1
            return cache[key]
        nf = []
        for a, b, c in f:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        f = np.array(nf, np.int64)
    return np.array(verts, np.float64), f


_FACES = [((0, 1, 3, 2), (0, -1, 0)), ((4, 6, 7, 5), (0, 1, 0)), ((0, 4, 5, 1), (0, 0, -1)),
          ((2, 3, 7, 6), (0, 0, 1)), ((0, 2, 6, 4), (-1, 0, 0)), ((1, 5, 7, 3), (1, 0, 0))]


def _boxes_tris(centres, sides, yaws):
    """12 triangles per box (positions and face normals, (12 n, 9) each): footprint centres
    (x, z), sides (sx, sy, sz), boxes resting on y = 0 and rotated by their yaw about the
    vertical axis."""
    n = len(centres)
    hx, hz, h = sides[:, 0] / 2.0, sides[:, 2] / 2.0, sides[:, 1]
    corners = np.empty((n, 8, 3))
    q = 0
    for yv in (0, 1):
        for zs in (-1, 1):
            for xs in (-1, 1):
                corners[:, q, 0] = hx if xs > 0 else -hx
                corners[:, q, 1] = h if yv else 0.0
                corners[:, q, 2] = hz if zs > 0 else -hz
                q += 1
    cy, sy = np.cos(yaws), np.sin(yaws)
    rot = np.zeros((n, 3, 3))
    rot[:, 0, 0], rot[:, 0, 2], rot[:, 1, 1], rot[:, 2, 0], rot[:, 2, 2] = cy, sy, 1.0, -sy, cy
    p = np.matmul(corners, rot.transpose(0, 2, 1)) + np.stack([centres[:, 0], np.zeros(n), centres[:, 1]], 1)[:, None, :]
    tris = np.empty((n, 12, 9))
    nrms = np.empty((n, 12, 9))
    t = 0
    for (a, b, cc, d), nv in _FACES:
        nr = np.matmul(rot, np.array(nv, np.float64))
        for t3 in ((a, b, cc), (a, cc, d)):
            tris[:, t] = np.concatenate([p[:, t3[0]], p[:, t3[1]], p[:, t3[2]]], 1)
            nrms[:, t] = np.concatenate([nr, nr, nr], 1)
            t += 1
    return tris.reshape(-1, 9), nrms.reshape(-1, 9)


def build_synthetic_scene(seed: int, n_boxes: int, n_spheres: int, grid: int = 200, half: float = 50.0,
                          subdiv: int = 3) -> Scene:
    rng = np.random.Generator(np.random.PCG64(seed))
    # ground: grid x grid quads on [-half, half]^2 at y = 0
    xs = np.linspace(-half, half, grid + 1)
    i, j = np.meshgrid(np.arange(grid), np.arange(grid), indexing="ij")
    x0, x1, z0, z1 = xs[i].ravel(), xs[i + 1].ravel(), xs[j].ravel(), xs[j + 1].ravel()
    zero = np.zeros_like(x0)
    a = np.stack([x0, zero, z0], 1); b = np.stack([x1, zero, z0], 1)
    c = np.stack([x1, zero, z1], 1); d = np.stack([x0, zero, z1], 1)
    ground = np.stack([np.concatenate([a, b, c], 1), np.concatenate([a, c, d], 1)], 1).reshape(-1, 9)
    # boxes
    centres = rng.uniform(-half, half, (n_boxes, 2))
    sides = rng.uniform(0.2, 3.0, (n_boxes, 3))
    yaws = rng.uniform(0.0, 2.0 * np.pi, n_boxes)
    if n_spheres:
        v, f = _icosphere(subdiv)
        unit = v[f].reshape(-1, 9)                    # (faces, 9) corner positions on the unit sphere
        sc = rng.uniform(-half, half, (n_spheres, 2))
        r = np.clip(rng.lognormal(0.0, 0.5, n_spheres), 0.2, 4.0)
    # the output arrays are filled in place: positions computed in FP64, stored as FP32
    nsph = len(unit) * n_spheres if n_spheres else 0
    total = len(ground) + 12 * n_boxes + nsph
    tris = np.empty((total, 9), np.float32)
    nrms = np.empty((total, 9), np.float32)
    tris[:len(ground)] = ground
    nrms[:len(ground)] = np.array([0, 1, 0] * 3, np.float32)
    o = len(ground)
    if n_boxes:
        t, n = _boxes_tris(centres, sides, yaws)
        tris[o:o + 12 * n_boxes] = t
        nrms[o:o + 12 * n_boxes] = n
        o += 12 * n_boxes
    # icospheres resting on the ground, centres at height r
    if n_spheres:
        off = np.tile(np.stack([sc[:, 0], r, sc[:, 1]], 1), 3)
        nf = len(unit)
        step = max(1, (1 << 20) // nf)
        for k0 in range(0, n_spheres, step):
            k1 = min(n_spheres, k0 + step)
            sph = unit[None, :, :] * r[k0:k1, None, None] + off[k0:k1, None, :]
            tris[o + k0 * nf:o + k1 * nf] = sph.reshape(-1, 9)
        nrms[o:o + nsph].reshape(n_spheres, nf, 9)[:] = unit.astype(np.float32)[None]
    return Scene(tris, nrms, _normalize((-0.4, -1.0, -0.3)), (40.0, 12.0, 0.0, 0.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.9))


RESOLUTIONS = ((512, 512), (1280, 720), (1920, 1080), (2560, 1440))
SPPS = (16, 64, 256)


def orbit_views(seed: int, n: int, radius: float = 40.0, heights=(3.0, 20.0), fovy: float = 0.9,
                resolutions=RESOLUTIONS, spps=SPPS):
    """n cameras evenly around an orbit of `radius`, heights uniform in `heights`, looking at
    the origin; each draws a resolution and an spp. Returns [(w, h, spp, camera10)]."""
    rng = np.random.Generator(np.random.PCG64(seed ^ 0x5EED))
    hs = rng.uniform(heights[0], heights[1], n)
    ri = rng.integers(0, len(resolutions), n)
    si = rng.integers(0, len(spps), n)
    views = []
    for k in range(n):
        th = 2.0 * np.pi * k / n
        cam = (float(radius * np.cos(th)), float(hs[k]), float(radius * np.sin(th)), 0.0, 0.0, 0.0, 0.0, 1.0, 0.0, fovy)
        w, h = resolutions[ri[k]]
        views.append((w, h, int(spps[si[k]]), cam))
    return views
