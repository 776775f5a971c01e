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
