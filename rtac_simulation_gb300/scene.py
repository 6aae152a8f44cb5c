"""Synthetic meshes and cameras for the rasterised echo samples
(rtacx_rasterize). The reference's own scenes need private models; these are
small procedural stand-ins: a seafloor grid below the sensor and a sphere."""
from __future__ import annotations

import math

import numpy as np


def perspective(fovy_deg: float, aspect: float, near: float, far: float) -> np.ndarray:
    """OpenGL-style perspective projection (row-major, p' = M p)."""
    f = 1.0 / math.tan(math.radians(fovy_deg) / 2.0)
    return np.array([[f / aspect, 0, 0, 0],
                     [0, f, 0, 0],
                     [0, 0, (far + near) / (near - far), 2 * far * near / (near - far)],
                     [0, 0, -1, 0]], dtype=np.float64)


def _grid_triangles(rows: int, quads: int, cols: int, split) -> np.ndarray:
    """Two triangles per quad of a rows x quads grid of vertices laid out with
    `cols` vertices per row, quad by quad in row order; split(a, b, c, d)
    gives the two triangles of the quad with corners a (r, q), b (r, q+1),
    c (r+1, q), d (r+1, q+1)."""
    r, q = np.meshgrid(np.arange(rows, dtype=np.int64), np.arange(quads, dtype=np.int64), indexing="ij")
    a = (r * cols + q).ravel()
    t0, t1 = split(a, a + 1, a + cols, a + cols + 1)
    return np.stack([np.stack(t0, axis=1), np.stack(t1, axis=1)], axis=1).reshape(-1, 3)


def seafloor_and_sphere(grid: int = 40, depth: float = 3.0, extent: float = 20.0, length: float = 40.0,
                        sphere_center=(2.0, -1.0, -10.0), radius: float = 1.5, sphere_steps: int = 24):
    """(vertices [n][3], normals [n][3], triangles [m][3]) in a camera frame
    looking along -z: a plane y = -depth over x in [-extent, extent],
    z in [-length, -0.5], plus a UV sphere."""
    xs = np.linspace(-extent, extent, grid + 1)
    zs = np.linspace(-length, -0.5, grid + 1)
    X, Z = np.meshgrid(xs, zs)
    pv = np.stack([X.ravel(), np.full(X.size, -depth), Z.ravel()], axis=1)
    pn = np.tile([0.0, 1.0, 0.0], (pv.shape[0], 1))
    pt = _grid_triangles(grid, grid, grid + 1, lambda a, b, c_, d: ((a, c_, b), (b, c_, d)))
    th = np.linspace(0, math.pi, sphere_steps + 1)
    ph = np.linspace(0, 2 * math.pi, 2 * sphere_steps + 1)
    T, P = np.meshgrid(th, ph, indexing="ij")
    n = np.stack([np.sin(T) * np.cos(P), np.cos(T), np.sin(T) * np.sin(P)], axis=-1).reshape(-1, 3)
    sv = np.asarray(sphere_center) + radius * n
    st = _grid_triangles(sphere_steps, 2 * sphere_steps, 2 * sphere_steps + 1,
                         lambda a, b, c_, d: ((a, b, c_), (b, d, c_))) + pv.shape[0]
    V = np.concatenate([pv, sv]).astype(np.float32)
    N = np.concatenate([pn, n]).astype(np.float32)
    return V, N, np.concatenate([pt, st]).astype(np.uint32)
