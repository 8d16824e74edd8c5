"""Seeded synthetic inputs for the query-path workloads (host-side, numpy).

Random numbers come from a counter-based SplitMix64 (value i of stream s = mix(seed + s*C + (i+1)*G)),
so every array is a pure function of (seed, stream, index) and identical on x86-64 and aarch64.
Workloads:
  - terrain ray casts: a (nx+1) x (nz+1) height-field TriMesh (x, z spacing 1, heights U[0, 4)),
    2 triangles per cell wound counter-clockwise seen from +y, and rays with origins
    U([0, nx) x [10, 20) x [0, nz)) and directions uniform on the downward unit hemisphere.
"""
from __future__ import annotations

import numpy as np

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_STREAM = np.uint64(0xD1B54A32D192ED03)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed: int, stream: int, n: int) -> np.ndarray:
    idx = np.arange(1, n + 1, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = np.uint64(seed & 0xFFFFFFFFFFFFFFFF) + np.uint64(stream) * _STREAM + idx * _GOLDEN
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        z = z ^ (z >> np.uint64(31))
    return z


def uniform(seed: int, stream: int, n: int, lo: float = 0.0, hi: float = 1.0) -> np.ndarray:
    """float64 values in [lo, hi) with 53-bit resolution."""
    u = (splitmix64(seed, stream, n) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
    return lo + (hi - lo) * u


def terrain_mesh(nx: int = 256, nz: int = 128, seed: int = 0x9A77E0) -> tuple[np.ndarray, np.ndarray]:
    """Height-field TriMesh: ((nx+1)*(nz+1), 3) f32 vertices and (2*nx*nz, 3) u32 indices."""
    ix, iz = np.meshgrid(np.arange(nx + 1), np.arange(nz + 1), indexing="ij")
    h = uniform(seed, 1, (nx + 1) * (nz + 1), 0.0, 4.0).reshape(nx + 1, nz + 1)
    verts = np.stack([ix.astype(np.float64), h, iz.astype(np.float64)], axis=-1).reshape(-1, 3).astype(np.float32)
    cx, cz = np.meshgrid(np.arange(nx), np.arange(nz), indexing="ij")
    cx = cx.reshape(-1).astype(np.int64)
    cz = cz.reshape(-1).astype(np.int64)
    v00 = cx * (nz + 1) + cz
    v10 = (cx + 1) * (nz + 1) + cz
    v01 = cx * (nz + 1) + cz + 1
    v11 = (cx + 1) * (nz + 1) + cz + 1
    t0 = np.stack([v00, v01, v10], axis=-1)
    t1 = np.stack([v10, v01, v11], axis=-1)
    idx = np.stack([t0, t1], axis=1).reshape(-1, 3).astype(np.uint32)
    return verts, idx


def terrain_rays(n: int, nx: int = 256, nz: int = 128, seed: int = 0x9A77E0) -> np.ndarray:
    """(n, 6) f32 rays: origin U([0,nx) x [10,20) x [0,nz)), direction on the downward hemisphere."""
    ox = uniform(seed, 2, n, 0.0, float(nx))
    oy = uniform(seed, 3, n, 10.0, 20.0)
    oz = uniform(seed, 4, n, 0.0, float(nz))
    dy = -uniform(seed, 5, n)
    phi = uniform(seed, 6, n, 0.0, 2.0 * np.pi)
    r = np.sqrt(np.maximum(0.0, 1.0 - dy * dy))
    rays = np.stack([ox, oy, oz, r * np.cos(phi), dy, r * np.sin(phi)], axis=-1)
    return rays.astype(np.float32)
