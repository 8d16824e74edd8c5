"""Generates tests/golden/terrain_small.npz: a small terrain TriMesh, seeded rays and the oracle's
f32 (parry3d) and f64 (parry3d-f64) answers. Re-run after an intentional oracle change:

    python tests/golden/make_golden.py

The fixture pins the oracle across machines (x86-64 here, aarch64 on the GPU host) and gives the
GPU parity test committed vectors to compare against.
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import build as ob  # noqa: E402
from oracle import oracle as O  # noqa: E402
from parry_gb300 import workloads as W  # noqa: E402


def main():
    ob.build()
    v, i = W.terrain_mesh(16, 8, seed=7)
    rays = W.terrain_rays(2048, 16, 8, seed=7)
    # a few axis-aligned rays (exact zero direction components exercise the slab special case)
    extra = np.array([[3.5, 15.0, 2.5, 0.0, -1.0, 0.0],
                      [0.0, 12.0, 0.0, 0.0, -1.0, 0.0],
                      [7.25, 11.0, 4.75, 1.0, -1.0, 0.0],
                      [15.9, 10.5, 7.9, 0.0, -1.0, 1.0]], dtype=np.float32)
    rays = np.concatenate([rays, extra]).astype(np.float32)
    m32 = O.TriMesh(v, i, "f32")
    m64 = O.TriMesh(v, i, "f64")
    f32, t32, n32 = m32.cast_rays_and_get_normal(rays, 100.0, threads=1)
    f64, t64, n64 = m64.cast_rays_and_get_normal(rays, 100.0, threads=1)
    out = Path(__file__).resolve().parent / "terrain_small.npz"
    np.savez_compressed(out, vertices=v, indices=i, rays=rays, max_toi=np.float32(100.0),
                        feature_f32=f32, toi_f32=t32, normal_f32=n32, feature_f64=f64, toi_f64=t64, normal_f64=n64)
    print(out, "hits:", int((f32 != 0xFFFFFFFF).sum()), "of", len(rays))


if __name__ == "__main__":
    main()
