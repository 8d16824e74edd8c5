"""ConvexPolyhedron topology (the host-side input of the hull contact-manifold generators).

build_polyhedra(pool, first, count) runs ConvexPolyhedron::from_convex_hull for many point clouds
at once through libparrygpu's builder - on the GPU (parrygpu_polyhedra_build_gpu) when given a
Context, else on host threads (parrygpu_polyhedra_build) - and returns the hull points and the
topology arrays in the parrygpu_polyhedra layout (include/parry_gpu.h).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

TOPOLOGY_KEYS = ("face_normals", "face_ranges", "face_vertices", "face_edges", "vertex_ranges", "vertex_faces", "vertex_edges",
                 "edge_dirs")


def build_polyhedra(pool: np.ndarray, first: np.ndarray, count: np.ndarray, threads: int = 0, ctx=None,
                    with_triangles: bool = False, out: dict | None = None):
    """Returns (points (m, 3) f32, hulls (n, 8) u32, topology dict). hulls rows: first vertex (in
    `points`), vertex count, first face, face count, first edge, edge count, ok, 0. With a Context
    `ctx` the clouds are built on its GPU (parrygpu_polyhedra_build_gpu: the same bytes as the host
    builder), else on `threads` host threads. With `with_triangles` the topology dict also holds
    transformation::convex_hull's triangulation of every cloud: "tri_ranges" (n, 2) = first
    triangle, count and "triangles" (t, 3) of hull-local vertex ids. `out` (GPU builds, optional):
    destination arrays under the keys "points", "hulls" and the topology keys, at least as long as
    the build's (numpy arrays, or numpy views of pinned memory so that the copies run at the host
    link's speed); the returned arrays are then views of their leading rows."""
    from ._capi import lib, check
    pool = np.ascontiguousarray(pool, np.float32).reshape(-1, 3)
    first = np.ascontiguousarray(first, np.uint32)
    count = np.ascontiguousarray(count, np.uint32)
    n = len(first)
    L = lib()
    if ctx is not None:
        return _build_gpu(ctx, pool, first, count, with_triangles, out)
    h = C.c_void_p()
    check(L.parrygpu_polyhedra_build(pool.ctypes.data, first.ctypes.data, count.ctypes.data, n, int(threads), C.byref(h)))
    try:
        sizes = np.zeros(5, np.uint64)
        check(L.parrygpu_polyhedra_sizes(h, sizes.ctypes.data))
        npts, nf, nfe, nve, ne = (int(x) for x in sizes)
        points = np.zeros((npts, 3), np.float32)
        hulls = np.zeros((n, 8), np.uint32)
        topo = {
            "face_normals": np.zeros((nf, 3), np.float32), "face_ranges": np.zeros((nf, 2), np.uint32),
            "face_vertices": np.zeros(nfe, np.uint32), "face_edges": np.zeros(nfe, np.uint32),
            "vertex_ranges": np.zeros((npts, 2), np.uint32), "vertex_faces": np.zeros(nve, np.uint32),
            "vertex_edges": np.zeros(nve, np.uint32), "edge_dirs": np.zeros((ne, 3), np.float32),
        }
        check(L.parrygpu_polyhedra_copy(h, points.ctypes.data, hulls.ctypes.data, *[topo[k].ctypes.data for k in TOPOLOGY_KEYS]))
        if with_triangles:
            nt = C.c_uint64()
            check(L.parrygpu_polyhedra_triangles(h, C.byref(nt), None, None))
            topo["tri_ranges"] = np.zeros((n, 2), np.uint32)
            topo["triangles"] = np.zeros((nt.value, 3), np.uint32)
            check(L.parrygpu_polyhedra_triangles(h, None, topo["tri_ranges"].ctypes.data if n else None,
                                                 topo["triangles"].ctypes.data if nt.value else None))
    finally:
        L.parrygpu_polyhedra_builder_destroy(h)
    return points, hulls, topo


def _build_gpu(ctx, pool, first, count, with_triangles=False, out=None):
    from ._capi import lib, check
    L = lib()
    n = len(first)
    h = C.c_void_p()
    check(L.parrygpu_polyhedra_build_gpu(ctx.handle, C.c_void_p(pool.ctypes.data) if len(pool) else None, len(pool),
                                         C.c_void_p(first.ctypes.data) if n else None, C.c_void_p(count.ctypes.data) if n else None,
                                         n, C.byref(h)), ctx.handle)
    try:
        sizes = np.zeros(5, np.uint64)
        check(L.parrygpu_polyhedra_gpu_sizes(h, C.c_void_p(sizes.ctypes.data)))
        npts, nf, nfe, nve, ne = (int(x) for x in sizes)
        rows = {"points": npts, "hulls": n, "face_normals": nf, "face_ranges": nf, "face_vertices": nfe, "face_edges": nfe,
                "vertex_ranges": npts, "vertex_faces": nve, "vertex_edges": nve, "edge_dirs": ne}
        if out is not None:
            for k, m in rows.items():
                if len(out[k]) < m:
                    raise ValueError(f"out[{k!r}] holds {len(out[k])} rows, the build needs {m}")
            points, hulls = out["points"][:npts], out["hulls"][:n]
            topo = {k: out[k][:rows[k]] for k in TOPOLOGY_KEYS}
        else:
            points = np.empty((npts, 3), np.float32)
            hulls = np.empty((n, 8), np.uint32)
            topo = {
                "face_normals": np.empty((nf, 3), np.float32), "face_ranges": np.empty((nf, 2), np.uint32),
                "face_vertices": np.empty(nfe, np.uint32), "face_edges": np.empty(nfe, np.uint32),
                "vertex_ranges": np.empty((npts, 2), np.uint32), "vertex_faces": np.empty(nve, np.uint32),
                "vertex_edges": np.empty(nve, np.uint32), "edge_dirs": np.empty((ne, 3), np.float32),
            }
        ptr = lambda a: C.c_void_p(a.ctypes.data) if a.size else None
        check(L.parrygpu_polyhedra_gpu_copy(ctx.handle, h, ptr(points), ptr(hulls), *[ptr(topo[k]) for k in TOPOLOGY_KEYS]), ctx.handle)
        if with_triangles:
            nt = C.c_uint64()
            check(L.parrygpu_polyhedra_gpu_triangles(ctx.handle, h, C.byref(nt), None, None), ctx.handle)
            topo["tri_ranges"] = np.zeros((n, 2), np.uint32)
            topo["triangles"] = np.zeros((nt.value, 3), np.uint32)
            check(L.parrygpu_polyhedra_gpu_triangles(ctx.handle, h, None, ptr(topo["tri_ranges"]), ptr(topo["triangles"])),
                  ctx.handle)
    finally:
        L.parrygpu_polyhedra_gpu_destroy(h)
    return points, hulls, topo


def empty_topology() -> dict:
    return {"face_normals": np.zeros((0, 3), np.float32), "face_ranges": np.zeros((0, 2), np.uint32),
            "face_vertices": np.zeros(0, np.uint32), "face_edges": np.zeros(0, np.uint32),
            "vertex_ranges": np.zeros((0, 2), np.uint32), "vertex_faces": np.zeros(0, np.uint32),
            "vertex_edges": np.zeros(0, np.uint32), "edge_dirs": np.zeros((0, 3), np.float32)}
