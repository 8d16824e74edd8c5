"""parry_gb300 — GB300-native batched replacement for parry3d's data-parallel query path.

The Python surface mirrors the reference API names so that a CPU loop over parry calls maps onto
one batched call here:

    parry3d                                            parry_gb300
    -------------------------------------------------  ------------------------------------------------
    Bvh::from_leaves(strategy, &aabbs)                 Bvh.from_leaves(ctx, aabbs)
    Bvh::refit(&mut ws) (+ insert_or_update_partially) Bvh.refit(aabbs)
    Bvh::traverse_bvtt_single_tree(&mut ws, &mut f)    Bvh.traverse_bvtt_single_tree() -> (k, 2) pairs
    Bvh::leaf_pairs(&other, check)                     Bvh.leaf_pairs(other) -> (k, 2) pairs
    TriMesh::new(vertices, indices)                    TriMesh(ctx, vertices, indices)
    TriMesh::cast_ray_and_get_normal(m, ray, t, solid) TriMesh.cast_rays_and_get_normal(rays, t, solid, pose)
    TriMesh::cast_ray(m, ray, t, solid)                TriMesh.cast_rays(rays, t, solid, pose)
    Shape::compute_aabb(pos).loosened(m)               shape_aabbs(ctx, shapes, margin)
    query::contact(pos1, g1, pos2, g2, prediction)     contacts(ctx, shapes, pairs, prediction, init_dirs)
    dispatcher.contact_manifold_convex_convex(...)     contact_manifolds(ctx, shapes, pairs, prediction, manifolds)
    a physics step's queries on moving shapes          Scene(ctx, shapes, velocities, prediction, capacity).step(dt, frames)
    Compound::new(shapes)                              Compound(ctx, shapes)
    Compound::cast_ray_and_get_normal(m, ray, t, s)    Compound.cast_rays_and_get_normal(rays, t, solid, pose)

Arrays may be numpy arrays (host memory, staged by the library) or torch tensors (CUDA tensors are
used in place; outputs are then allocated on the same device). Every call goes through the C ABI
of libparrygpu.so (include/parry_gpu.h); there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _capi
from ._capi import ParryGpuError, lib, check

__all__ = ["Context", "Bvh", "TriMesh", "Compound", "ShapeSet", "Scene", "WarmStartMLP", "shape_aabbs", "contacts", "contact_manifolds",
           "new_manifolds", "ParryGpuError", "NO_HIT", "lib"]

from .shapes import ShapeSet  # noqa: E402
from .manifold import new_manifolds, MANIFOLD_DTYPE, RECORD_WORDS  # noqa: E402

NO_HIT = 0xFFFFFFFF

try:  # torch is optional plumbing (device memory, streams); numpy inputs work without it.
    import torch
except Exception:  # pragma: no cover
    torch = None


def _is_torch(x) -> bool:
    return torch is not None and isinstance(x, torch.Tensor)


def _as_input(x, dtype):
    """Returns (keepalive, pointer) for an input array (numpy or torch), C-contiguous."""
    if x is None:
        return None, None
    if _is_torch(x):
        tdt = {np.float32: torch.float32, np.uint32: torch.int32, np.uint8: torch.uint8}[dtype]
        if x.dtype != tdt and not (dtype is np.uint32 and x.dtype in (torch.int32, torch.uint32)):
            x = x.to(tdt)
        x = x.contiguous()
        return x, C.c_void_p(x.data_ptr())
    a = np.ascontiguousarray(x, dtype=dtype)
    return a, C.c_void_p(a.ctypes.data)


def _alloc_like(ref, shape, dtype):
    """Allocates an output on the same side (numpy / torch CPU / torch CUDA) as `ref`."""
    if _is_torch(ref):
        tdt = {np.float32: torch.float32, np.uint32: torch.int32, np.uint8: torch.uint8}[dtype]
        pin = ref.device.type == "cpu" and ref.is_pinned()
        t = torch.empty(shape, dtype=tdt, device=ref.device, pin_memory=pin)
        return t, C.c_void_p(t.data_ptr())
    a = np.empty(shape, dtype=dtype)
    return a, C.c_void_p(a.ctypes.data)


def _config_dict(cfg) -> dict:
    return {"device": cfg.device, "ray_block": cfg.ray_block, "sort_rays": bool(cfg.sort_rays), "ray_sort_key": cfg.ray_sort_key,
            "epa_blocks_per_sm": cfg.epa_blocks_per_sm, "ray_traversal": cfg.ray_traversal, "ray_refill": cfg.ray_refill, "ray_chunks": cfg.ray_chunks,
            "ray_host_access": cfg.ray_host_access, "contact_warp_cost": cfg.contact_warp_cost,
            "contact_epa_inline": cfg.contact_epa_inline, "mlp_infer": cfg.mlp_infer,
            "scene_ray_order": cfg.scene_ray_order,
            "scene_ray_grid": cfg.scene_ray_grid}


class Context:
    """A device context (one CUDA stream). Mirrors nothing in parry, which is single-threaded CPU."""

    def __init__(self, device: int = 0, ray_block: int = 0, sort_rays: bool = True, ray_sort_key: int = 0,
                 epa_blocks_per_sm: int = 0, ray_traversal: int = 0, ray_refill: int = 0, ray_chunks: int = 0,
                 ray_host_access: int = 0, contact_warp_cost: int = 0, contact_epa_inline: int = 0,
                 mlp_infer: int = 0, scene_ray_order: int = 0,
                 scene_ray_grid: int = 0):
        cfg = _capi.ParryGpuConfig()
        lib().parrygpu_default_config(C.byref(cfg))
        cfg.device = device
        cfg.ray_block = ray_block
        cfg.sort_rays = 1 if sort_rays else 0
        cfg.ray_sort_key = ray_sort_key
        cfg.epa_blocks_per_sm = epa_blocks_per_sm
        cfg.ray_traversal = ray_traversal
        cfg.ray_refill = ray_refill
        cfg.ray_chunks = ray_chunks
        cfg.ray_host_access = ray_host_access
        cfg.contact_warp_cost = contact_warp_cost
        cfg.contact_epa_inline = contact_epa_inline
        cfg.mlp_infer = mlp_infer
        cfg.scene_ray_order = scene_ray_order
        cfg.scene_ray_grid = scene_ray_grid
        h = C.c_void_p()
        check(lib().parrygpu_create(C.byref(h), C.byref(cfg)))
        self._h = h
        self.device = device

    @property
    def handle(self):
        return self._h

    def set_stream(self, stream_ptr: int | None) -> None:
        check(lib().parrygpu_set_stream(self._h, C.c_void_p(stream_ptr or 0)), self._h)

    def sync(self) -> None:
        check(lib().parrygpu_sync(self._h), self._h)

    @property
    def kernel_launches(self) -> int:
        return int(lib().parrygpu_kernel_launches(self._h))

    def enable_kernel_timing(self, on: bool = True) -> None:
        check(lib().parrygpu_enable_kernel_timing(self._h, 1 if on else 0), self._h)

    def reset_kernel_timing(self) -> None:
        check(lib().parrygpu_reset_kernel_timing(self._h), self._h)

    def kernel_time(self, kernel: str) -> tuple[float, int]:
        """(total ms, launches) of the event-timed launches of `kernel` since the last reset."""
        ms, n = C.c_double(0.0), C.c_uint64(0)
        check(lib().parrygpu_kernel_time(self._h, kernel.encode(), C.byref(ms), C.byref(n)), self._h)
        return ms.value, n.value

    @property
    def config(self) -> dict:
        """The context's launch configuration (parrygpu_config fields)."""
        cfg = _capi.ParryGpuConfig()
        check(lib().parrygpu_get_config(self._h, C.byref(cfg)), self._h)
        return _config_dict(cfg)

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().parrygpu_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _pairs_call(ctx: Context, fn, args, sorted_: bool, cap_hint: int):
    cap = max(int(cap_hint), 1024)
    while True:
        out = np.empty((cap, 2), dtype=np.uint32)
        n = C.c_uint64(0)
        st = fn(ctx.handle, *args, C.c_void_p(out.ctypes.data), C.c_uint64(cap), C.byref(n), 1 if sorted_ else 0)
        if st == 3 and n.value > cap:  # capacity exceeded: retry with the exact count
            cap = int(n.value)
            continue
        check(st, ctx.handle)
        return out[: n.value]


class Bvh:
    """partitioning::Bvh on the GPU: LBVH built from 30-bit Morton codes (see include/parry_gpu.h)."""

    def __init__(self, ctx: Context, handle):
        self.ctx = ctx
        self._h = handle

    @classmethod
    def from_leaves(cls, ctx: Context, aabbs) -> "Bvh":
        """Bvh::from_leaves: `aabbs` is (n, 6) = mins xyz, maxs xyz; leaf data = row index."""
        keep, p = _as_input(aabbs, np.float32)
        n = int(keep.shape[0]) if keep is not None else 0
        h = C.c_void_p()
        check(lib().parrygpu_bvh_build(ctx.handle, p, n, C.byref(h)), ctx.handle)
        return cls(ctx, h)

    @classmethod
    def from_serialized(cls, ctx: Context, nodes) -> "Bvh":
        """A tree in the reference's serialised layout (Bvh::nodes, BvhNodeWide records: (n_wide, 16)
        float32 words or 64-byte rows), e.g. one built by parry; parents and leaf positions are
        derived on the device."""
        raw = np.ascontiguousarray(nodes)
        raw = raw.view(np.float32).reshape(-1, 16) if raw.size else np.zeros((0, 16), np.float32)
        h = C.c_void_p()
        check(lib().parrygpu_bvh_import(ctx.handle, C.c_void_p(raw.ctypes.data) if len(raw) else None, len(raw), C.byref(h)), ctx.handle)
        return cls(ctx, h)

    def serialize(self, leaf_capacity: int | None = None):
        """The reference's serialised Bvh: (nodes (n_wide, 16) f32 words in BvhNodeWide layout,
        parents (n_wide,) u64 BvhNodeIndex, leaf_node_indices (leaf_capacity,) u64 BvhNodeIndex per
        leaf index, 2**64 - 1 where no leaf has that index)."""
        lc, wc = self.info()
        cap = int(leaf_capacity) if leaf_capacity is not None else self.id_bound()
        nodes = np.zeros((wc, 16), np.float32)
        parents = np.zeros(wc, np.uint64)
        leaves = np.zeros(cap, np.uint64)
        check(lib().parrygpu_bvh_export(self.ctx.handle, self._h, C.c_void_p(nodes.ctypes.data) if wc else None,
                                        C.c_void_p(parents.ctypes.data) if wc else None, C.c_void_p(leaves.ctypes.data) if cap else None,
                                        cap), self.ctx.handle)
        return nodes, parents, leaves

    def id_bound(self) -> int:
        """1 + the largest leaf index (the row count refit() expects)."""
        nodes = self.nodes()
        if len(nodes) == 0:
            return 0
        w = nodes.view(np.uint32)
        leaf = (w[:, [7, 15]] & 0x3FFFFFFF) == 1
        ids = w[:, [3, 11]][leaf]
        return int(ids.max()) + 1 if len(ids) else 0

    def insert(self, aabbs, leaf_ids) -> None:
        """Bvh::insert for each (aabb, leaf index) row: new indices are added, existing ones get the
        new AABB (the last row wins). The tree is rebuilt over the resulting leaves; refit() then
        takes AABBs indexed by leaf index."""
        ka, pa = _as_input(aabbs, np.float32)
        ki, pi = _as_input(leaf_ids, np.uint32)
        k = int(ki.shape[0]) if ki is not None else 0
        check(lib().parrygpu_bvh_insert(self.ctx.handle, self._h, pa, pi, k), self.ctx.handle)

    def remove(self, leaf_ids) -> None:
        """Bvh::remove for each leaf index (indices without a leaf are ignored)."""
        ki, pi = _as_input(leaf_ids, np.uint32)
        k = int(ki.shape[0]) if ki is not None else 0
        check(lib().parrygpu_bvh_remove(self.ctx.handle, self._h, pi, k), self.ctx.handle)

    def rebuild(self, aabbs) -> None:
        """Bvh::from_leaves over new AABBs into this handle (its device storage is reused)."""
        ka, pa = _as_input(aabbs, np.float32)
        check(lib().parrygpu_bvh_rebuild(self.ctx.handle, self._h, pa, int(ka.shape[0])), self.ctx.handle)

    def refit(self, aabbs) -> None:
        """insert_or_update_partially for every leaf, then Bvh::refit (topology kept)."""
        keep, p = _as_input(aabbs, np.float32)
        check(lib().parrygpu_bvh_refit(self.ctx.handle, self._h, p), self.ctx.handle)

    def info(self) -> tuple[int, int]:
        lc, wc = C.c_uint32(0), C.c_uint32(0)
        check(lib().parrygpu_bvh_info(self._h, C.byref(lc), C.byref(wc)))
        return lc.value, wc.value

    def leaf_count(self) -> int:
        return self.info()[0]

    def nodes(self) -> np.ndarray:
        """Wide nodes as a structured array in the reference's BvhNodeWide layout."""
        _, wc = self.info()
        raw = np.empty(wc * 16, dtype=np.float32)
        if wc:
            check(lib().parrygpu_bvh_copy_nodes(self.ctx.handle, self._h, C.c_void_p(raw.ctypes.data)), self.ctx.handle)
        return raw.reshape(wc, 16)

    def traverse_bvtt_single_tree(self, sorted: bool = True, cap_hint: int | None = None) -> np.ndarray:
        """All intersecting leaf pairs (each unordered pair once) as canonical (min, max) rows."""
        hint = cap_hint if cap_hint is not None else 4 * self.leaf_count()
        return _pairs_call(self.ctx, lib().parrygpu_bvh_self_pairs, (self._h,), sorted, hint)

    def traverse_bvtt_single_tree_into(self, out, sorted: bool = False) -> int:
        """The same pairs written into `out` ((cap, 2) u32 / int32, host or device); returns the total
        pair count (raises CAPACITY_EXCEEDED when it is above cap, with the count in the message)."""
        n = C.c_uint64(0)
        st = lib().parrygpu_bvh_self_pairs(self.ctx.handle, self._h, C.c_void_p(_dptr(out)), C.c_uint64(int(out.shape[0])), C.byref(n),
                                           1 if sorted else 0)
        if st == 3:
            raise RuntimeError(f"pair capacity {int(out.shape[0])} exceeded: {n.value} pairs")
        check(st, self.ctx.handle)
        return int(n.value)

    def leaf_pairs(self, other: "Bvh", sorted: bool = True, cap_hint: int | None = None) -> np.ndarray:
        """Bvh::leaf_pairs(&other, aabb-intersection check) as (leaf of self, leaf of other) rows."""
        hint = cap_hint if cap_hint is not None else 4 * max(self.leaf_count(), other.leaf_count())
        return _pairs_call(self.ctx, lib().parrygpu_bvh_leaf_pairs, (self._h, other._h), sorted, hint)

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().parrygpu_bvh_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# TriMeshFlags bits (src/shape/trimesh.rs:470-507) accepted by TriMesh(..., flags=) / set_flags.
TRIMESH_ORIENTED = 1 << 3
TRIMESH_MERGE_DUPLICATE_VERTICES = 1 << 4
TRIMESH_FIX_INTERNAL_EDGES = (1 << 7) | (1 << 4)


class TriMesh:
    """shape::TriMesh: vertices (n_v, 3) f32, indices (n_t, 3) u32, optional TriMeshFlags
    (TriMesh::with_flags; FIX_INTERNAL_EDGES computes the triangles' pseudo-normals, which then
    constrain contact-manifold normals against the mesh)."""

    def __init__(self, ctx: Context, vertices, indices, flags: int = 0):
        kv, pv = _as_input(vertices, np.float32)
        ki, pi = _as_input(indices, np.uint32)
        self.ctx = ctx
        self.n_vertices = int(kv.shape[0])
        self.n_triangles = int(ki.shape[0])
        h = C.c_void_p()
        check(lib().parrygpu_trimesh_create(ctx.handle, pv, self.n_vertices, pi, self.n_triangles, C.byref(h)), ctx.handle)
        self._h = h
        self.flags = 0
        if flags:
            self.set_flags(flags)

    def set_flags(self, flags: int) -> None:
        """TriMesh::set_flags for ORIENTED / MERGE_DUPLICATE_VERTICES / FIX_INTERNAL_EDGES."""
        check(lib().parrygpu_trimesh_set_flags(self.ctx.handle, self._h, int(flags)), self.ctx.handle)
        self.flags = int(flags)

    def normal_constraints(self):
        """TriMesh::triangle_normal_constraints of every triangle: ((n_t, 12) f32 rows = face normal,
        pseudo-normals of edges 01, 12, 20; (n_t,) bool, False where the reference returns None)."""
        pn = np.zeros((self.n_triangles, 12), np.float32)
        ok = np.zeros(self.n_triangles, np.uint8)
        check(lib().parrygpu_trimesh_normal_constraints(self.ctx.handle, self._h, C.c_void_p(pn.ctypes.data),
                                                        C.c_void_p(ok.ctypes.data)), self.ctx.handle)
        return pn, ok.astype(bool)

    def _cast(self, rays, max_toi, solid, pose, want_normal, out=None):
        kr, pr = _as_input(rays, np.float32)
        n = int(kr.shape[0])
        kp, pp = _as_input(pose, np.float32) if pose is not None else (None, None)
        if out is None:
            feat, pf = _alloc_like(kr, (n,), np.uint32)
            toi, pt = _alloc_like(kr, (n,), np.float32)
            nrm, pn = _alloc_like(kr, (n, 3), np.float32) if want_normal else (None, None)
        else:
            feat, toi, nrm = out
            pf, pt = C.c_void_p(_dptr(feat)), C.c_void_p(_dptr(toi))
            pn = C.c_void_p(_dptr(nrm)) if (want_normal and nrm is not None) else None
        check(lib().parrygpu_trimesh_cast_rays(self.ctx.handle, self._h, pp, pr, n, float(max_toi), 1 if solid else 0,
                                               pf, pt, pn), self.ctx.handle)
        return feat, toi, nrm

    def cast_rays_and_get_normal(self, rays, max_toi: float, solid: bool = True, pose=None, out=None):
        """Batched RayCast::cast_ray_and_get_normal. Returns (feature, toi, normal):
        feature = triangle (front face), triangle + n_triangles (back face) or NO_HIT."""
        return self._cast(rays, max_toi, solid, pose, True, out)

    def autotune(self, rays, max_toi: float, pose=None, reps: int = 3) -> dict:
        """Times this mesh's ray cast on `rays` for each candidate ray ordering and block size and
        keeps the fastest in the context's configuration; returns the chosen configuration."""
        kr, pr = _as_input(rays, np.float32)
        kp, pp = _as_input(pose, np.float32) if pose is not None else (None, None)
        cfg = _capi.ParryGpuConfig()
        check(lib().parrygpu_autotune_trimesh_rays(self.ctx.handle, self._h, pp, pr, int(kr.shape[0]), float(max_toi), int(reps),
                                                   C.byref(cfg)), self.ctx.handle)
        return _config_dict(cfg)

    def cast_rays(self, rays, max_toi: float, solid: bool = True, pose=None, out=None):
        """Batched RayCast::cast_ray (toi only). Returns (feature, toi)."""
        f, t, _ = self._cast(rays, max_toi, solid, pose, False, out)
        return f, t

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().parrygpu_trimesh_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _dptr(x) -> int:
    if _is_torch(x):
        return x.data_ptr()
    return x.ctypes.data


class _StagedShapes:
    """Keeps the arrays of a ShapeSet (or of device tensors) alive behind a parrygpu_shapes struct."""

    def __init__(self, shapes):
        poly = None
        if isinstance(shapes, ShapeSet):
            t, prm, pos, pool = shapes.arrays()
            poly = shapes.polyhedra()
        elif len(shapes) == 5:
            t, prm, pos, pool, poly = shapes
        else:
            t, prm, pos, pool = shapes
        kt, pt = _as_input(t, np.uint32)
        kp, pp = _as_input(prm, np.float32)
        kq, pq = _as_input(pos, np.float32)
        kv, pv = _as_input(pool, np.float32)
        self.keep = [kt, kp, kq, kv]
        self.n = int(kt.shape[0])
        self.poly_struct = None
        poly_ptr = None
        if poly is not None:
            hulls, topo = poly
            ptrs = {}
            for name, arr, dt in [("hulls", hulls, np.uint32)] + [(k, topo[k], np.float32 if k in ("face_normals", "edge_dirs")
                                                                   else np.uint32) for k in topo]:
                ka, pa = _as_input(arr, dt)
                self.keep.append(ka)
                size = ka.numel() if _is_torch(ka) else ka.size
                ptrs[name] = pa.value if (pa is not None and size) else None
            self.poly_struct = _capi.ParryGpuPolyhedra(
                int(hulls.shape[0]), ptrs["hulls"], int(topo["face_normals"].shape[0]), ptrs["face_normals"], ptrs["face_ranges"],
                int(topo["face_vertices"].shape[0]), ptrs["face_vertices"], ptrs["face_edges"], ptrs["vertex_ranges"],
                int(topo["vertex_faces"].shape[0]), ptrs["vertex_faces"], ptrs["vertex_edges"], int(topo["edge_dirs"].shape[0]),
                ptrs["edge_dirs"])
            poly_ptr = C.cast(C.pointer(self.poly_struct), C.c_void_p).value
        self.struct = _capi.ParryGpuShapes(self.n, pt.value if pt else None, pp.value if pp else None,
                                           pq.value if pq else None, pv.value if (pv and kv.shape[0]) else None,
                                           int(kv.shape[0]) if kv is not None else 0, poly_ptr)
        self.ref = kq


def shape_aabbs(ctx: Context, shapes, margin: float = 0.0, out=None):
    """Shape::compute_aabb(pos).loosened(margin) for every shape: (n, 6) = mins, maxs."""
    st = _StagedShapes(shapes)
    if out is None:
        out, po = _alloc_like(st.ref, (st.n, 6), np.float32)
    else:
        po = C.c_void_p(_dptr(out))
    check(lib().parrygpu_shapes_aabbs(ctx.handle, C.byref(st.struct), float(margin), po), ctx.handle)
    return out


def contacts(ctx: Context, shapes, pairs, prediction: float, init_dirs=None, want_stats: bool = False, out=None,
             final_dirs=None):
    """Batched query::contact over the (a, b) rows of `pairs`.

    Returns (has_contact u8 (k,), contacts f32 (k, 13) = point1, point2, normal1, normal2, dist)
    [, stats dict]. `final_dirs` (k x 3 buffer) receives the direction GJK/EPA ended with."""
    st = _StagedShapes(shapes)
    kp, pp = _as_input(pairs, np.uint32)
    k = int(kp.shape[0]) if kp is not None else 0
    ki, pi = _as_input(init_dirs, np.float32) if init_dirs is not None else (None, None)
    if out is None:
        res, pr = _alloc_like(kp, (k, 13), np.float32)
        if _is_torch(kp):
            has = torch.empty(k, dtype=torch.uint8, device=kp.device, pin_memory=kp.device.type == "cpu" and kp.is_pinned())
            ph = C.c_void_p(has.data_ptr())
        else:
            has = np.empty(k, np.uint8)
            ph = C.c_void_p(has.ctypes.data)
    else:
        has, res = out
        ph, pr = C.c_void_p(_dptr(has)), C.c_void_p(_dptr(res))
    stats = _capi.ParryGpuGjkStats()
    pd = C.c_void_p(_dptr(final_dirs)) if final_dirs is not None else None
    check(lib().parrygpu_contacts_with_dirs(ctx.handle, C.byref(st.struct), pp, k, float(prediction), pi, pr, ph,
                                            C.byref(stats) if want_stats else None, pd), ctx.handle)
    if want_stats:
        return has, res, {"gjk_iters": stats.gjk_iterations, "epa_iters": stats.epa_iterations, "epa_calls": stats.epa_calls}
    return has, res


class TriMeshContacts:
    """contact_manifolds_trimesh_shape for n_shapes shapes against one TriMesh, frame after frame
    (the workspace and the per-triangle ContactManifolds live on the device). update() runs one
    frame; read() returns (counts (n,), triangles (n, K) u32, manifolds (n, K) MANIFOLD_DTYPE),
    slot j of shape s valid for j < counts[s]; shape 1 of each manifold is the triangle."""

    def __init__(self, ctx: Context, mesh: TriMesh, n_shapes: int, max_per_shape: int = 64):
        self.ctx, self.mesh, self.n, self.k = ctx, mesh, int(n_shapes), int(max_per_shape)
        h = C.c_void_p()
        check(lib().parrygpu_trimesh_contacts_create(ctx.handle, mesh._h, self.n, self.k, C.byref(h)), ctx.handle)
        self._h = h

    def update(self, shapes, prediction: float, mesh_pose=None) -> None:
        st = _StagedShapes(shapes)
        pp = None
        if mesh_pose is not None:
            self._pose = np.ascontiguousarray(mesh_pose, np.float32).reshape(7)
            pp = C.c_void_p(self._pose.ctypes.data)
        check(lib().parrygpu_trimesh_contacts_update(self.ctx.handle, self._h, pp, C.byref(st.struct), float(prediction)), self.ctx.handle)
        self._staged = st  # keep device inputs alive until the next update

    def read(self):
        counts = np.empty(self.n, np.uint32)
        tris = np.empty((self.n, self.k), np.uint32)
        recs = np.zeros(self.n * self.k, MANIFOLD_DTYPE)
        check(lib().parrygpu_trimesh_contacts_read(self.ctx.handle, self._h, C.c_void_p(counts.ctypes.data), C.c_void_p(tris.ctypes.data),
                                                   C.c_void_p(recs.ctypes.data)), self.ctx.handle)
        return counts, tris, recs.reshape(self.n, self.k)

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().parrygpu_trimesh_contacts_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def project_local_normals(ctx: Context, pseudo, dirs):
    """TrianglePseudoNormals::project_local_normal per row: pseudo (n, 12) f32 (face, e01, e12, e20),
    dirs (n, 3) f32. Returns (projected (n, 3) f32, ok (n,) bool; False = None)."""
    pn = np.ascontiguousarray(pseudo, np.float32).reshape(-1, 12)
    d = np.ascontiguousarray(dirs, np.float32).reshape(-1, 3)
    if len(pn) != len(d):
        raise ValueError("one pseudo-normal row per direction")
    out = np.zeros_like(d)
    ok = np.zeros(len(d), np.uint8)
    check(lib().parrygpu_project_local_normals(ctx.handle, C.c_void_p(pn.ctypes.data), C.c_void_p(d.ctypes.data), len(d),
                                               C.c_void_p(out.ctypes.data), C.c_void_p(ok.ctypes.data)), ctx.handle)
    return out, ok.astype(bool)


CAST_NONE = 255


def cast_shapes(ctx: Context, shapes, pairs, velocities, max_toi: float = float(np.finfo(np.float32).max),
                target_distance: float = 0.0, stop_at_penetration: bool = True, compute_impact_geometry_on_penetration: bool = True,
                want_stats: bool = False, out=None):
    """Batched query::cast_shapes over the (a, b) rows of `pairs`; velocities = per-shape linear
    velocities (n, 3). Returns (status u8 (k,) = ShapeCastStatus or CAST_NONE, hits f32 (k, 13) =
    toi, witness1, witness2, normal1, normal2 in each shape's local frame) [, stats dict]."""
    st = _StagedShapes(shapes)
    kp, pp = _as_input(pairs, np.uint32)
    kv, pv = _as_input(velocities, np.float32)
    k = int(kp.shape[0]) if kp is not None else 0
    if out is None:
        res, pr = _alloc_like(kp, (k, 13), np.float32)
        status, ps = _alloc_like(kp, (k,), np.uint8)
    else:
        status, res = out
        ps, pr = C.c_void_p(_dptr(status)), C.c_void_p(_dptr(res))
    opts = _capi.ParryGpuShapeCastOptions(float(max_toi), float(target_distance), 1 if stop_at_penetration else 0,
                                          1 if compute_impact_geometry_on_penetration else 0)
    stats = _capi.ParryGpuGjkStats()
    check(lib().parrygpu_cast_shapes(ctx.handle, C.byref(st.struct), pp, k, pv, C.byref(opts), pr, ps,
                                     C.byref(stats) if want_stats else None), ctx.handle)
    if want_stats:
        return status, res, {"gjk_iters": stats.gjk_iterations, "epa_iters": stats.epa_iterations, "epa_calls": stats.epa_calls}
    return status, res


def autotune_contacts(ctx: Context, shapes, pairs, prediction: float = 0.0, reps: int = 2) -> dict:
    """Times contacts(shapes, pairs, prediction) for each EPA residency, then with the dearest pairs
    one warp each and with EPA inline, and keeps the fastest in the context's configuration; returns
    the chosen configuration."""
    st = _StagedShapes(shapes)
    kp, pp = _as_input(pairs, np.uint32)
    cfg = _capi.ParryGpuConfig()
    check(lib().parrygpu_autotune_contacts(ctx.handle, C.byref(st.struct), pp, int(kp.shape[0]), float(prediction), int(reps),
                                           C.byref(cfg)), ctx.handle)
    return _config_dict(cfg)


def contact_manifolds(ctx: Context, shapes, pairs, prediction: float, manifolds, want_stats: bool = False, init_dirs=None):
    """Batched DefaultQueryDispatcher::contact_manifold_convex_convex over the (a, b) rows of `pairs`,
    updating `manifolds` in place: a numpy array of parry_gb300.manifold.MANIFOLD_DTYPE records (k,),
    or a torch int32/uint32 tensor of shape (k, RECORD_WORDS) (a CUDA tensor is updated on the device).
    init_dirs (k x 3, optional): the polyhedral generator's GJK start direction for pairs whose record
    holds no cached normal (parrygpu_contact_manifolds_with_dirs). Returns the stats dict when
    want_stats."""
    st = _StagedShapes(shapes)
    kp, pp = _as_input(pairs, np.uint32)
    k = int(kp.shape[0]) if kp is not None else 0
    ki, pi = _as_input(init_dirs, np.float32) if init_dirs is not None else (None, None)
    if ki is not None:
        assert tuple(ki.shape) in ((k, 3), (k * 3,)), "init_dirs must hold 3 floats per pair"
    if _is_torch(manifolds):
        assert manifolds.is_contiguous() and tuple(manifolds.shape) == (k, RECORD_WORDS) and manifolds.element_size() == 4
    else:
        assert manifolds.dtype == MANIFOLD_DTYPE and manifolds.flags.c_contiguous and len(manifolds) == k
    stats = _capi.ParryGpuGjkStats()
    check(lib().parrygpu_contact_manifolds_with_dirs(ctx.handle, C.byref(st.struct), pp, k, float(prediction), pi,
                                                     C.c_void_p(_dptr(manifolds)), C.byref(stats) if want_stats else None),
          ctx.handle)
    if want_stats:
        return {"gjk_iters": stats.gjk_iterations, "epa_iters": stats.epa_iterations, "epa_calls": stats.epa_calls}
    return None


class Scene:
    """The per-frame pipeline over moving convex shapes (parrygpu_scene): integrate (x += v dt,
    q := normalize(q + dt/2 (0, w) q)), AABBs loosened by prediction / 2, BVH refit, overlapping pairs,
    contact manifolds kept per pair across frames, and a fixed ray set cast against the shapes."""

    def __init__(self, ctx: Context, shapes, velocities, prediction: float, pair_capacity: int):
        self._ctx = ctx
        st = _StagedShapes(shapes)
        self.n = st.n
        kv, pv = _as_input(velocities, np.float32)
        h = C.c_void_p()
        check(lib().parrygpu_scene_create(ctx.handle, C.byref(st.struct), pv, float(prediction), int(pair_capacity), C.byref(h)),
              ctx.handle)
        self._h = h
        self.capacity = int(pair_capacity)
        self.n_rays = 0

    def set_rays(self, rays, max_toi: float) -> None:
        kr, pr = _as_input(rays, np.float32)
        n = int(kr.shape[0]) if kr is not None else 0
        check(lib().parrygpu_scene_set_rays(self._ctx.handle, self._h, pr, n, float(max_toi)), self._ctx.handle)
        self.n_rays = n

    def set_mlp(self, mlp) -> None:
        """Seeds the polyhedral pairs without a cached normal (new pairs) with the network's GJK start
        direction each frame (parrygpu_scene_set_mlp); the scene keeps a snapshot of the weights.
        None turns seeding off."""
        check(lib().parrygpu_scene_set_mlp(self._ctx.handle, self._h, mlp._h if mlp is not None else None), self._ctx.handle)

    def step(self, dt: float, frames: int = 1, use_graph: bool = True) -> None:
        check(lib().parrygpu_scene_step(self._ctx.handle, self._h, float(dt), int(frames), 1 if use_graph else 0), self._ctx.handle)

    def info(self) -> tuple[int, int]:
        """(frames advanced, current pair count)."""
        f, n = C.c_uint64(), C.c_uint64()
        check(lib().parrygpu_scene_info(self._ctx.handle, self._h, C.byref(f), C.byref(n)), self._ctx.handle)
        return f.value, n.value

    def read(self, out: dict | None = None, wait: bool = True) -> dict:
        """Host copies of the current poses, pairs (unsorted) with their manifold records, and the
        last frame's ray results. `out` (optional) holds preallocated destinations under the same
        keys - numpy arrays or (pinned) CPU torch tensors: poses (n, 7) f32, pairs (capacity, 2) u32,
        manifolds (capacity, RECORD_WORDS) u32 words, ray_part (n_rays,) u32, ray_toi (n_rays,) f32,
        ray_normal (n_rays, 3) f32 - so a frame loop reads into pinned memory without allocating;
        the returned dict then views their first n_pairs rows. wait=False (with `out`) returns once
        the frame has finished and its copies are queued (parrygpu_scene_read_async): the next
        step() runs while they proceed, and the buffers hold this frame's outputs after read_wait()."""
        from .manifold import new_manifolds
        if not wait:
            if out is None:
                raise ValueError("an asynchronous read needs its destination buffers (out=)")
            return self._read_async(out)
        _, npairs = self.info()
        npairs = min(npairs, self.capacity)
        if out is None:
            dst = {"poses": np.empty((self.n, 7), np.float32), "pairs": np.empty((npairs, 2), np.uint32),
                   "manifolds": new_manifolds(npairs), "ray_part": np.empty(self.n_rays, np.uint32),
                   "ray_toi": np.empty(self.n_rays, np.float32), "ray_normal": np.empty((self.n_rays, 3), np.float32)}
        else:
            dst = out
            assert tuple(dst["poses"].shape) == (self.n, 7) and len(dst["pairs"]) >= npairs and len(dst["manifolds"]) >= npairs
            assert len(dst["ray_part"]) == self.n_rays and len(dst["ray_toi"]) == self.n_rays and len(dst["ray_normal"]) == self.n_rays

        def ptr(a):
            return a.data_ptr() if _is_torch(a) else a.ctypes.data
        has_rays = self.n_rays > 0
        check(lib().parrygpu_scene_read(self._ctx.handle, self._h, ptr(dst["poses"]), ptr(dst["pairs"]) if npairs else None,
                                        ptr(dst["manifolds"]) if npairs else None, npairs, ptr(dst["ray_part"]) if has_rays else None,
                                        ptr(dst["ray_toi"]) if has_rays else None, ptr(dst["ray_normal"]) if has_rays else None),
              self._ctx.handle)
        if out is None:
            return dst
        res = dict(dst)
        res["pairs"] = dst["pairs"][:npairs]
        res["manifolds"] = dst["manifolds"][:npairs]
        return res

    def _read_async(self, dst: dict) -> dict:
        assert tuple(dst["poses"].shape) == (self.n, 7) and len(dst["pairs"]) == len(dst["manifolds"])
        assert len(dst["ray_part"]) == self.n_rays and len(dst["ray_toi"]) == self.n_rays and len(dst["ray_normal"]) == self.n_rays

        def ptr(a):
            return a.data_ptr() if _is_torch(a) else a.ctypes.data
        has_rays = self.n_rays > 0
        npairs = C.c_uint64()
        check(lib().parrygpu_scene_read_async(self._ctx.handle, self._h, ptr(dst["poses"]), ptr(dst["pairs"]), ptr(dst["manifolds"]),
                                              len(dst["pairs"]), ptr(dst["ray_part"]) if has_rays else None,
                                              ptr(dst["ray_toi"]) if has_rays else None, ptr(dst["ray_normal"]) if has_rays else None,
                                              C.byref(npairs)), self._ctx.handle)
        self._pending = dst  # the buffers the copies write stay referenced until read_wait
        res = dict(dst)
        res["pairs"] = dst["pairs"][:npairs.value]
        res["manifolds"] = dst["manifolds"][:npairs.value]
        return res

    def read_wait(self) -> None:
        """Waits for the copies of the last read(wait=False)."""
        check(lib().parrygpu_scene_read_wait(self._ctx.handle, self._h), self._ctx.handle)
        self._pending = None

    def stats(self) -> dict:
        """The last frame's narrow-phase counters: GJK / EPA iterations, EPA calls, and the pairs that
        took a learned GJK start direction."""
        st = _capi.ParryGpuGjkStats()
        seeded = C.c_uint64()
        check(lib().parrygpu_scene_stats(self._ctx.handle, self._h, C.byref(st), C.byref(seeded)), self._ctx.handle)
        return {"gjk_iters": st.gjk_iterations, "epa_iters": st.epa_iterations, "epa_calls": st.epa_calls,
                "seeded_pairs": seeded.value}

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            lib().parrygpu_scene_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Compound:
    """shape::Compound on the GPU: parts with poses under one LBVH, for batched ray casts."""

    def __init__(self, ctx: Context, shapes):
        self.ctx = ctx
        st = _StagedShapes(shapes)
        self.n = st.n
        h = C.c_void_p()
        check(lib().parrygpu_compound_create(ctx.handle, C.byref(st.struct), C.byref(h)), ctx.handle)
        self._h = h

    def set_poses(self, poses) -> None:
        """Moves the parts ((n, 7) poses) and refits the BVH."""
        kp, pp = _as_input(poses, np.float32)
        check(lib().parrygpu_compound_set_poses(self.ctx.handle, self._h, pp), self.ctx.handle)

    def cast_rays_and_get_normal(self, rays, max_toi: float, solid: bool = True, pose=None, out=None):
        """Batched Compound::cast_ray_and_get_normal: (part, toi, normal); part = NO_HIT on a miss."""
        kr, pr = _as_input(rays, np.float32)
        n = int(kr.shape[0])
        kq, pq = _as_input(pose, np.float32) if pose is not None else (None, None)
        if out is None:
            part, pp = _alloc_like(kr, (n,), np.uint32)
            toi, pt = _alloc_like(kr, (n,), np.float32)
            nrm, pn = _alloc_like(kr, (n, 3), np.float32)
        else:
            part, toi, nrm = out
            pp, pt, pn = C.c_void_p(_dptr(part)), C.c_void_p(_dptr(toi)), C.c_void_p(_dptr(nrm)) if nrm is not None else None
        check(lib().parrygpu_compound_cast_rays(self.ctx.handle, self._h, pq, pr, n, float(max_toi), 1 if solid else 0, pp, pt, pn),
              self.ctx.handle)
        return part, toi, nrm

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().parrygpu_compound_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class WarmStartMLP:
    """Learned GJK initial direction (BF16 tensor-core MLP, see include/parry_gpu.h)."""

    IN = 48

    def __init__(self, ctx: Context, seed: int = 0):
        self.ctx = ctx
        h = C.c_void_p()
        check(lib().parrygpu_mlp_create(ctx.handle, C.c_uint64(seed), C.byref(h)), ctx.handle)
        self._h = h

    @staticmethod
    def param_count() -> int:
        return int(lib().parrygpu_mlp_param_count())

    def features(self, shapes, pairs):
        st = _StagedShapes(shapes)
        kp, pp = _as_input(pairs, np.uint32)
        k = int(kp.shape[0])
        out, po = _alloc_like(kp, (k, self.IN), np.float32)
        check(lib().parrygpu_mlp_features(self.ctx.handle, C.byref(st.struct), pp, k, po), self.ctx.handle)
        return out

    def train(self, features, targets, epochs: int = 1, batch: int = 8192, lr: float = 1e-3):
        """Adam on mean(1 - cos(prediction, target)); features and targets must be CUDA tensors."""
        kf, pf = _as_input(features, np.float32)
        kt, pt = _as_input(targets, np.float32)
        losses = np.zeros(max(1, epochs), np.float32)
        check(lib().parrygpu_mlp_train(self.ctx.handle, self._h, pf, pt, int(kf.shape[0]), int(epochs), int(batch), float(lr),
                                       C.c_void_p(losses.ctypes.data)), self.ctx.handle)
        return losses[:epochs]

    def predict(self, features):
        kf, pf = _as_input(features, np.float32)
        n = int(kf.shape[0])
        out, po = _alloc_like(kf, (n, 3), np.float32)
        check(lib().parrygpu_mlp_predict(self.ctx.handle, self._h, pf, n, po), self.ctx.handle)
        return out

    def loss_and_grads(self, features, targets):
        kf, pf = _as_input(features, np.float32)
        kt, pt = _as_input(targets, np.float32)
        loss = C.c_float(0.0)
        grads = np.zeros(self.param_count(), np.float32)
        check(lib().parrygpu_mlp_loss_and_grads(self.ctx.handle, self._h, pf, pt, int(kf.shape[0]), C.byref(loss),
                                                C.c_void_p(grads.ctypes.data)), self.ctx.handle)
        return float(loss.value), grads

    def get_params(self) -> np.ndarray:
        p = np.zeros(self.param_count(), np.float32)
        check(lib().parrygpu_mlp_get_params(self.ctx.handle, self._h, C.c_void_p(p.ctypes.data)), self.ctx.handle)
        return p

    def set_params(self, params) -> None:
        p = np.ascontiguousarray(params, np.float32)
        assert p.size == self.param_count()
        check(lib().parrygpu_mlp_set_params(self.ctx.handle, self._h, C.c_void_p(p.ctypes.data)), self.ctx.handle)

    def save(self, path) -> None:
        """Checkpoint: a JSON header line then the raw float32 parameters."""
        import json
        p = self.get_params()
        with open(path, "wb") as f:
            f.write((json.dumps({"format": "parry_gb300.warm_start_mlp", "version": 1, "params": int(p.size)}) + "\n").encode())
            f.write(p.tobytes())

    def load(self, path) -> None:
        import json
        with open(path, "rb") as f:
            hdr = json.loads(f.readline().decode())
            if hdr.get("format") != "parry_gb300.warm_start_mlp" or hdr.get("params") != self.param_count():
                raise ValueError(f"not a compatible warm-start checkpoint: {hdr}")
            self.set_params(np.frombuffer(f.read(), np.float32))

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().parrygpu_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
