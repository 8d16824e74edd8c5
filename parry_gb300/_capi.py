"""ctypes binding of libparrygpu's C ABI (include/parry_gpu.h).

This is the same binding a Python user of the C library would write; a Rust caller binds the same
`extern "C"` declarations. Loading fails loudly when the compiled library is missing: there is no
CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

_LIB_PATH = Path(__file__).resolve().parent / "libparrygpu.so"

P = C.c_void_p
U32 = C.c_uint32
U64 = C.c_uint64
I32 = C.c_int
F32 = C.c_float
PU64 = C.POINTER(C.c_uint64)
PU32 = C.POINTER(C.c_uint32)

STATUS = {
    0: "ok",
    1: "invalid argument",
    2: "unsupported shape pair",
    3: "capacity exceeded",
    5: "device wait timed out",
    6: "CUDA error",
    7: "traversal stack overflow",
    8: "no CUDA device",
}

# name -> (restype, argtypes); every symbol declared in include/parry_gpu.h.
SIGNATURES: dict[str, tuple] = {
    "parrygpu_default_config": (None, [P]),
    "parrygpu_create": (I32, [C.POINTER(P), P]),
    "parrygpu_destroy": (None, [P]),
    "parrygpu_set_stream": (I32, [P, P]),
    "parrygpu_sync": (I32, [P]),
    "parrygpu_last_error": (C.c_char_p, [P]),
    "parrygpu_status_string": (C.c_char_p, [I32]),
    "parrygpu_kernel_launches": (U64, [P]),
    "parrygpu_enable_kernel_timing": (I32, [P, I32]),
    "parrygpu_kernel_time": (I32, [P, C.c_char_p, C.POINTER(C.c_double), PU64]),
    "parrygpu_reset_kernel_timing": (I32, [P]),
    "parrygpu_bvh_build": (I32, [P, P, U32, C.POINTER(P)]),
    "parrygpu_bvh_rebuild": (I32, [P, P, P, U32]),
    "parrygpu_bvh_destroy": (None, [P]),
    "parrygpu_bvh_refit": (I32, [P, P, P]),
    "parrygpu_bvh_self_pairs": (I32, [P, P, P, U64, PU64, I32]),
    "parrygpu_bvh_leaf_pairs": (I32, [P, P, P, P, U64, PU64, I32]),
    "parrygpu_bvh_info": (I32, [P, PU32, PU32]),
    "parrygpu_bvh_copy_nodes": (I32, [P, P, P]),
    "parrygpu_bvh_export": (I32, [P, P, P, P, P, U64]),
    "parrygpu_bvh_import": (I32, [P, P, U32, C.POINTER(P)]),
    "parrygpu_bvh_insert": (I32, [P, P, P, P, U32]),
    "parrygpu_bvh_remove": (I32, [P, P, P, U32]),
    "parrygpu_trimesh_create": (I32, [P, P, U32, P, U32, C.POINTER(P)]),
    "parrygpu_trimesh_destroy": (None, [P]),
    "parrygpu_polyhedra_build_gpu": (I32, [P, P, U64, P, P, U64, C.POINTER(P)]),
    "parrygpu_polyhedra_gpu_sizes": (I32, [P, P]),
    "parrygpu_polyhedra_gpu_copy": (I32, [P, P, P, P, P, P, P, P, P, P, P, P]),
    "parrygpu_polyhedra_gpu_view": (I32, [P, P, P]),
    "parrygpu_polyhedra_gpu_triangles": (I32, [P, P, P, P, P]),
    "parrygpu_polyhedra_gpu_destroy": (None, [P]),
    "parrygpu_trimesh_set_flags": (I32, [P, P, U32]),
    "parrygpu_trimesh_normal_constraints": (I32, [P, P, P, P]),
    "parrygpu_project_local_normals": (I32, [P, P, P, U64, P, P]),
    "parrygpu_trimesh_cast_rays": (I32, [P, P, P, P, U32, F32, I32, P, P, P]),
    "parrygpu_trimesh_cast_rays_noalloc": (I32, [P, P, P, P, U32, F32, I32, P, P, P]),
    "parrygpu_shapes_aabbs": (I32, [P, P, F32, P]),
    "parrygpu_contacts": (I32, [P, P, P, U64, F32, P, P, P, P]),
    "parrygpu_get_config": (I32, [P, P]),
    "parrygpu_cast_shapes": (I32, [P, P, P, U64, P, P, P, P, P]),
    "parrygpu_trimesh_contacts_create": (I32, [P, P, U32, U32, C.POINTER(P)]),
    "parrygpu_trimesh_contacts_destroy": (None, [P]),
    "parrygpu_trimesh_contacts_update": (I32, [P, P, P, P, F32]),
    "parrygpu_trimesh_contacts_read": (I32, [P, P, P, P, P]),
    "parrygpu_autotune_trimesh_rays": (I32, [P, P, P, P, U32, F32, U32, P]),
    "parrygpu_autotune_contacts": (I32, [P, P, P, U64, F32, U32, P]),
    "parrygpu_contacts_with_dirs": (I32, [P, P, P, U64, F32, P, P, P, P, P]),
    "parrygpu_contact_manifolds": (I32, [P, P, P, U64, F32, P, P]),
    "parrygpu_contact_manifolds_with_dirs": (I32, [P, P, P, U64, F32, P, P, P]),
    "parrygpu_polyhedra_build": (I32, [P, P, P, U64, U32, C.POINTER(P)]),
    "parrygpu_scene_create": (I32, [P, P, P, F32, U64, C.POINTER(P)]),
    "parrygpu_scene_destroy": (None, [P]),
    "parrygpu_scene_set_rays": (I32, [P, P, P, U64, F32]),
    "parrygpu_scene_step": (I32, [P, P, F32, U32, I32]),
    "parrygpu_scene_info": (I32, [P, P, P, P]),
    "parrygpu_scene_read": (I32, [P, P, P, P, P, U64, P, P, P]),
    "parrygpu_scene_read_async": (I32, [P, P, P, P, P, U64, P, P, P, P]),
    "parrygpu_scene_read_wait": (I32, [P, P]),
    "parrygpu_scene_set_mlp": (I32, [P, P, P]),
    "parrygpu_scene_stats": (I32, [P, P, P, P]),
    "parrygpu_polyhedra_sizes": (I32, [P, P]),
    "parrygpu_polyhedra_copy": (I32, [P, P, P, P, P, P, P, P, P, P, P]),
    "parrygpu_polyhedra_triangles": (I32, [P, P, P, P]),
    "parrygpu_polyhedra_builder_destroy": (None, [P]),
    "parrygpu_mlp_create": (I32, [P, U64, C.POINTER(P)]),
    "parrygpu_mlp_destroy": (None, [P]),
    "parrygpu_mlp_features": (I32, [P, P, P, U64, P]),
    "parrygpu_mlp_train": (I32, [P, P, P, P, U64, U32, U32, F32, P]),
    "parrygpu_mlp_predict": (I32, [P, P, P, U64, P]),
    "parrygpu_mlp_loss_and_grads": (I32, [P, P, P, P, U64, P, P]),
    "parrygpu_mlp_param_count": (U64, []),
    "parrygpu_mlp_get_params": (I32, [P, P, P]),
    "parrygpu_mlp_set_params": (I32, [P, P, P]),
    "parrygpu_compound_create": (I32, [P, P, C.POINTER(P)]),
    "parrygpu_compound_destroy": (None, [P]),
    "parrygpu_compound_set_poses": (I32, [P, P, P]),
    "parrygpu_compound_cast_rays": (I32, [P, P, P, P, U32, F32, I32, P, P, P]),
}


class ParryGpuPolyhedra(C.Structure):
    _fields_ = [("n_hulls", C.c_uint64), ("hulls", C.c_void_p), ("n_faces", C.c_uint64), ("face_normals", C.c_void_p),
                ("face_ranges", C.c_void_p), ("n_face_entries", C.c_uint64), ("face_vertices", C.c_void_p),
                ("face_edges", C.c_void_p), ("vertex_ranges", C.c_void_p), ("n_vertex_entries", C.c_uint64),
                ("vertex_faces", C.c_void_p), ("vertex_edges", C.c_void_p), ("n_edges", C.c_uint64), ("edge_dirs", C.c_void_p)]


class ParryGpuShapes(C.Structure):
    _fields_ = [("n", C.c_uint64), ("types", C.c_void_p), ("params", C.c_void_p), ("poses", C.c_void_p),
                ("vertices", C.c_void_p), ("n_vertices", C.c_uint64), ("polyhedra", C.c_void_p)]


class ParryGpuShapeCastOptions(C.Structure):
    _fields_ = [("max_time_of_impact", C.c_float), ("target_distance", C.c_float), ("stop_at_penetration", C.c_uint32),
                ("compute_impact_geometry_on_penetration", C.c_uint32)]


class ParryGpuGjkStats(C.Structure):
    _fields_ = [("gjk_iterations", C.c_uint64), ("epa_iterations", C.c_uint64), ("epa_calls", C.c_uint64),
                ("reserved", C.c_uint64)]


class ParryGpuError(RuntimeError):
    def __init__(self, status: int, msg: str = ""):
        self.status = status
        super().__init__(f"{STATUS.get(status, 'unknown status')} ({status}){': ' + msg if msg else ''}")


class ParryGpuConfig(C.Structure):
    _fields_ = [("device", C.c_int), ("ray_block", C.c_uint32), ("sort_rays", C.c_uint32), ("ray_sort_key", C.c_uint32),
                ("epa_blocks_per_sm", C.c_uint32), ("ray_traversal", C.c_uint32), ("ray_refill", C.c_uint32),
                ("ray_chunks", C.c_uint32), ("ray_host_access", C.c_uint32), ("contact_warp_cost", C.c_uint32),
                ("contact_epa_inline", C.c_uint32), ("mlp_infer", C.c_uint32),
                ("scene_ray_order", C.c_uint32),
                ("scene_ray_grid", C.c_uint32)]


_lib = None


def lib() -> C.CDLL:
    """Loads libparrygpu.so (built by parry_gb300._build / __graft_entry__.build())."""
    global _lib
    if _lib is None:
        if not _LIB_PATH.exists():
            raise ImportError(f"{_LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
        l = C.CDLL(str(_LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            f = getattr(l, name)
            f.restype = res
            f.argtypes = args
        _lib = l
    return _lib


def check(status: int, ctx=None) -> None:
    if status != 0:
        msg = ""
        if ctx is not None:
            raw = lib().parrygpu_last_error(ctx)
            msg = raw.decode() if raw else ""
        raise ParryGpuError(status, msg)
