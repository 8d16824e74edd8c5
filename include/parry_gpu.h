/*
 * libparrygpu — GB300 (sm_103a) batched implementation of parry3d's data-parallel query path,
 * exported as a plain C ABI.
 *
 * Every entry point replaces a CPU loop over one parry3d call; the reference interface each one
 * replaces is cited (paths relative to the parry repository).
 *
 * Conventions
 *  - Pointers may be device pointers or host pointers (pageable or pinned); the library checks
 *    each with cudaPointerGetAttributes. Host inputs are staged through library-owned device
 *    buffers. A call whose outputs are all device pointers is asynchronous on the context's
 *    stream; a call with any host output synchronises that stream before returning.
 *  - Layouts follow parry3d's #[repr(C)] types: Aabb = {mins xyz, maxs xyz} (6 floats),
 *    Ray = {origin xyz, dir xyz} (6 floats), Isometry = pose7 {qi, qj, qk, qw, tx, ty, tz}.
 *  - The library owns the device memory behind each handle; the caller owns every output buffer.
 *  - One stream per context. A context is not thread-safe; distinct contexts are.
 *  - Errors: every function returns a parrygpu_status. Query results that parry expresses as
 *    Option::None (no hit, no contact) are reported in the output arrays, not as errors.
 */
#ifndef PARRY_GPU_H
#define PARRY_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum parrygpu_status {
  PARRYGPU_OK = 0,
  PARRYGPU_INVALID_ARG = 1,
  /* parry: Err(Unsupported) for a shape pair without an implementation (src/query/error.rs:146-147). */
  PARRYGPU_UNSUPPORTED_PAIR = 2,
  /* The caller's pair buffer is too small; *n_out still holds the full pair count. */
  PARRYGPU_CAPACITY_EXCEEDED = 3,
  PARRYGPU_TIMEOUT = 5,
  PARRYGPU_CUDA_ERROR = 6,
  /* A traversal stack overflowed its fixed depth (the affected queries report no result). */
  PARRYGPU_STACK_OVERFLOW = 7,
  PARRYGPU_NO_DEVICE = 8
} parrygpu_status;

typedef struct parrygpu_ctx parrygpu_ctx;
typedef struct parrygpu_bvh parrygpu_bvh;
typedef struct parrygpu_trimesh parrygpu_trimesh;
typedef struct parrygpu_compound parrygpu_compound;

typedef struct parrygpu_config {
  int device;              /* CUDA device ordinal */
  uint32_t ray_block;      /* threads per block for TriMesh ray traversal: 0 (library default, 128) or a
                              multiple of 32 up to 1024 */
  uint32_t sort_rays;      /* 1 = Morton-sort rays before traversal (default), 0 = input order */
  uint32_t ray_sort_key;   /* 0 = 30-bit Morton code of the origin; 1 = direction octant (3 bits)
                              above a 27-bit Morton code of the origin; 2 = the top 16 bits of the
                              origin's Morton code (two radix passes instead of four) */
  uint32_t epa_blocks_per_sm; /* contacts EPA: resident 64-thread blocks per SM (0 = library default, 8; at most 32) */
  uint32_t ray_traversal;  /* TriMesh ray traversal: 0 = library default (1); 1 = one ray per thread;
                              2 = persistent warps that fetch new rays as lanes finish theirs;
                              3 = one ray per thread with leaf tests postponed until the warp's
                              lanes all hold one ("while-while") */
  uint32_t ray_refill;     /* traversal 2: a warp fetches rays once this many of its lanes are idle
                              (0 = library default, 16; at most 32) */
  uint32_t ray_chunks;     /* host-buffer ray casts without a ray ordering: chunks over two streams
                              (0 = library default: one per 262,144 rays, 2 to 4; 1 = no chunking; at
                              most 64) */
  uint32_t ray_host_access; /* host-buffer ray casts without a ray ordering whose host buffers are all
                              page-locked (cudaHostAlloc / cudaHostRegister): 1 = the kernel reads the
                              rays and writes the results in place over the host link (on
                              Grace-Blackwell the coherent NVLink-C2C); 2 = staged through device
                              copies, as ray_chunks says; 0 = library default: in place when the
                              device's host link is coherent (it reads host memory through the
                              host's page tables), else staged. Other host buffers are staged. */
  uint32_t contact_warp_cost; /* query::contact on more than 4096 pairs: pairs whose support-scan cost
                              (vertices one support evaluation scans, summed over the two shapes, at
                              most 1023) is at least this run one warp per pair, hulls staged in shared
                              memory; 0 = library default; 1024 or more = never (one thread per pair) */
  uint32_t contact_epa_inline; /* query::contact: 1 = a pair's EPA runs in the same thread right after its
                              GJK (one workspace slot per thread of the persistent grid); 2 = through a
                              queue, in a second persistent pass over the pairs that reach EPA; 0 =
                              library default (2) */
  uint32_t mlp_infer;      /* parrygpu_mlp_predict: 1 = one fused kernel on the fifth-generation tensor
                              cores (tcgen05.mma into TMEM, weights resident in shared memory); 2 = the
                              training path's per-layer mma.sync GEMMs; 0 = library default (1) */
  uint32_t scene_ray_order; /* parrygpu_scene: the order the rays are stored and cast in (answers keep the
                              input order): 1 = Morton code of the origin; 2 = direction octant above
                              it; 3 = direction octant and dominant axis above it; 0 = library default */
  uint32_t scene_ray_grid; /* parrygpu_scene rays: 1 = walk a uniform grid over the shapes, rebuilt each
                              frame (falls back to the BVH on the device when its entries outgrow their
                              capacity); 2 = traverse the BVH; 0 = library default (1). Same answers. */
} parrygpu_config;

/* ---- context ---------------------------------------------------------------------------- */

/* Fills *cfg with the library defaults. */
void parrygpu_default_config(parrygpu_config* cfg);
/* Creates a context on cfg->device (cfg may be NULL for defaults) with its own stream. */
parrygpu_status parrygpu_create(parrygpu_ctx** out, const parrygpu_config* cfg);
void parrygpu_destroy(parrygpu_ctx* ctx);
/* Makes the context launch on `stream` (a cudaStream_t; NULL = the context's own stream). */
parrygpu_status parrygpu_set_stream(parrygpu_ctx* ctx, void* stream);
/* Waits for the context's stream; reports device-side error flags raised since the last sync. */
parrygpu_status parrygpu_sync(parrygpu_ctx* ctx);
const char* parrygpu_last_error(const parrygpu_ctx* ctx);
const char* parrygpu_status_string(parrygpu_status s);
/* Number of kernels this context has launched since creation. */
uint64_t parrygpu_kernel_launches(const parrygpu_ctx* ctx);
/* Per-kernel timing: when enabled, the main kernel of each call is bracketed with CUDA events on
 * the context stream. parrygpu_kernel_time synchronises and returns the total milliseconds and
 * launch count recorded for `kernel` (e.g. "trimesh_rays", "ray_sort", "lbvh_build") since the
 * last reset. No reference counterpart (parry has no device timing). */
parrygpu_status parrygpu_enable_kernel_timing(parrygpu_ctx* ctx, int enable);
parrygpu_status parrygpu_kernel_time(parrygpu_ctx* ctx, const char* kernel, double* total_ms, uint64_t* launches);
parrygpu_status parrygpu_reset_kernel_timing(parrygpu_ctx* ctx);

/* ---- partitioning::Bvh -------------------------------------------------------------------- */

/* Replaces Bvh::from_leaves(strategy, &[Aabb]) (src/partitioning/bvh/bvh_tree.rs:1835-1837).
 * Builds an LBVH (30-bit Morton codes, device radix sort, Karras hierarchy, atomic bottom-up fit)
 * over `n` AABBs (n x 6 floats). Leaf data = the AABB's index, as in from_leaves. The tree is
 * stored in the reference's 64-byte BvhNodeWide layout with the root in wide node 0. */
parrygpu_status parrygpu_bvh_build(parrygpu_ctx* ctx, const float* aabbs, uint32_t n, parrygpu_bvh** out);
void parrygpu_bvh_destroy(parrygpu_bvh* bvh);
/* Bvh::from_leaves again into an existing handle (a new tree over `n` AABBs; the handle's device
 * storage is reused and grows only when n exceeds every earlier size). Asynchronous for device
 * AABBs, like parrygpu_bvh_build. */
parrygpu_status parrygpu_bvh_rebuild(parrygpu_ctx* ctx, parrygpu_bvh* bvh, const float* aabbs, uint32_t n);
/* Replaces Bvh::insert_or_update_partially for every leaf followed by Bvh::refit
 * (src/partitioning/bvh/bvh_insert.rs:209-231, src/partitioning/bvh/bvh_refit.rs:170-180):
 * leaf i takes aabbs[i] and every internal AABB is recomputed bottom-up; topology is kept. */
parrygpu_status parrygpu_bvh_refit(parrygpu_ctx* ctx, parrygpu_bvh* bvh, const float* aabbs);
/* Replaces Bvh::traverse_bvtt_single_tree::<false> (src/partitioning/bvh/bvh_traverse_bvtt.rs:19-31):
 * every unordered pair of leaves whose AABBs intersect (inclusive), written as (min, max) pairs
 * (2 x u32 each) into pairs[0 .. 2*cap). *n_out (host) receives the total pair count. With
 * sorted != 0 the pairs are in ascending lexicographic order. */
parrygpu_status parrygpu_bvh_self_pairs(parrygpu_ctx* ctx, const parrygpu_bvh* bvh, uint32_t* pairs, uint64_t cap,
                                        uint64_t* n_out, int sorted);
/* Replaces Bvh::leaf_pairs(&other, |a, b| a.intersects(b)) (src/partitioning/bvh/bvh_traverse_bvtt.rs:210-316):
 * (leaf of a, leaf of b) pairs. As in the reference iterator, the pairs formed by the two roots'
 * direct children are taken without an AABB check. */
parrygpu_status parrygpu_bvh_leaf_pairs(parrygpu_ctx* ctx, const parrygpu_bvh* a, const parrygpu_bvh* b, uint32_t* pairs,
                                        uint64_t cap, uint64_t* n_out, int sorted);
/* Leaf count (Bvh::leaf_count, bvh_tree.rs:2295-2301) and wide-node count of the tree. */
parrygpu_status parrygpu_bvh_info(const parrygpu_bvh* bvh, uint32_t* leaf_count, uint32_t* wide_node_count);
/* Copies the tree's wide nodes (wide_node_count x 64 bytes, BvhNodeWide layout) into `out`. */
parrygpu_status parrygpu_bvh_copy_nodes(parrygpu_ctx* ctx, const parrygpu_bvh* bvh, void* out);
/* The reference's serialised Bvh (src/partitioning/bvh/bvh_tree.rs:1748-1761: nodes, parents,
 * leaf_node_indices; BvhNodeIndex = (wide node << 1) | is_right, bvh_tree.rs:1244-1290), host or
 * device buffers, any may be NULL: nodes = wide_node_count x 64 bytes, parents = wide_node_count
 * u64 (the root's entry 0), leaf_nodes = leaf_capacity u64 indexed by leaf index (UINT64_MAX where no
 * leaf has that index; a leaf index >= leaf_capacity raises CAPACITY_EXCEEDED). */
parrygpu_status parrygpu_bvh_export(parrygpu_ctx* ctx, const parrygpu_bvh* bvh, void* nodes, uint64_t* parents, uint64_t* leaf_nodes,
                                    uint64_t leaf_capacity);
/* Leaf indices (the `data` of a leaf node, the `leaf_ids` of an insert) are below this bound. A
 * tree whose largest leaf index is L takes L + 1 AABB rows in parrygpu_bvh_refit, so the bound keeps
 * that row count and the pair index range representable. */
#define PARRYGPU_MAX_LEAF_INDEX 0x7ffffffeu
/* A tree from the reference's serialised nodes (n_wide BvhNodeWide records, host or device; e.g.
 * deserialised from parry's serde / rkyv form): parents and depth-first leaf positions are derived
 * on the device. Malformed trees (child index out of range, a node with two parents or none, leaf
 * counts that do not add up, a leaf index above PARRYGPU_MAX_LEAF_INDEX) are rejected with
 * INVALID_ARG. */
parrygpu_status parrygpu_bvh_import(parrygpu_ctx* ctx, const void* nodes, uint32_t n_wide, parrygpu_bvh** out);
/* Bvh::insert(aabb, leaf_index) (bvh_insert.rs:126-133) for k rows: a new leaf index is added, an
 * existing one takes the new AABB (the last row wins); Bvh::remove(leaf_index) (bvh_tree.rs:2360) for
 * k indices (indices without a leaf are ignored). The tree is rebuilt over the resulting leaf set
 * (decision D-9: the layout differs from the reference's incremental edits, query answers do not).
 * Afterwards parrygpu_bvh_refit takes 1 + (largest leaf index) AABB rows indexed by leaf index.
 * A leaf index above PARRYGPU_MAX_LEAF_INDEX is rejected with INVALID_ARG and leaves the tree as it was. */
parrygpu_status parrygpu_bvh_insert(parrygpu_ctx* ctx, parrygpu_bvh* bvh, const float* aabbs, const uint32_t* leaf_ids, uint32_t k);
parrygpu_status parrygpu_bvh_remove(parrygpu_ctx* ctx, parrygpu_bvh* bvh, const uint32_t* leaf_ids, uint32_t k);

/* ---- TriMesh ray casts ------------------------------------------------------------------- */

/* Replaces TriMesh::new(vertices, indices) (src/shape/trimesh.rs:607, BVH :1159-1171). */
parrygpu_status parrygpu_trimesh_create(parrygpu_ctx* ctx, const float* vertices, uint32_t n_vertices,
                                        const uint32_t* indices, uint32_t n_triangles, parrygpu_trimesh** out);
void parrygpu_trimesh_destroy(parrygpu_trimesh* mesh);

/* TriMeshFlags bits (src/shape/trimesh.rs:470-507) that parrygpu_trimesh_set_flags accepts. */
#define PARRYGPU_TRIMESH_ORIENTED (1u << 3)
#define PARRYGPU_TRIMESH_MERGE_DUPLICATE_VERTICES (1u << 4)
#define PARRYGPU_TRIMESH_FIX_INTERNAL_EDGES ((1u << 7) | (1u << 4))
/* Replaces TriMesh::set_flags (trimesh.rs:748-800) for ORIENTED, MERGE_DUPLICATE_VERTICES and
 * FIX_INTERNAL_EDGES; the other flags (topology, connected components, triangle deletion) return
 * PARRYGPU_UNSUPPORTED_PAIR. With FIX_INTERNAL_EDGES the triangles' pseudo-normals are computed on
 * the device (bit-identical vertices merged, edge pseudo-normal = sum of the unit normals of the
 * triangles sharing the edge, compute_pseudo_normals :1348-1407) and every contact manifold against
 * the mesh applies them as normal constraints. Triangle ids, the BVH and ray casts do not change. */
parrygpu_status parrygpu_trimesh_set_flags(parrygpu_ctx* ctx, parrygpu_trimesh* mesh, uint32_t flags);
/* TriMesh::triangle_normal_constraints for every triangle (trimesh.rs:1911-1931): pseudo = n_triangles
 * x 12 floats (face normal, then the edge pseudo-normals of edges 01, 12, 20), valid[t] = 1 when the
 * reference returns Some (FIX_INTERNAL_EDGES set, the face and all three edges normalisable). */
parrygpu_status parrygpu_trimesh_normal_constraints(parrygpu_ctx* ctx, const parrygpu_trimesh* mesh, float* pseudo, uint8_t* valid);
/* TrianglePseudoNormals::project_local_normal (src/shape/triangle_pseudo_normals.rs:35-99) for n rows:
 * pseudo = n x 12 floats, dirs / out = n x 3 floats, ok[i] = 0 where the reference returns None. */
parrygpu_status parrygpu_project_local_normals(parrygpu_ctx* ctx, const float* pseudo, const float* dirs, uint64_t n, float* out,
                                               uint8_t* ok);
/* Replaces a loop of RayCast::cast_ray_and_get_normal(m, ray, max_toi, solid) on a TriMesh
 * (src/query/ray/ray.rs:393-403 -> src/query/ray/ray_trimesh.rs:17-35). pose7 = the mesh pose m
 * (NULL = identity). rays: n x 6 floats. Outputs per ray:
 *   feature[i] = hit triangle t for a front-face hit, t + n_triangles for a back-face hit
 *                (FeatureId::Face), UINT32_MAX for no hit;
 *   toi[i]     = time of impact (0 on a miss);
 *   normal     = n x 3 floats, world-space normal facing the ray origin (may be NULL: then this
 *                is RayCast::cast_ray, which returns the toi only).
 * Exact toi ties resolve to the lowest triangle index. `solid` has no effect on triangles in 3-D,
 * as in the reference. */
parrygpu_status parrygpu_trimesh_cast_rays(parrygpu_ctx* ctx, const parrygpu_trimesh* mesh, const float* pose7,
                                           const float* rays, uint32_t n, float max_toi, int solid, uint32_t* feature,
                                           float* toi, float* normal);

/* Largest batch parrygpu_trimesh_cast_rays_noalloc accepts. */
#define PARRYGPU_NOALLOC_MAX_RAYS 262144u

/* No counterpart in the reference (parry allocates nothing on a device): the same ray cast as
 * parrygpu_trimesh_cast_rays, for callers that may not allocate device memory while they run (an
 * engine that owns the whole device budget, a frame loop that must never block on cudaMalloc or on
 * cudaFree's device-wide wait). It allocates nothing: the ray-ordering scratch is a fixed array
 * inside the library, sized for PARRYGPU_NOALLOC_MAX_RAYS rays (about 4.3 MB, held on every GPU
 * that loads the library until exit). Larger batches are rejected with PARRYGPU_INVALID_ARG; split
 * them. rays, feature, toi and normal must be device memory of the context's GPU (host buffers
 * would need staging; another GPU's memory is rejected). pose7 may be host or device memory; a
 * device pose7 is read back first, which waits for the context stream's earlier work and cannot
 * happen inside a stream capture, so a frame loop that must not block passes a host pose7. The
 * first call on a device looks up the array's device address; make that first call before any
 * stream capture (later calls outside capture look it up again, so a cudaDeviceReset between calls
 * is harmless). Every call shares the one array and it keeps the last call's contents, so calls
 * that overlap on the GPU race: keep them on one stream or synchronise between them. Results match
 * parrygpu_trimesh_cast_rays. */
parrygpu_status parrygpu_trimesh_cast_rays_noalloc(parrygpu_ctx* ctx, const parrygpu_trimesh* mesh, const float* pose7,
                                                   const float* rays, uint32_t n, float max_toi, int solid, uint32_t* feature,
                                                   float* toi, float* normal);

/* ---- convex shapes and query::contact ------------------------------------------------------ */

typedef enum parrygpu_shape_type {
  PARRYGPU_BALL = 0,     /* Ball::new(r)                        params {r, 0, 0, 0} */
  PARRYGPU_CUBOID = 1,   /* Cuboid::new(half_extents)           params {hx, hy, hz, 0} */
  PARRYGPU_CAPSULE = 2,  /* Capsule::new_y(half_height, radius) params {half_height, radius, 0, 0} */
  PARRYGPU_CONVEX = 3,   /* ConvexPolyhedron                    params {first vertex, vertex count, hull + 1, 0} (u32 bits);
                          * hull + 1 = 0: a vertex cloud without topology (support maps only, no manifolds) */
  PARRYGPU_TRIANGLE = 4  /* Triangle::new(a, b, c)              params {first vertex (u32 bits), 3, 0, 0} */
} parrygpu_shape_type;

/* Topology of ConvexPolyhedron shapes (src/shape/convex_polyhedron.rs:172-185), all hulls
 * concatenated. Ids stored in the index arrays are hull-local, as the reference's feature ids are.
 *   hulls          n_hulls x 8 u32: first vertex (in the shapes' vertex pool), vertex count,
 *                  first face, face count, first edge, edge count, ok, reserved
 *   face_normals   n_faces x 3            Face::normal
 *   face_ranges    n_faces x 2 u32        first entry (global) in face_vertices / face_edges, count
 *   face_vertices  n_face_entries         vertices_adj_to_face (hull-local vertex ids)
 *   face_edges     n_face_entries         edges_adj_to_face (hull-local edge ids)
 *   vertex_ranges  n_vertices x 2 u32     per vertex of the shapes' pool: first entry (global) in
 *                                         vertex_faces / vertex_edges, count (Vertex)
 *   vertex_faces   n_vertex_entries       faces_adj_to_vertex (hull-local face ids)
 *   vertex_edges   n_vertex_entries       edges_adj_to_vertex (hull-local edge ids)
 *   edge_dirs      n_edges x 3            Edge::dir */
typedef struct parrygpu_polyhedra {
  uint64_t n_hulls;
  const uint32_t* hulls;
  uint64_t n_faces;
  const float* face_normals;
  const uint32_t* face_ranges;
  uint64_t n_face_entries;
  const uint32_t* face_vertices;
  const uint32_t* face_edges;
  const uint32_t* vertex_ranges;
  uint64_t n_vertex_entries;
  const uint32_t* vertex_faces;
  const uint32_t* vertex_edges;
  uint64_t n_edges;
  const float* edge_dirs;
} parrygpu_polyhedra;

/* A set of shapes with their poses (SoA). Convex and triangle vertices live in one pool.
 * polyhedra (may be NULL) carries the topology the manifold generators need for CONVEX shapes. */
typedef struct parrygpu_shapes {
  uint64_t n;
  const uint32_t* types;   /* n */
  const float* params;     /* n x 4 */
  const float* poses;      /* n x 7 (pose7) */
  const float* vertices;   /* n_vertices x 3 */
  uint64_t n_vertices;
  const parrygpu_polyhedra* polyhedra;
} parrygpu_shapes;

/* ConvexPolyhedron::from_convex_hull (src/shape/convex_polyhedron.rs:264-268) for n_hulls point
 * clouds (hull h = points[first[h] .. first[h] + count[h]]), on the host with `threads` threads
 * (0 = all). The triangulation comes from this library's own hull builder (the reference's
 * quickhull numbering is not reproduced: identical triangles for points in general position, other
 * face / vertex ids); from_convex_mesh (:390-639) is restated step for step. As parry's
 * convex_hull, a coplanar cloud gets a double-sided polygon (two faces); a hull whose points span
 * less than 2-D keeps its points with no topology (ok = 0). Read the result with
 * parrygpu_polyhedra_sizes (points, faces, face entries, vertex entries, edges) and
 * parrygpu_polyhedra_copy (buffers sized from those counts; hulls: n_hulls x 8). */
typedef struct parrygpu_polyhedra_builder parrygpu_polyhedra_builder;
parrygpu_status parrygpu_polyhedra_build(const float* points, const uint32_t* first, const uint32_t* count, uint64_t n_hulls,
                                         uint32_t threads, parrygpu_polyhedra_builder** out);
parrygpu_status parrygpu_polyhedra_sizes(const parrygpu_polyhedra_builder* b, uint64_t* sizes);
parrygpu_status parrygpu_polyhedra_copy(const parrygpu_polyhedra_builder* b, float* points, uint32_t* hulls, float* face_normals,
                                        uint32_t* face_ranges, uint32_t* face_vertices, uint32_t* face_edges, uint32_t* vertex_ranges,
                                        uint32_t* vertex_faces, uint32_t* vertex_edges, float* edge_dirs);
/* transformation::convex_hull's triangulation of each cloud (src/transformation/convex_hull3/
 * convex_hull.rs:13-27: closed, counter-clockwise seen from outside, the (vertices, indices) pair
 * that check_convex_hull validates), before from_convex_mesh merges coplanar triangles: 3 hull-local
 * vertex ids per triangle (into the hull's points as parrygpu_polyhedra_copy returns them, whose
 * order is utils::remove_unused_points'); tri_ranges = n_hulls x (first triangle, count). Any output
 * may be NULL; *n_triangles receives the total. */
parrygpu_status parrygpu_polyhedra_triangles(const parrygpu_polyhedra_builder* b, uint64_t* n_triangles, uint32_t* tri_ranges,
                                             uint32_t* triangles);
void parrygpu_polyhedra_builder_destroy(parrygpu_polyhedra_builder* b);

/* The same build on the GPU (one thread per cloud; the host builder's algorithm, the same bytes):
 * points = n_points x 3, first / count = n_hulls (host or device; clouds of at most 65535 points).
 * The result stays in device arrays owned by the handle: parrygpu_polyhedra_gpu_view gives a
 * parrygpu_polyhedra of device pointers (and the hull points) to pass straight to the shape set,
 * parrygpu_polyhedra_gpu_sizes / _copy read it out in the host builder's layout. */
typedef struct parrygpu_polyhedra_gpu parrygpu_polyhedra_gpu;
parrygpu_status parrygpu_polyhedra_build_gpu(parrygpu_ctx* ctx, const float* points, uint64_t n_points, const uint32_t* first,
                                             const uint32_t* count, uint64_t n_hulls, parrygpu_polyhedra_gpu** out);
parrygpu_status parrygpu_polyhedra_gpu_sizes(const parrygpu_polyhedra_gpu* g, uint64_t* sizes);
parrygpu_status parrygpu_polyhedra_gpu_copy(parrygpu_ctx* ctx, const parrygpu_polyhedra_gpu* g, float* points, uint32_t* hulls,
                                            float* face_normals, uint32_t* face_ranges, uint32_t* face_vertices, uint32_t* face_edges,
                                            uint32_t* vertex_ranges, uint32_t* vertex_faces, uint32_t* vertex_edges, float* edge_dirs);
parrygpu_status parrygpu_polyhedra_gpu_view(const parrygpu_polyhedra_gpu* g, const float** points, parrygpu_polyhedra* view);
/* The GPU build's triangulations, as parrygpu_polyhedra_triangles (host or device buffers). */
parrygpu_status parrygpu_polyhedra_gpu_triangles(parrygpu_ctx* ctx, const parrygpu_polyhedra_gpu* g, uint64_t* n_triangles,
                                                 uint32_t* tri_ranges, uint32_t* triangles);
void parrygpu_polyhedra_gpu_destroy(parrygpu_polyhedra_gpu* g);

/* Same layout as the reference's Contact (src/query/contact/contact.rs:71-105), world space. */
typedef struct parrygpu_contact {
  float point1[3];
  float point2[3];
  float normal1[3];
  float normal2[3];
  float dist;
} parrygpu_contact;

typedef struct parrygpu_gjk_stats {
  uint64_t gjk_iterations;  /* support evaluations inside GJK loops */
  uint64_t epa_iterations;  /* support evaluations inside EPA loops */
  uint64_t epa_calls;
  uint64_t reserved;
} parrygpu_gjk_stats;

/* Replaces Shape::compute_aabb(pos) (src/bounding_volume/aabb_ball.rs:25-27, aabb_cuboid.rs:9-14,
 * aabb_capsule.rs:8-10, aabb_convex_polyhedron.rs:8-10) followed by Aabb::loosened(margin)
 * (src/bounding_volume/aabb.rs:982) when margin > 0. aabbs: n x 6 floats. */
parrygpu_status parrygpu_shapes_aabbs(parrygpu_ctx* ctx, const parrygpu_shapes* shapes, float margin, float* aabbs);
/* Replaces a loop of query::contact(pos_a, a, pos_b, b, prediction) over the (a, b) rows of `pairs`
 * (src/query/contact/contact_shape_shape.rs:123-138 -> DefaultQueryDispatcher::contact,
 * src/query/default_query_dispatcher.rs:302-356). out[k] is written and has_contact[k] = 1 for
 * Some(contact); has_contact[k] = 0 for None. init_dirs (n_pairs x 3, may be NULL) is the
 * init_dir warm start of contact_support_map_support_map_with_params
 * (src/query/contact/contact_support_map_support_map.rs:40-62), used by pairs that take the
 * GJK/EPA path; NULL gives the reference default. stats may be NULL (else the call synchronises). */
parrygpu_status parrygpu_contacts(parrygpu_ctx* ctx, const parrygpu_shapes* shapes, const uint32_t* pairs, uint64_t n_pairs,
                                  float prediction, const float* init_dirs, parrygpu_contact* out, uint8_t* has_contact,
                                  parrygpu_gjk_stats* stats);

/* Same as parrygpu_contacts, and also writes final_dirs[k] (n_pairs x 3, may be NULL): the
 * direction the reference's GJK/EPA ends with, in the first shape's local frame - the contact
 * normal1 for ClosestPoints (closest points or EPA), the separating direction for NoIntersection,
 * zero for pairs that take the ball paths. These are the labels of the learned warm start. */
parrygpu_status parrygpu_contacts_with_dirs(parrygpu_ctx* ctx, const parrygpu_shapes* shapes, const uint32_t* pairs, uint64_t n_pairs,
                                            float prediction, const float* init_dirs, parrygpu_contact* out, uint8_t* has_contact,
                                            parrygpu_gjk_stats* stats, float* final_dirs);

/* ---- persistent contact manifolds ----
 * One fixed-size record per pair, the reference's ContactManifold<(), f32-data> with
 * TrackedContact points (src/query/contact_manifolds/contact_manifold.rs:108-226, 662-800).
 * 24 points bound every supported pair (face-face cuboids: 4 + 4 vertex and 16 edge contacts). */
#define PARRYGPU_MANIFOLD_MAX_POINTS 24

typedef struct parrygpu_tracked_contact {
  float local_p1[3]; /* in shape 1's local frame */
  float local_p2[3]; /* in shape 2's local frame */
  float dist;        /* negative when penetrating */
  uint32_t fid1;     /* PackedFeatureId: kind in bits 30-31 (1 vertex, 2 edge, 3 face, 0 unknown) */
  uint32_t fid2;
  float data;        /* user payload (e.g. an impulse), 0 for a new contact, carried by match_contacts */
} parrygpu_tracked_contact;

typedef struct parrygpu_manifold {
  uint32_t n_points;
  uint32_t status;   /* PARRYGPU_OK, or PARRYGPU_UNSUPPORTED_PAIR / PARRYGPU_INVALID_ARG for that pair */
  float local_n1[3]; /* contact normal in shape 1's frame (also the GJK warm-start cache) */
  float local_n2[3];
  parrygpu_tracked_contact points[PARRYGPU_MANIFOLD_MAX_POINTS];
} parrygpu_manifold;

/* Replaces a loop of DefaultQueryDispatcher::contact_manifold_convex_convex(pos_a^-1 pos_b, a, b,
 * None, None, prediction, &mut manifold) over the (a, b) rows of `pairs`
 * (src/query/default_query_dispatcher.rs:749-831), updating `manifolds` (n_pairs records, host or
 * device memory) in place: try_update_contacts, then the ball-ball, cuboid-cuboid (SAT + feature
 * clipping), capsule-capsule, convex-ball and polygonal-feature-map (GJK/EPA + clipping) generators,
 * then match_contacts; triangles take the convex-ball, cuboid-triangle (SAT + clipping) and
 * polygonal-feature-map paths. Zeroed records are ContactManifold::new(). Pairs with a shape that has
 * no generator (a convex hull given without ConvexPolyhedron topology, a segment) get status
 * PARRYGPU_UNSUPPORTED_PAIR and keep their record (the reference's Err(Unsupported) leaves the
 * manifold untouched). A row (PARRYGPU_PAIR_NONE, PARRYGPU_PAIR_NONE) is an empty slot: skipped, its
 * record and status untouched. stats may be NULL (else the call synchronises). */
#define PARRYGPU_PAIR_NONE 0xFFFFFFFFu
parrygpu_status parrygpu_contact_manifolds(parrygpu_ctx* ctx, const parrygpu_shapes* shapes, const uint32_t* pairs, uint64_t n_pairs,
                                           float prediction, parrygpu_manifold* manifolds, parrygpu_gjk_stats* stats);
/* parrygpu_contact_manifolds with a GJK start direction per pair for the polygonal-feature-map
 * generator (init_dirs: n_pairs x 3 floats, host or device; NULL = none). A pair's direction is used
 * where its record holds no cached normal (local_n1 does not normalise, e.g. a new pair);
 * contact_manifolds_pfm_pfm.rs:67-76 otherwise starts from the relative translation. A row that does
 * not normalise keeps that default. This is the hook the learned warm start seeds new pairs through. */
parrygpu_status parrygpu_contact_manifolds_with_dirs(parrygpu_ctx* ctx, const parrygpu_shapes* shapes, const uint32_t* pairs,
                                                     uint64_t n_pairs, float prediction, const float* init_dirs,
                                                     parrygpu_manifold* manifolds, parrygpu_gjk_stats* stats);

/* ---- per-frame pipeline over moving shapes ----
 * No single reference counterpart: one frame chains the parry calls a physics engine makes each step
 * on a set of convex shapes —
 *   pose integration (decision D-5, parry has no integrator: x += v dt; q := normalize(q + dt/2 (0, w) q)),
 *   Shape::compute_aabb(pos).loosened(prediction / 2) (aabb.rs:982), Bvh refit (bvh_refit.rs:170),
 *   Bvh::traverse_bvtt_single_tree (bvh_traverse_bvtt.rs:19), contact_manifold_convex_convex per pair
 *   (default_query_dispatcher.rs:749) with each pair's manifold kept from the previous frame while the
 *   pair persists (a new pair starts from ContactManifold::new()), and
 *   RayCast::cast_ray_and_get_normal of a fixed ray set against the shapes (Compound semantics,
 *   ray_composite_shape.rs:86-105, lowest shape index on exact ties).
 * velocities: n x 6 floats (linear xyz, angular xyz, world frame). The scene copies every input; the
 * BVH is built once at creation and refit each frame. pair_capacity bounds the pairs kept per frame
 * (pairs beyond it are dropped and raise CAPACITY_EXCEEDED at the next sync). */
typedef struct parrygpu_scene parrygpu_scene;
parrygpu_status parrygpu_scene_create(parrygpu_ctx* ctx, const parrygpu_shapes* shapes, const float* velocities, float prediction,
                                      uint64_t pair_capacity, parrygpu_scene** out);
void parrygpu_scene_destroy(parrygpu_scene* scene);
/* The rays cast each frame (n x 6 floats) and their max_toi; outputs are read with parrygpu_scene_read. */
parrygpu_status parrygpu_scene_set_rays(parrygpu_ctx* ctx, parrygpu_scene* scene, const float* rays, uint64_t n_rays, float max_toi);
/* Advances `frames` frames of duration dt, asynchronously. With use_graph != 0 the frame pair is
 * captured once into a CUDA graph (re-captured when dt or the rays change) and replayed. */
parrygpu_status parrygpu_scene_step(parrygpu_ctx* ctx, parrygpu_scene* scene, float dt, uint32_t frames, int use_graph);
/* Frames advanced so far and the current frame's pair count (synchronises; reports device errors). */
parrygpu_status parrygpu_scene_info(parrygpu_ctx* ctx, const parrygpu_scene* scene, uint64_t* frame, uint64_t* n_pairs);
/* Copies the current state (every pointer may be NULL): poses (n x 7), the first min(cap, n_pairs)
 * pairs (2 x u32, unsorted) with their manifold records, and the last frame's ray results (shape
 * index or UINT32_MAX, toi, world normal). Synchronises. */
parrygpu_status parrygpu_scene_read(parrygpu_ctx* ctx, const parrygpu_scene* scene, float* poses, uint32_t* pairs,
                                    parrygpu_manifold* manifolds, uint64_t cap, uint32_t* ray_part, float* ray_toi, float* ray_normal);
/* parrygpu_scene_read without waiting for the copies: returns once the current frame has finished
 * and its outputs' copies are queued on a copy stream (*n_pairs = the pair rows copied), so the next
 * frames (parrygpu_scene_step, eager) run while the copies proceed; their kernels that overwrite what
 * the copies read wait for them on the device. The host buffers hold the frame's outputs once
 * parrygpu_scene_read_wait returns; they must be page-locked for the copies to overlap. A further
 * read waits for this one first. */
parrygpu_status parrygpu_scene_read_async(parrygpu_ctx* ctx, parrygpu_scene* scene, float* poses, uint32_t* pairs,
                                          parrygpu_manifold* manifolds, uint64_t cap, uint32_t* ray_part, float* ray_toi, float* ray_normal,
                                          uint64_t* n_pairs);
/* Waits for the copies of the last parrygpu_scene_read_async (returns at once when none is in flight). */
parrygpu_status parrygpu_scene_read_wait(parrygpu_ctx* ctx, parrygpu_scene* scene);
/* The last frame's narrow-phase counters (synchronises): GJK and EPA iterations and EPA calls of its
 * manifold updates, and (seeded_pairs, may be NULL) how many pairs took a learned GJK start direction
 * (parrygpu_scene_set_mlp; 0 without a network). */
parrygpu_status parrygpu_scene_stats(parrygpu_ctx* ctx, const parrygpu_scene* scene, parrygpu_gjk_stats* stats, uint64_t* seeded_pairs);

/* ---- learned GJK warm start (no reference counterpart: parry's init_dir hook is its only tie) ----
 * A 39 -> 128 -> 128 -> 128 -> 128 -> 3 MLP (GELU, BF16 weights and activations, FP32 accumulation
 * on the tensor cores) predicts contact_support_map_support_map_with_params's init_dir from the
 * relative pose (7) and a 16-float descriptor per shape. Inputs are padded to 48 features. */
typedef struct parrygpu_mlp parrygpu_mlp;

#define PARRYGPU_MLP_IN 48
#define PARRYGPU_MLP_HIDDEN 128
#define PARRYGPU_MLP_LAYERS 5

/* Xavier-uniform initialisation from `seed`. */
parrygpu_status parrygpu_mlp_create(parrygpu_ctx* ctx, uint64_t seed, parrygpu_mlp** out);
void parrygpu_mlp_destroy(parrygpu_mlp* mlp);
/* Pair features (n_pairs x 48 floats: relative pose of b in a's frame, descriptors of a and b) into a
 * 16-byte aligned buffer. Asynchronous when every buffer is on the device; synchronises otherwise. */
parrygpu_status parrygpu_mlp_features(parrygpu_ctx* ctx, const parrygpu_shapes* shapes, const uint32_t* pairs, uint64_t n_pairs,
                                      float* features);
/* Trains on (features, unit target directions) with Adam for `epochs` passes in minibatches of
 * `batch` pairs (loss = mean(1 - cos(prediction, target))). loss_per_epoch (epochs floats) may be NULL. */
parrygpu_status parrygpu_mlp_train(parrygpu_ctx* ctx, parrygpu_mlp* mlp, const float* features, const float* targets, uint64_t n,
                                   uint32_t epochs, uint32_t batch, float lr, float* loss_per_epoch);
/* Predicted unit init directions (n x 3). Degenerate outputs fall back to the reference default
 * (the relative translation, else +x), which the caller passes as is. */
parrygpu_status parrygpu_mlp_predict(parrygpu_ctx* ctx, const parrygpu_mlp* mlp, const float* features, uint64_t n, float* dirs);
/* Loss and gradients of one batch without updating (gradient checks): grads receives the
 * parameters' gradients in the layout of parrygpu_mlp_get_params. */
parrygpu_status parrygpu_mlp_loss_and_grads(parrygpu_ctx* ctx, const parrygpu_mlp* mlp, const float* features, const float* targets,
                                            uint64_t n, float* loss, float* grads);
/* Number of parameters (float32 master weights and biases, layer by layer: W [out x in] then b). */
uint64_t parrygpu_mlp_param_count(void);
/* Copies the FP32 master parameters out / in (checkpoint and resume; the BF16 copies follow). */
parrygpu_status parrygpu_mlp_get_params(parrygpu_ctx* ctx, const parrygpu_mlp* mlp, float* params);
parrygpu_status parrygpu_mlp_set_params(parrygpu_ctx* ctx, parrygpu_mlp* mlp, const float* params);
/* Seeds the scene's polygonal-feature-map pairs that hold no cached normal (the pairs new in a frame)
 * with the network's GJK start direction, as parrygpu_contact_manifolds_with_dirs does; pairs that
 * persist keep their cached normal. Each frame the pairs are listed on the device, their features
 * computed and the network run by the fused tensor-core kernel, all inside the frame (and its graph).
 * The scene keeps a snapshot of the weights taken by this call (later training does not reach it
 * until the call is repeated) and computes the shape descriptors once. mlp = NULL turns seeding off. */
parrygpu_status parrygpu_scene_set_mlp(parrygpu_ctx* ctx, parrygpu_scene* scene, const parrygpu_mlp* mlp);

/* ---- contact manifolds against a TriMesh ------------------------------------------------- */

typedef struct parrygpu_trimesh_contacts parrygpu_trimesh_contacts;

/* Replaces, for n_shapes shapes against one TriMesh, the per-pair state of
 * contact_manifolds_trimesh_shape (src/query/contact_manifolds/contact_manifolds_trimesh_shape.rs:
 * 82-228): its TriMeshShapeContactManifoldsWorkspace (the shape's AABB in the mesh frame and the
 * interfering triangles) and one ContactManifold per interfering triangle. Each shape holds at most
 * max_per_shape triangles at once (more raises PARRYGPU_CAPACITY_EXCEEDED at the next sync). */
parrygpu_status parrygpu_trimesh_contacts_create(parrygpu_ctx* ctx, const parrygpu_trimesh* mesh, uint32_t n_shapes, uint32_t max_per_shape,
                                                 parrygpu_trimesh_contacts** out);
void parrygpu_trimesh_contacts_destroy(parrygpu_trimesh_contacts* contacts);
/* One frame: for every shape s (shapes->n == n_shapes) the reference's
 * contact_manifolds_trimesh_shape(dispatcher, mesh_pose^-1 * pose_s, mesh, shape_s, prediction,
 * manifolds, workspace) with the mesh as shape 1; when the mesh has FIX_INTERNAL_EDGES
 * (parrygpu_trimesh_set_flags) each triangle's pseudo-normals constrain its manifolds' normals.
 * mesh_pose7: host pointer to the mesh pose, NULL = identity. Interfering triangles are kept in
 * ascending index order. */
parrygpu_status parrygpu_trimesh_contacts_update(parrygpu_ctx* ctx, parrygpu_trimesh_contacts* contacts, const float* mesh_pose7,
                                                 const parrygpu_shapes* shapes, float prediction);
/* Copies the current state (host or device buffers; any may be NULL): counts (n_shapes), triangles
 * (n_shapes x max_per_shape: slot j of shape s is valid for j < counts[s]) and the manifold of each
 * slot (n_shapes x max_per_shape records; shape 1 of a record is the triangle). Synchronises. */
parrygpu_status parrygpu_trimesh_contacts_read(parrygpu_ctx* ctx, const parrygpu_trimesh_contacts* contacts, uint32_t* counts,
                                               uint32_t* triangles, parrygpu_manifold* manifolds);

/* ---- shape casting (time of impact under translation) ------------------------------------- */

/* ShapeCastOptions (src/query/shape_cast/shape_cast.rs:230-270); the reference's default is
 * {FLT_MAX, 0, 1, 1}. */
typedef struct parrygpu_shape_cast_options {
  float max_time_of_impact;
  float target_distance;
  uint32_t stop_at_penetration;
  uint32_t compute_impact_geometry_on_penetration;
} parrygpu_shape_cast_options;

/* ShapeCastHit (shape_cast.rs:40-60): witness points and normals in each shape's local frame. */
typedef struct parrygpu_shape_cast_hit {
  float time_of_impact;
  float witness1[3];
  float witness2[3];
  float normal1[3];
  float normal2[3];
} parrygpu_shape_cast_hit;

/* ShapeCastStatus values written per pair; PARRYGPU_CAST_NONE where the reference returns None. */
enum {
  PARRYGPU_CAST_OUT_OF_ITERATIONS = 0,
  PARRYGPU_CAST_CONVERGED = 1,
  PARRYGPU_CAST_FAILED = 2,
  PARRYGPU_CAST_PENETRATING_OR_WITHIN_TARGET_DIST = 3,
  PARRYGPU_CAST_NONE = 255
};

/* Replaces a loop of query::cast_shapes(pos_a, vel_a, a, pos_b, vel_b, b, options)
 * (src/query/shape_cast/shape_cast.rs:275-286 -> DefaultQueryDispatcher::cast_shapes,
 * src/query/default_query_dispatcher.rs:434-538) over the (a, b) rows of `pairs`, for balls
 * (cast_shapes_ball_ball) and support-map shapes (cuboid, capsule, convex, triangle:
 * cast_shapes_support_map_support_map). velocities: one linear velocity per shape (n x 3 floats).
 * out[k] / status[k] receive the hit of pair k. stats (may be NULL; else the call synchronises)
 * counts the GJK / EPA work of the penetration contacts. */
parrygpu_status parrygpu_cast_shapes(parrygpu_ctx* ctx, const parrygpu_shapes* shapes, const uint32_t* pairs, uint64_t n_pairs,
                                     const float* velocities, const parrygpu_shape_cast_options* options, parrygpu_shape_cast_hit* out,
                                     uint8_t* status, parrygpu_gjk_stats* stats);

/* ---- Compound (shape set) ray casts ------------------------------------------------------- */

/* Replaces Compound::new(shapes) (src/shape/compound.rs:113-144): copies the parts (with their poses)
 * to the device and builds an LBVH over their world AABBs. Leaf data = part index. */
parrygpu_status parrygpu_compound_create(parrygpu_ctx* ctx, const parrygpu_shapes* shapes, parrygpu_compound** out);
void parrygpu_compound_destroy(parrygpu_compound* compound);
/* Moves the parts (n x 7 poses) and refits the compound's BVH (topology kept). */
parrygpu_status parrygpu_compound_set_poses(parrygpu_ctx* ctx, parrygpu_compound* compound, const float* poses);
/* Replaces a loop of RayCast::cast_ray_and_get_normal(m, ray, max_toi, solid) on a Compound
 * (src/query/ray/ray.rs:393-403 -> src/query/ray/ray_composite_shape.rs:95-104). pose7 = the
 * compound's pose (NULL = identity). Outputs per ray: part index (UINT32_MAX on a miss), toi and
 * world-space normal (normal may be NULL). Exact toi ties resolve to the lowest part index. */
parrygpu_status parrygpu_compound_cast_rays(parrygpu_ctx* ctx, const parrygpu_compound* compound, const float* pose7, const float* rays,
                                            uint32_t n, float max_toi, int solid, uint32_t* part, float* toi, float* normal);

/* ---- launch-configuration autotuner -------------------------------------------------------- */
/* No reference counterpart (parry runs on the CPU). Answers never depend on the configuration;
 * these only pick how the same work maps onto the SMs, for the caller's own inputs. */

/* Copies the context's current configuration into *out. */
parrygpu_status parrygpu_get_config(const parrygpu_ctx* ctx, parrygpu_config* out);
/* Times parrygpu_trimesh_cast_rays on `rays` (device or host; copied to the device once, outputs
 * kept on the device) for each candidate ray ordering (input order; 30-bit Morton; octant + 27-bit
 * Morton; 16-bit Morton prefix) x traversal (one ray per thread, and postponed leaves, at 64, 128,
 * 256 threads per block; dynamic fetch refilling at 8, 16, 24 idle lanes): one untimed run then
 * `reps` timed runs each (0 = 3). The fastest candidate becomes the context's configuration and is
 * copied to *chosen (may be NULL). On an error the configuration is left unchanged. */
parrygpu_status parrygpu_autotune_trimesh_rays(parrygpu_ctx* ctx, const parrygpu_trimesh* mesh, const float* pose7, const float* rays,
                                               uint32_t n, float max_toi, uint32_t reps, parrygpu_config* chosen);
/* Times parrygpu_contacts on (shapes, pairs) for each EPA residency (4, 6, 8, 12, 16 blocks per
 * SM, one thread per pair, EPA through the queue), then at the best residency with the pairs of cost
 * 512 or more, then 256 or more, one warp each, and with EPA right after GJK in the same thread;
 * `reps` timed runs each (0 = 2); keeps the fastest as for the ray tuner. */
parrygpu_status parrygpu_autotune_contacts(parrygpu_ctx* ctx, const parrygpu_shapes* shapes, const uint32_t* pairs, uint64_t n_pairs,
                                           float prediction, uint32_t reps, parrygpu_config* chosen);

#ifdef __cplusplus
}
#endif

#endif /* PARRY_GPU_H */
