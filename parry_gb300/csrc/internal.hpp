// Internal declarations shared by the translation units of libparrygpu.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>
#include <map>
#include <utility>
#include "../../include/parry_gpu.h"

// Device-side error word bits (set by kernels, read and cleared by parrygpu_sync).
enum : uint32_t {
  ERR_STACK_OVERFLOW = 1u << 0,
  ERR_CAPACITY = 1u << 1,
  ERR_TIMEOUT = 1u << 2,
  ERR_POLYTOPE_FULL = 1u << 3,
  ERR_BAD_INDEX = 1u << 4,
};

// A grow-only device buffer owned by a context or a handle.
struct DevBuf {
  void* ptr = nullptr;
  size_t bytes = 0;
  cudaError_t reserve(size_t need) {
    if (need <= bytes) return cudaSuccess;
    if (ptr) { cudaError_t e = cudaFree(ptr); if (e != cudaSuccess) return e; ptr = nullptr; bytes = 0; }
    size_t cap = need < 256 ? 256 : need;
    cudaError_t e = cudaMalloc(&ptr, cap);
    if (e == cudaSuccess) bytes = cap;
    return e;
  }
  void release() { if (ptr) cudaFree(ptr); ptr = nullptr; bytes = 0; }
  template <class T> T* as() const { return (T*)ptr; }
};

// Scratch of the wavefront shape-set ray cast (shape_ray.cu): candidate list, its counter, one
// best-hit key and one overflow flag per ray.
struct RayWaveScratch {
  DevBuf cands, counter, keys, ovf;
  uint64_t cap = 0;
};

// A uniform grid over a shape set's AABBs, rebuilt on the device each frame (shape_ray.cu): cell
// ranges into the entry array (shape indices), the grid's placement (from the BVH root box), its
// resolution (fixed when the scratch is reserved) and the entry capacity.
struct RayGridScratch {
  DevBuf dev, starts, cursor, entries, sums;
  uint32_t res[3] = {0, 0, 0};
  uint64_t cells = 0, cap = 0;
};

// Scratch of the contact-manifold kernels (manifold.cu): EPA queue, counters (queue length, stats,
// bin lengths), per-kind pair bins, per-slot EPA polytope workspaces.
struct MfScratch {
  DevBuf queue, counters, bins, epa_ws;
  uint64_t cap = 0;
};

struct parrygpu_ctx {
  int device = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  parrygpu_config cfg{};
  std::string last_error;
  uint64_t launches = 0;
  uint32_t* d_err = nullptr;    // device error word
  uint32_t* h_err = nullptr;    // pinned mirror
  // Scratch reused across calls (sort buffers, staging of host inputs/outputs, counters).
  DevBuf sort_k[2], sort_v[2], sort_hist, stage_in[8], stage_out[4], misc, counters, stage_poly[9];
  DevBuf ray_keys, ray_order;
  // contact pipeline scratch: EPA queue (pair + simplex per entry) and per-slot polytope workspaces
  DevBuf ct_queue, ct_counters, epa_ws, epa_ws_big, ct_ovf;
  RayWaveScratch ray_wave;
  MfScratch mf;
  int sm_count = 0;
  bool coherent_host = false;  // the device reads pageable host memory through the host's page tables (Grace NVLink-C2C)
  // Second stream for pipelined host-buffer calls (chunks alternate between it and `stream`),
  // with the fork / join events that order it after and before the context stream's work.
  cudaStream_t aux_stream = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  // Copy streams and per-chunk events of the pipelined host-record manifold update (uploads on one,
  // downloads on the other, compute on `stream`).
  cudaStream_t up_stream = nullptr, down_stream = nullptr;
  static constexpr int PIPE_EVENTS = 16;
  cudaEvent_t pipe_ev[PIPE_EVENTS] = {};
  unsigned long long* h_pipe = nullptr;  // pinned, PIPE_EVENTS words: per-chunk figures read back by a pipelined call
  // Optional per-kernel event timing (parrygpu_enable_kernel_timing).
  bool timing = false;
  std::map<std::string, std::vector<std::pair<cudaEvent_t, cudaEvent_t>>> pending;
  std::map<std::string, std::pair<double, uint64_t>> timed;
};

// Brackets one kernel launch with CUDA events when the context has timing enabled.
struct KernelTimer {
  parrygpu_ctx* ctx;
  const char* name;
  cudaEvent_t a = nullptr, b = nullptr;
  KernelTimer(parrygpu_ctx* c, const char* n) : ctx(c), name(n) {
    if (ctx->timing && cudaEventCreate(&a) == cudaSuccess && cudaEventCreate(&b) == cudaSuccess) cudaEventRecord(a, ctx->stream);
    else { a = b = nullptr; cudaGetLastError(); }
  }
  void stop() {
    if (!a) return;
    cudaEventRecord(b, ctx->stream);
    ctx->pending[name].push_back({a, b});
    a = b = nullptr;
  }
};

struct parrygpu_bvh {
  uint32_t n_leaves = 0;
  uint32_t n_wide = 0;
  DevBuf wide;          // n_wide x 64 B  (BvhNodeWide layout)
  DevBuf leaf_parent;   // per sorted leaf: (wide << 1) | side
  DevBuf node_parent;   // per internal node: (wide << 1) | side, root = UINT32_MAX
  DevBuf leaf_index;    // sorted position -> leaf data (user index)
  DevBuf flags;         // per internal node arrival counters for the bottom-up fit
  DevBuf info;          // per internal node: (split position gamma, last sorted leaf of its range)
  DevBuf root_aabb;     // 6 floats
  bool leaf_data_is_position = false;
  uint32_t id_bound = 0;  // 1 + the largest leaf index (= n_leaves for a tree built over 0..n-1)
};

struct parrygpu_trimesh {
  uint32_t n_vertices = 0, n_triangles = 0;
  parrygpu_bvh bvh;     // leaves store the sorted position of the triangle in `soup`
  DevBuf soup;          // per sorted position: a.xyz b.x | b.yz c.xy | c.z orig 0 0  (3 x float4)
  uint32_t flags = 0;   // TriMeshFlags bits
  DevBuf pseudo;        // with FIX_INTERNAL_EDGES: per original triangle, TrianglePseudoNormals (12 floats)
  DevBuf pseudo_ok;     // per original triangle: 1 when triangle_normal_constraints is Some
  bool constrained() const { return (flags & PARRYGPU_TRIMESH_FIX_INTERNAL_EDGES) == PARRYGPU_TRIMESH_FIX_INTERNAL_EDGES && pseudo.ptr; }
};

// A shape set under one BVH (the reference's Compound), with device copies of the shape arrays.
struct parrygpu_compound {
  uint64_t n = 0, n_vertices = 0;
  DevBuf types, params, poses, pool, aabbs, hull_box;
  parrygpu_bvh bvh;
};

// ---- status helpers ----
parrygpu_status set_error(parrygpu_ctx* ctx, parrygpu_status s, const char* fmt, ...);
parrygpu_status check_cuda(parrygpu_ctx* ctx, cudaError_t e, const char* what);
#define PG_CUDA(ctx, call)                                                   \
  do {                                                                       \
    cudaError_t _e = (call);                                                 \
    if (_e != cudaSuccess) return check_cuda((ctx), _e, #call);              \
  } while (0)
#define PG_LAUNCHED(ctx)                                                     \
  do {                                                                       \
    (ctx)->launches++;                                                       \
    cudaError_t _e = cudaGetLastError();                                     \
    if (_e != cudaSuccess) return check_cuda((ctx), _e, "kernel launch");    \
  } while (0)

// ---- host/device pointer staging ----
bool is_device_ptr(const void* p);
// Device memory, or page-locked host memory with a device mapping (readable by kernels in place).
bool is_addressable(const void* p);
// True when p is device memory of a GPU other than `device` (managed and host memory: false).
bool on_other_device(const void* p, int device);
// The device-side address of an addressable pointer (the same value under unified addressing).
void* device_view_ptr(const void* p);
template <class T> inline T* device_view(T* p) { return static_cast<T*>(device_view_ptr(p)); }
template <class T> inline const T* device_view(const T* p) { return static_cast<const T*>(device_view_ptr(p)); }
// Returns a device pointer holding `bytes` of `src` (src itself when already on the device).
parrygpu_status stage_input(parrygpu_ctx* ctx, DevBuf& buf, const void* src, size_t bytes, const void** dptr);
// Returns a device pointer for an output of `bytes`; *needs_copy tells whether `dst` is host memory.
parrygpu_status stage_output(parrygpu_ctx* ctx, DevBuf& buf, void* dst, size_t bytes, void** dptr, bool* needs_copy);

// ---- radix sort (sort.cu) ----
// Stable LSD sort of (keys, values) by the low `key_bits` bits. In/out in ctx scratch; returns the
// buffer index (0/1) holding the result in ctx->sort_k / ctx->sort_v.
parrygpu_status radix_sort_pairs(parrygpu_ctx* ctx, uint32_t n, int key_bits, int* result_buf);
parrygpu_status radix_sort_reserve(parrygpu_ctx* ctx, uint32_t n);
// The same sort on caller-provided device buffers (no allocation); hist needs
// radix_sort_hist_entries(n) words.
parrygpu_status radix_sort_pairs_in(parrygpu_ctx* ctx, uint32_t n, int key_bits, uint32_t* k0, uint32_t* v0, uint32_t* k1,
                                    uint32_t* v1, uint32_t* hist, int* result_buf);
uint32_t radix_sort_hist_entries(uint32_t n);
// In-place exclusive prefix sum of m words (buffer padded to a multiple of 4 words with zeros).
parrygpu_status exclusive_scan_u32(parrygpu_ctx* ctx, uint32_t* data, uint32_t m);
// The same over many blocks for long arrays (tile sums, one-block scan of the sums, tile scans);
// `sums` holds exclusive_scan_u32_sums(m) words. No allocation, no host synchronisation.
uint32_t exclusive_scan_u32_sums(uint32_t m);
parrygpu_status exclusive_scan_u32_wide(parrygpu_ctx* ctx, uint32_t* data, uint32_t m, uint32_t* sums);

// ---- ray casts (ray.cu): launch helpers on caller-provided device buffers (no allocation) ----
// Key width (bits) of the ray ordering for the context's ray_sort_key mode.
inline int ray_sort_bits(const parrygpu_ctx* ctx) { return ctx->cfg.ray_sort_key == 2 ? 16 : 30; }
parrygpu_status launch_ray_keys(parrygpu_ctx* ctx, const float* d_rays, uint32_t n, uint32_t* bounds, uint32_t* keys, uint32_t* vals,
                                uint32_t key_mode);
parrygpu_status launch_trimesh_rays(parrygpu_ctx* ctx, const parrygpu_trimesh* mesh, const float* pose7_host, const float* d_rays,
                                    const uint32_t* order, uint32_t n, float max_toi, uint32_t* d_feat, float* d_toi, float* d_nrm,
                                    uint32_t* counter);

// ---- LBVH (lbvh.cu) ----
// Builds `bvh` from `n` device AABBs (n x 6 floats). When leaf_data_is_position, leaf nodes store
// their sorted position instead of the AABB index.
// d_ids (may be null): leaf data of input leaf i is d_ids[i] instead of i (then id_bound = max id + 1).
parrygpu_status lbvh_build(parrygpu_ctx* ctx, parrygpu_bvh* bvh, const float* d_aabbs, uint32_t n, bool leaf_data_is_position,
                           const uint32_t* d_ids = nullptr, uint32_t id_bound = 0);
parrygpu_status lbvh_refit(parrygpu_ctx* ctx, parrygpu_bvh* bvh, const float* d_aabbs);
// traverse_bvtt_single_tree into device buffers: pairs beyond `cap` are counted in *d_count but not
// written. No allocation, no host synchronisation.
parrygpu_status launch_self_pairs(parrygpu_ctx* ctx, const parrygpu_bvh* bvh, uint32_t* d_pairs, unsigned long long cap,
                                  unsigned long long* d_count);

// ---- shape-set ray casts (shape_ray.cu) on device buffers; `bvh` leaves hold shape indices ----
// `order` (may be null): thread k casts ray order[k], stored at slot k of d_rays (the rays were
// permuted into that order), and writes its results to slot order[k].
// Runs the wavefront cast (shape_ray.cu) with `scratch` sized by shape_rays_reserve(n) beforehand.
parrygpu_status shape_rays_reserve(parrygpu_ctx* ctx, RayWaveScratch& scratch, uint32_t n);
// Local vertex bounds of the convex shapes (2 float4 per shape) for the shape-set ray filter.
parrygpu_status launch_hull_boxes(parrygpu_ctx* ctx, const uint32_t* types, const float* params, const float* pool, uint32_t n,
                                  uint64_t n_vertices, float* box);
parrygpu_status launch_shape_rays(parrygpu_ctx* ctx, const parrygpu_bvh* bvh, const uint32_t* types, const float* params,
                                  const float* poses, const float* pool, const float* hull_box, const float* d_rays, const uint32_t* order,
                                  uint32_t n, float max_toi, uint32_t* d_part, float* d_toi, float* d_nrm, RayWaveScratch& scratch,
                                  RayGridScratch* grid = nullptr, const float* d_aabbs = nullptr);
// Grid resolution for n shapes in the box root[6] (about 4 cells per shape, at most 1024 a side and
// 2^22 cells) and the entry capacity; no allocation happens in the frame afterwards.
parrygpu_status shape_ray_grid_reserve(parrygpu_ctx* ctx, RayGridScratch& grid, uint64_t n_shapes, const float* root);

// ---- shapes (contact.cu) ----
// World AABBs of a compound's parts (Shape::compute_aabb(pos)) into d_out (n x 6 floats).
parrygpu_status compound_part_aabbs(parrygpu_ctx* ctx, const parrygpu_compound* c, float* d_out);

// Launch configuration helpers.
static inline uint32_t div_up(uint64_t a, uint64_t b) { return (uint32_t)((a + b - 1) / b); }
