// The per-frame query pipeline over a set of moving convex shapes, as a physics engine drives parry
// each frame (no single reference counterpart; each stage replaces the parry call named):
//
//   k_integrate         pose integration, decision D-5 (parry has no integrator): x += v dt,
//                       q := normalize(q + dt/2 (0, w) q)
//   shape AABBs         Shape::compute_aabb(pos).loosened(prediction / 2)   (aabb_*.rs, aabb.rs:982)
//   refit               Bvh::insert_or_update_partially + Bvh::refit       (bvh_insert.rs:209, bvh_refit.rs:170)
//   pairs               Bvh::traverse_bvtt_single_tree                      (bvh_traverse_bvtt.rs:19)
//   k_carry_records     the narrow phase's per-pair manifold persistence: a pair found in the previous
//                       frame keeps its ContactManifold, a new pair starts from ContactManifold::new()
//   manifolds           contact_manifold_convex_convex per pair            (default_query_dispatcher.rs:749);
//                       with a network set (parrygpu_scene_set_mlp), the polyhedral pairs without a
//                       cached normal start GJK from its predicted direction (listed, featurised and
//                       inferred on the device inside the frame)
//   rays                RayCast::cast_ray_and_get_normal on the shape set   (ray_composite_shape.rs:86-105),
//                       walking a uniform grid over the shapes rebuilt each frame (the BVH traversal's
//                       answers; the BVH kernel takes over on the device when the grid overflows)
//
// Everything stays on the device: the pair count lives in device memory and bounds the later kernels,
// buffers are sized at creation (pair capacity), so a frame is a fixed sequence of kernel launches and
// memsets on one stream. parrygpu_scene_step captures two frames (the double buffers swap back) into a
// CUDA graph and replays it.
#include "internal.hpp"
#include "contact_device.cuh"
#include <cstring>

using namespace pg;

struct parrygpu_scene {
  uint64_t n = 0, n_vertices = 0, cap = 0, table_size = 0, n_rays = 0;
  float prediction = 0.0f, max_toi = 0.0f;
  DevBuf types, params, poses, vel, pool, aabbs, hull_box, poly[9];
  parrygpu_polyhedra poly_counts{};
  bool has_poly = false;
  parrygpu_bvh bvh;
  DevBuf pairs[2], recs[2], keys[2], vals[2], counts;
  MfScratch mf;  // narrow-phase scratch owned by the scene (stable for the graph)
  DevBuf rays, ray_order, ray_part, ray_toi, ray_nrm;  // rays stored in Morton order of their origins
  RayWaveScratch ray_wave;
  RayGridScratch ray_grid;  // the rays' uniform grid (cells == 0: the BVH is traversed)
  DevBuf seed_desc, seed_wb, seed_wf, seed_feat, seed_list, seed_dirs;  // learned seeding (parrygpu_scene_set_mlp)
  bool seeded = false;
  int cur = 0;
  uint64_t frame = 0;
  // An asynchronous read (parrygpu_scene_read_async): its copies run on the context's download
  // stream between read_start and read_done, the poses from a snapshot, the pairs and records from
  // buffer parity read_cur, the ray results in place. read_order: the context stream has not yet been
  // ordered after read_done (a frame does so before it overwrites the ray results or that buffer);
  // read_inflight: the host has not yet waited for it.
  DevBuf pose_snap;
  cudaEvent_t read_start = nullptr, read_done = nullptr;
  bool read_order = false, read_inflight = false;
  int read_cur = 0;
  cudaGraphExec_t exec = nullptr;
  float graph_dt = 0.0f;
  int graph_cur = 0;  // the buffer parity the graph was captured at
  uint64_t graph_launches = 0;
};

namespace {

constexpr int SC_THREADS = 256;
constexpr uint32_t DEFAULT_SCENE_RAY_ORDER = 1;  // the origins' Morton order
constexpr int REC_WORDS = 8 + 10 * PARRYGPU_MANIFOLD_MAX_POINTS;
constexpr unsigned long long EMPTY_KEY = ~0ull;

// Decision D-5: explicit Euler on the translation, first-order quaternion update renormalised.
__global__ void k_integrate(float* __restrict__ poses, const float* __restrict__ vel, uint64_t n, float dt) {
  uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  float* p = poses + 7 * i;
  const float* v = vel + 6 * i;
  float qi = p[0], qj = p[1], qk = p[2], qw = p[3];
  float wx = v[3], wy = v[4], wz = v[5];
  float h = 0.5f * dt;
  float ri = (wx * qw + wy * qk) - wz * qj;
  float rj = (wy * qw + wz * qi) - wx * qk;
  float rk = (wz * qw + wx * qj) - wy * qi;
  float rw = -((wx * qi + wy * qj) + wz * qk);
  qi = qi + ri * h;
  qj = qj + rj * h;
  qk = qk + rk * h;
  qw = qw + rw * h;
  float l = sqrtf(((qi * qi + qj * qj) + qk * qk) + qw * qw);
  p[0] = qi / l;
  p[1] = qj / l;
  p[2] = qk / l;
  p[3] = qw / l;
  p[4] = p[4] + v[0] * dt;
  p[5] = p[5] + v[1] * dt;
  p[6] = p[6] + v[2] * dt;
}

__device__ __forceinline__ unsigned long long pair_key(const uint32_t* pairs, uint64_t i) {
  return ((unsigned long long)pairs[2 * i] << 32) | pairs[2 * i + 1];
}
__device__ __forceinline__ uint64_t slot_of(unsigned long long key, uint64_t mask) {
  return (uint64_t)((key * 0x9E3779B97F4A7C15ull) >> 17) & mask;
}

// Previous-frame records follow their pair; new pairs start empty. Open addressing, linear probing,
// at most table_size probes.
__global__ void k_carry_records(const uint32_t* __restrict__ pairs, const unsigned long long* __restrict__ count, uint64_t cap,
                                const unsigned long long* __restrict__ old_keys, const uint32_t* __restrict__ old_vals, uint64_t tsize,
                                const uint32_t* __restrict__ old_recs, uint32_t* __restrict__ recs, uint32_t* __restrict__ err) {
  uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  unsigned long long c = *count;
  if (i == 0 && c > cap) atomicOr(err, ERR_CAPACITY);
  if (i >= cap || i >= c) return;
  unsigned long long key = pair_key(pairs, i);
  uint64_t mask = tsize - 1, s = slot_of(key, mask);
  int64_t found = -1;
  for (uint64_t probe = 0; probe < tsize; ++probe) {
    unsigned long long k = old_keys[s];
    if (k == key) { found = old_vals[s]; break; }
    if (k == EMPTY_KEY) break;
    s = (s + 1) & mask;
  }
  uint32_t* dst = recs + (size_t)i * REC_WORDS;
  if (found < 0) {
#pragma unroll
    for (int w = 0; w < 8; ++w) dst[w] = 0u;
    return;
  }
  const uint32_t* src = old_recs + (size_t)found * REC_WORDS;
  uint32_t np = src[0] > (uint32_t)PARRYGPU_MANIFOLD_MAX_POINTS ? (uint32_t)PARRYGPU_MANIFOLD_MAX_POINTS : src[0];
  uint32_t words = 8 + 10 * np;
  for (uint32_t w = 0; w < words; ++w) dst[w] = src[w];
}

__global__ void k_table_insert(const uint32_t* __restrict__ pairs, const unsigned long long* __restrict__ count, uint64_t cap,
                               unsigned long long* __restrict__ keys, uint32_t* __restrict__ vals, uint64_t tsize,
                               uint32_t* __restrict__ err) {
  uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  unsigned long long c = *count;
  if (i >= cap || i >= c) return;
  unsigned long long key = pair_key(pairs, i);
  uint64_t mask = tsize - 1, s = slot_of(key, mask);
  for (uint64_t probe = 0; probe < tsize; ++probe) {
    unsigned long long prev = atomicCAS(&keys[s], EMPTY_KEY, key);
    if (prev == EMPTY_KEY || prev == key) { vals[s] = (uint32_t)i; return; }
    s = (s + 1) & mask;
  }
  atomicOr(err, ERR_CAPACITY);
}

__global__ void k_gather_rays(const float* __restrict__ src, const uint32_t* __restrict__ order, uint64_t n, float* __restrict__ dst) {
  uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (k >= n) return;
  const float* a = src + 6 * (size_t)order[k];
  float* b = dst + 6 * k;
#pragma unroll
  for (int j = 0; j < 6; ++j) b[j] = a[j];
}

}  // namespace

static ShapeArrays scene_shapes(const parrygpu_scene* sc) {
  ShapeArrays sh{sc->types.as<uint32_t>(), sc->params.as<float4>(), sc->poses.as<float>(), sc->pool.as<float>(), sc->n, sc->n_vertices,
                 PolyArrays{}};
  if (sc->has_poly) {
    PolyArrays& pa = sh.poly;
    pa.hulls = sc->poly[0].as<uint32_t>();
    pa.face_normals = sc->poly[1].as<float>();
    pa.face_ranges = sc->poly[2].as<uint32_t>();
    pa.face_vertices = sc->poly[3].as<uint32_t>();
    pa.face_edges = sc->poly[4].as<uint32_t>();
    pa.vertex_ranges = sc->poly[5].as<uint32_t>();
    pa.vertex_faces = sc->poly[6].as<uint32_t>();
    pa.vertex_edges = sc->poly[7].as<uint32_t>();
    pa.edge_dirs = sc->poly[8].as<float>();
    pa.n_hulls = sc->poly_counts.n_hulls;
    pa.n_faces = sc->poly_counts.n_faces;
    pa.n_face_entries = sc->poly_counts.n_face_entries;
    pa.n_vertex_entries = sc->poly_counts.n_vertex_entries;
    pa.n_edges = sc->poly_counts.n_edges;
  }
  return sh;
}

// One frame: integrate, AABBs, refit, pairs into the other buffer, carry the records, manifolds, rays.
// With kernel timing on (and outside graph capture) each stage is bracketed as "scene_<stage>".
// The context stream waits for an asynchronous read's copies (before a kernel that overwrites what
// they read).
static parrygpu_status order_after_read(parrygpu_ctx* ctx, parrygpu_scene* sc) {
  if (sc->read_order) {
    PG_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, sc->read_done, 0));
    sc->read_order = false;
  }
  return PARRYGPU_OK;
}

static parrygpu_status scene_frame(parrygpu_ctx* ctx, parrygpu_scene* sc, float dt) {
  int old = sc->cur, nw = 1 - sc->cur;
  cudaStream_t st = ctx->stream;
  parrygpu_status s;
  {
    KernelTimer kt(ctx, "scene_integrate");
    k_integrate<<<div_up(sc->n, SC_THREADS), SC_THREADS, 0, st>>>(sc->poses.as<float>(), sc->vel.as<float>(), sc->n, dt);
    kt.stop();
    PG_LAUNCHED(ctx);
  }
  ShapeArrays sh = scene_shapes(sc);
  {
    KernelTimer kt(ctx, "scene_aabbs");
    if ((s = launch_shape_aabbs(ctx, sh, sc->n, 0.5f * sc->prediction, sc->aabbs.as<float>())) != PARRYGPU_OK) return s;
    kt.stop();
  }
  {
    KernelTimer kt(ctx, "scene_refit");
    if ((s = lbvh_refit(ctx, &sc->bvh, sc->aabbs.as<float>())) != PARRYGPU_OK) return s;
    kt.stop();
  }
  unsigned long long* cnt = sc->counts.as<unsigned long long>();
  {
    // the pairs and records of buffer nw are an asynchronous read's source two frames after it
    if (nw == sc->read_cur && (s = order_after_read(ctx, sc)) != PARRYGPU_OK) return s;
    KernelTimer kt(ctx, "scene_pairs");
    PG_CUDA(ctx, cudaMemsetAsync(cnt + nw, 0, 8, st));
    if ((s = launch_self_pairs(ctx, &sc->bvh, sc->pairs[nw].as<uint32_t>(), sc->cap, cnt + nw)) != PARRYGPU_OK) return s;
    kt.stop();
  }
  {
    KernelTimer kt(ctx, "scene_carry");
    k_carry_records<<<div_up(sc->cap, SC_THREADS), SC_THREADS, 0, st>>>(
        sc->pairs[nw].as<uint32_t>(), cnt + nw, sc->cap, sc->keys[old].as<unsigned long long>(), sc->vals[old].as<uint32_t>(),
        sc->table_size, sc->recs[old].as<uint32_t>(), sc->recs[nw].as<uint32_t>(), ctx->d_err);
    PG_LAUNCHED(ctx);
    PG_CUDA(ctx, cudaMemsetAsync(sc->keys[nw].ptr, 0xff, sc->table_size * 8, st));
    k_table_insert<<<div_up(sc->cap, SC_THREADS), SC_THREADS, 0, st>>>(sc->pairs[nw].as<uint32_t>(), cnt + nw, sc->cap,
                                                                      sc->keys[nw].as<unsigned long long>(), sc->vals[nw].as<uint32_t>(),
                                                                      sc->table_size, ctx->d_err);
    PG_LAUNCHED(ctx);
    kt.stop();
  }
  {
    KernelTimer kt(ctx, "scene_manifolds");
    LearnedSeed seed;
    if (sc->seeded) {
      seed.desc = sc->seed_desc.as<float>();
      seed.wb = sc->seed_wb.ptr;
      seed.wf = sc->seed_wf.as<float>();
      seed.feat = sc->seed_feat.as<float>();
      seed.list = sc->seed_list.as<uint32_t>();
      seed.dirs = sc->seed_dirs.as<float>();
    }
    if ((s = launch_manifolds(ctx, sh, sc->pairs[nw].as<uint32_t>(), sc->cap, cnt + nw, sc->prediction, sc->recs[nw].as<uint32_t>(),
                              sc->mf, nullptr, sc->seeded ? &seed : nullptr)) != PARRYGPU_OK)
      return s;
    kt.stop();
  }
  if (sc->n_rays) {
    if ((s = order_after_read(ctx, sc)) != PARRYGPU_OK) return s;  // the ray results are a read's source
    KernelTimer kt(ctx, "scene_rays");
    if ((s = launch_shape_rays(ctx, &sc->bvh, sc->types.as<uint32_t>(), sc->params.as<float>(), sc->poses.as<float>(), sc->pool.as<float>(),
                               sc->hull_box.as<float>(), sc->rays.as<float>(), sc->ray_order.as<uint32_t>(), (uint32_t)sc->n_rays, sc->max_toi,
                               sc->ray_part.as<uint32_t>(), sc->ray_toi.as<float>(), sc->ray_nrm.as<float>(), sc->ray_wave,
                               sc->ray_grid.cells ? &sc->ray_grid : nullptr, sc->aabbs.as<float>())) != PARRYGPU_OK)
      return s;
    kt.stop();
  }
  sc->cur = nw;
  sc->frame++;
  return PARRYGPU_OK;
}

static void drop_graph(parrygpu_scene* sc) {
  if (sc->exec) cudaGraphExecDestroy(sc->exec);
  sc->exec = nullptr;
}

// Captures two frames (cur -> other -> cur) into a graph; frame and launch counters are restored
// since nothing ran.
static parrygpu_status capture_two_frames(parrygpu_ctx* ctx, parrygpu_scene* sc, float dt) {
  PG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));  // no replay of the old graph in flight
  parrygpu_status so = order_after_read(ctx, sc);  // no wait on a read's event inside the graph
  if (so != PARRYGPU_OK) return so;
  drop_graph(sc);
  int cur0 = sc->cur;
  uint64_t frame0 = sc->frame, launches0 = ctx->launches;
  bool timing0 = ctx->timing;
  ctx->timing = false;  // no event records inside the graph
  PG_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  parrygpu_status s = scene_frame(ctx, sc, dt);
  if (s == PARRYGPU_OK) s = scene_frame(ctx, sc, dt);
  cudaGraph_t graph = nullptr;
  cudaError_t e = cudaStreamEndCapture(ctx->stream, &graph);
  ctx->timing = timing0;
  sc->cur = cur0;
  sc->frame = frame0;
  sc->graph_launches = ctx->launches - launches0;
  ctx->launches = launches0;
  if (s != PARRYGPU_OK) {
    if (graph) cudaGraphDestroy(graph);
    return s;
  }
  if (e != cudaSuccess) return check_cuda(ctx, e, "cudaStreamEndCapture");
  e = cudaGraphInstantiate(&sc->exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) {
    sc->exec = nullptr;
    return check_cuda(ctx, e, "cudaGraphInstantiate");
  }
  sc->graph_dt = dt;
  sc->graph_cur = cur0;
  return PARRYGPU_OK;
}

static parrygpu_status copy_in(parrygpu_ctx* ctx, DevBuf& dst, const void* src, size_t bytes) {
  PG_CUDA(ctx, dst.reserve(bytes ? bytes : 16));
  if (bytes) {
    if (!src) return set_error(ctx, PARRYGPU_INVALID_ARG, "null scene input");
    PG_CUDA(ctx, cudaMemcpyAsync(dst.ptr, src, bytes, cudaMemcpyDefault, ctx->stream));
  }
  return PARRYGPU_OK;
}

extern "C" {

parrygpu_status parrygpu_scene_create(parrygpu_ctx* ctx, const parrygpu_shapes* shapes, const float* velocities, float prediction,
                                      uint64_t pair_capacity, parrygpu_scene** out) {
  if (!ctx || !shapes || !out) return PARRYGPU_INVALID_ARG;
  *out = nullptr;
  if (shapes->n == 0 || shapes->n > 0x7fffffffull) return set_error(ctx, PARRYGPU_INVALID_ARG, "a scene needs 1 .. 2^31 shapes");
  if (!velocities) return set_error(ctx, PARRYGPU_INVALID_ARG, "velocities are required");
  if (pair_capacity == 0 || pair_capacity > (1ull << 31)) return set_error(ctx, PARRYGPU_INVALID_ARG, "pair capacity must be in 1 .. 2^31");
  PG_CUDA(ctx, cudaSetDevice(ctx->device));
  auto* sc = new parrygpu_scene();
  auto fail = [&](parrygpu_status s) {
    parrygpu_scene_destroy(sc);
    return s;
  };
  sc->n = shapes->n;
  sc->n_vertices = shapes->n_vertices;
  sc->cap = pair_capacity;
  sc->prediction = prediction;
  uint64_t ts = 1024;
  while (ts < 2 * pair_capacity) ts <<= 1;
  sc->table_size = ts;
  parrygpu_status s;
  if ((s = copy_in(ctx, sc->types, shapes->types, sc->n * 4)) != PARRYGPU_OK) return fail(s);
  if ((s = copy_in(ctx, sc->params, shapes->params, sc->n * 16)) != PARRYGPU_OK) return fail(s);
  if ((s = copy_in(ctx, sc->poses, shapes->poses, sc->n * 28)) != PARRYGPU_OK) return fail(s);
  if ((s = copy_in(ctx, sc->vel, velocities, sc->n * 24)) != PARRYGPU_OK) return fail(s);
  if ((s = copy_in(ctx, sc->pool, shapes->vertices, sc->n_vertices * 12)) != PARRYGPU_OK) return fail(s);
  if (const parrygpu_polyhedra* ph = shapes->polyhedra) {
    sc->has_poly = true;
    sc->poly_counts = *ph;
    const void* src[9] = {ph->hulls, ph->face_normals, ph->face_ranges, ph->face_vertices, ph->face_edges, ph->vertex_ranges,
                          ph->vertex_faces, ph->vertex_edges, ph->edge_dirs};
    size_t bytes[9] = {(size_t)ph->n_hulls * 32, (size_t)ph->n_faces * 12, (size_t)ph->n_faces * 8, (size_t)ph->n_face_entries * 4,
                       (size_t)ph->n_face_entries * 4, (size_t)sc->n_vertices * 8, (size_t)ph->n_vertex_entries * 4,
                       (size_t)ph->n_vertex_entries * 4, (size_t)ph->n_edges * 12};
    for (int k = 0; k < 9; ++k)
      if ((s = copy_in(ctx, sc->poly[k], src[k], bytes[k])) != PARRYGPU_OK) return fail(s);
  }
  PG_CUDA(ctx, sc->aabbs.reserve(sc->n * 24));
  PG_CUDA(ctx, sc->hull_box.reserve(sc->n * 32));
  if ((s = launch_hull_boxes(ctx, sc->types.as<uint32_t>(), sc->params.as<float>(), sc->pool.as<float>(), (uint32_t)sc->n, sc->n_vertices,
                             sc->hull_box.as<float>())) != PARRYGPU_OK)
    return fail(s);
  for (int b = 0; b < 2; ++b) {
    PG_CUDA(ctx, sc->pairs[b].reserve(pair_capacity * 8));
    PG_CUDA(ctx, sc->recs[b].reserve(pair_capacity * (size_t)REC_WORDS * 4));
    PG_CUDA(ctx, sc->keys[b].reserve(ts * 8));
    PG_CUDA(ctx, sc->vals[b].reserve(ts * 4));
    PG_CUDA(ctx, cudaMemsetAsync(sc->keys[b].ptr, 0xff, ts * 8, ctx->stream));
  }
  PG_CUDA(ctx, sc->counts.reserve(16));
  PG_CUDA(ctx, cudaMemsetAsync(sc->counts.ptr, 0, 16, ctx->stream));
  if ((s = manifolds_reserve(ctx, pair_capacity, sc->mf)) != PARRYGPU_OK) return fail(s);
  ShapeArrays sh = scene_shapes(sc);
  if ((s = launch_shape_aabbs(ctx, sh, sc->n, 0.5f * prediction, sc->aabbs.as<float>())) != PARRYGPU_OK) return fail(s);
  if ((s = lbvh_build(ctx, &sc->bvh, sc->aabbs.as<float>(), (uint32_t)sc->n, false)) != PARRYGPU_OK) return fail(s);
  if ((s = parrygpu_sync(ctx)) != PARRYGPU_OK) return fail(s);
  *out = sc;
  return PARRYGPU_OK;
}

void parrygpu_scene_destroy(parrygpu_scene* sc) {
  if (!sc) return;
  cudaDeviceSynchronize();  // frames and reads in flight still use the scene's buffers
  drop_graph(sc);
  sc->pose_snap.release();
  if (sc->read_start) cudaEventDestroy(sc->read_start);
  if (sc->read_done) cudaEventDestroy(sc->read_done);
  for (DevBuf* d : {&sc->types, &sc->params, &sc->poses, &sc->vel, &sc->pool, &sc->aabbs, &sc->hull_box, &sc->counts, &sc->mf.queue, &sc->mf.counters,
                    &sc->mf.epa_ws, &sc->mf.bins, &sc->rays, &sc->ray_order, &sc->ray_part,
                    &sc->ray_toi, &sc->ray_nrm, &sc->bvh.wide, &sc->bvh.leaf_parent, &sc->bvh.node_parent, &sc->bvh.leaf_index,
                    &sc->bvh.flags, &sc->bvh.root_aabb, &sc->bvh.info})
    d->release();
  for (int k = 0; k < 9; ++k) sc->poly[k].release();
  for (DevBuf* d : {&sc->ray_wave.cands, &sc->ray_wave.counter, &sc->ray_wave.keys, &sc->ray_wave.ovf}) d->release();
  for (DevBuf* d : {&sc->seed_desc, &sc->seed_wb, &sc->seed_wf, &sc->seed_feat, &sc->seed_list, &sc->seed_dirs}) d->release();
  for (DevBuf* d : {&sc->ray_grid.dev, &sc->ray_grid.starts, &sc->ray_grid.cursor, &sc->ray_grid.entries, &sc->ray_grid.sums}) d->release();
  for (int b = 0; b < 2; ++b) {
    sc->pairs[b].release();
    sc->recs[b].release();
    sc->keys[b].release();
    sc->vals[b].release();
  }
  delete sc;
}

parrygpu_status parrygpu_scene_set_rays(parrygpu_ctx* ctx, parrygpu_scene* sc, const float* rays, uint64_t n_rays, float max_toi) {
  if (!ctx || !sc) return PARRYGPU_INVALID_ARG;
  if (n_rays > 0xffffffffull) return set_error(ctx, PARRYGPU_INVALID_ARG, "too many rays");
  PG_CUDA(ctx, cudaSetDevice(ctx->device));
  parrygpu_status sw = parrygpu_scene_read_wait(ctx, sc);  // the ray buffers may be reallocated
  if (sw != PARRYGPU_OK) return sw;
  PG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  drop_graph(sc);  // the captured frame bakes in the ray buffers
  parrygpu_status s;
  // rays in input order into scratch, then permuted into the Morton order of their origins (coherent
  // traversal); ray_order maps a stored slot back to the input slot for the results
  uint32_t n = (uint32_t)n_rays;
  PG_CUDA(ctx, sc->ray_order.reserve(n_rays * 4 + 16));
  PG_CUDA(ctx, sc->rays.reserve(n_rays * 24 + 16));
  if (n > 0) {
    DevBuf tmp;
    if ((s = copy_in(ctx, tmp, rays, n_rays * 24)) != PARRYGPU_OK) { tmp.release(); return s; }
    if ((s = radix_sort_reserve(ctx, n)) != PARRYGPU_OK) { tmp.release(); return s; }
    PG_CUDA(ctx, ctx->misc.reserve(64));
    uint32_t* bounds = ctx->misc.as<uint32_t>() + 8;
    // scene_ray_order 1 / 2 / 3 -> ray key 0 (origin) / 1 (octant, origin) / 3 (octant and dominant axis, origin)
    const uint32_t order_mode = ctx->cfg.scene_ray_order ? ctx->cfg.scene_ray_order : DEFAULT_SCENE_RAY_ORDER;
    const uint32_t key_mode = order_mode == 1 ? 0u : (order_mode == 2 ? 1u : 3u);
    if ((s = launch_ray_keys(ctx, tmp.as<float>(), n, bounds, ctx->sort_k[0].as<uint32_t>(), ctx->sort_v[0].as<uint32_t>(), key_mode)) !=
        PARRYGPU_OK) {
      tmp.release();
      return s;
    }
    int rb;
    if ((s = radix_sort_pairs(ctx, n, 30, &rb)) != PARRYGPU_OK) { tmp.release(); return s; }
    PG_CUDA(ctx, cudaMemcpyAsync(sc->ray_order.ptr, ctx->sort_v[rb].ptr, n_rays * 4, cudaMemcpyDeviceToDevice, ctx->stream));
    k_gather_rays<<<div_up(n_rays, SC_THREADS), SC_THREADS, 0, ctx->stream>>>(tmp.as<float>(), sc->ray_order.as<uint32_t>(), n_rays,
                                                                             sc->rays.as<float>());
    PG_LAUNCHED(ctx);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    tmp.release();
    if (e != cudaSuccess) return check_cuda(ctx, e, "scene ray ordering");
  }
  if ((s = shape_rays_reserve(ctx, sc->ray_wave, n)) != PARRYGPU_OK) return s;
  if (ctx->cfg.scene_ray_grid != 2 && n > 0) {
    // the grid's resolution from the shapes' current bounds (its placement follows them each frame)
    float root[6];
    PG_CUDA(ctx, cudaMemcpyAsync(root, sc->bvh.root_aabb.ptr, sizeof(root), cudaMemcpyDeviceToHost, ctx->stream));
    PG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if ((s = shape_ray_grid_reserve(ctx, sc->ray_grid, sc->n, root)) != PARRYGPU_OK) return s;
  } else {
    sc->ray_grid.cells = 0;
  }
  PG_CUDA(ctx, sc->ray_part.reserve(n_rays * 4 + 16));
  PG_CUDA(ctx, sc->ray_toi.reserve(n_rays * 4 + 16));
  PG_CUDA(ctx, sc->ray_nrm.reserve(n_rays * 12 + 16));
  sc->n_rays = n_rays;
  sc->max_toi = max_toi;
  return PARRYGPU_OK;
}

parrygpu_status parrygpu_scene_set_mlp(parrygpu_ctx* ctx, parrygpu_scene* sc, const parrygpu_mlp* mlp) {
  if (!ctx || !sc) return PARRYGPU_INVALID_ARG;
  PG_CUDA(ctx, cudaSetDevice(ctx->device));
  PG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  drop_graph(sc);  // the captured frame bakes in whether (and with which buffers) pairs are seeded
  sc->seeded = false;
  if (!mlp) return PARRYGPU_OK;
  PG_CUDA(ctx, sc->seed_feat.reserve(sc->cap * PARRYGPU_MLP_IN * 4));
  PG_CUDA(ctx, sc->seed_list.reserve(sc->cap * 4));
  PG_CUDA(ctx, sc->seed_dirs.reserve(sc->cap * 12));
  parrygpu_status s = seed_prepare(ctx, mlp, scene_shapes(sc), sc->seed_desc, sc->seed_wb, sc->seed_wf);
  if (s != PARRYGPU_OK) return s;
  if ((s = parrygpu_sync(ctx)) != PARRYGPU_OK) return s;
  sc->seeded = true;
  return PARRYGPU_OK;
}

parrygpu_status parrygpu_scene_step(parrygpu_ctx* ctx, parrygpu_scene* sc, float dt, uint32_t frames, int use_graph) {
  if (!ctx || !sc) return PARRYGPU_INVALID_ARG;
  PG_CUDA(ctx, cudaSetDevice(ctx->device));
  parrygpu_status s;
  if (use_graph && frames >= 2) {
    if (!sc->exec || sc->graph_dt != dt || sc->graph_cur != sc->cur) {
      if ((s = capture_two_frames(ctx, sc, dt)) != PARRYGPU_OK) return s;
    }
    if ((s = order_after_read(ctx, sc)) != PARRYGPU_OK) return s;  // replays start after a read's copies
    for (uint32_t k = 0; k + 2 <= frames; k += 2) {
      PG_CUDA(ctx, cudaGraphLaunch(sc->exec, ctx->stream));
      ctx->launches += sc->graph_launches;
      sc->frame += 2;
    }
    if (frames % 2) return scene_frame(ctx, sc, dt);
    return PARRYGPU_OK;
  }
  for (uint32_t k = 0; k < frames; ++k)
    if ((s = scene_frame(ctx, sc, dt)) != PARRYGPU_OK) return s;
  return PARRYGPU_OK;
}

parrygpu_status parrygpu_scene_info(parrygpu_ctx* ctx, const parrygpu_scene* sc, uint64_t* frame, uint64_t* n_pairs) {
  if (!ctx || !sc) return PARRYGPU_INVALID_ARG;
  PG_CUDA(ctx, cudaSetDevice(ctx->device));
  unsigned long long c = 0;
  PG_CUDA(ctx, cudaMemcpyAsync(&c, sc->counts.as<unsigned long long>() + sc->cur, 8, cudaMemcpyDeviceToHost, ctx->stream));
  parrygpu_status s = parrygpu_sync(ctx);
  if (frame) *frame = sc->frame;
  if (n_pairs) *n_pairs = c;
  return s;
}

parrygpu_status parrygpu_scene_read(parrygpu_ctx* ctx, const parrygpu_scene* sc, float* poses, uint32_t* pairs, parrygpu_manifold* manifolds,
                                    uint64_t cap, uint32_t* ray_part, float* ray_toi, float* ray_normal) {
  if (!ctx || !sc) return PARRYGPU_INVALID_ARG;
  PG_CUDA(ctx, cudaSetDevice(ctx->device));
  if (sc->read_inflight) PG_CUDA(ctx, cudaEventSynchronize(sc->read_done));  // its host buffers may be these
  unsigned long long c = 0;
  PG_CUDA(ctx, cudaMemcpyAsync(&c, sc->counts.as<unsigned long long>() + sc->cur, 8, cudaMemcpyDeviceToHost, ctx->stream));
  PG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  uint64_t np = c < sc->cap ? c : sc->cap;
  if (np > cap) np = cap;
  cudaStream_t st = ctx->stream;
  if (poses) PG_CUDA(ctx, cudaMemcpyAsync(poses, sc->poses.ptr, sc->n * 28, cudaMemcpyDefault, st));
  if (pairs && np) PG_CUDA(ctx, cudaMemcpyAsync(pairs, sc->pairs[sc->cur].ptr, np * 8, cudaMemcpyDefault, st));
  if (manifolds && np) PG_CUDA(ctx, cudaMemcpyAsync(manifolds, sc->recs[sc->cur].ptr, np * sizeof(parrygpu_manifold), cudaMemcpyDefault, st));
  if (sc->n_rays) {
    if (ray_part) PG_CUDA(ctx, cudaMemcpyAsync(ray_part, sc->ray_part.ptr, sc->n_rays * 4, cudaMemcpyDefault, st));
    if (ray_toi) PG_CUDA(ctx, cudaMemcpyAsync(ray_toi, sc->ray_toi.ptr, sc->n_rays * 4, cudaMemcpyDefault, st));
    if (ray_normal) PG_CUDA(ctx, cudaMemcpyAsync(ray_normal, sc->ray_nrm.ptr, sc->n_rays * 12, cudaMemcpyDefault, st));
  }
  return parrygpu_sync(ctx);
}

parrygpu_status parrygpu_scene_read_async(parrygpu_ctx* ctx, parrygpu_scene* sc, float* poses, uint32_t* pairs, parrygpu_manifold* manifolds,
                                          uint64_t cap, uint32_t* ray_part, float* ray_toi, float* ray_normal, uint64_t* n_pairs) {
  if (!ctx || !sc) return PARRYGPU_INVALID_ARG;
  PG_CUDA(ctx, cudaSetDevice(ctx->device));
  parrygpu_status s = parrygpu_scene_read_wait(ctx, sc);  // one read in flight at a time
  if (s != PARRYGPU_OK) return s;
  if (!ctx->down_stream) PG_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->down_stream, cudaStreamNonBlocking));
  if (!sc->read_start) {
    PG_CUDA(ctx, cudaEventCreateWithFlags(&sc->read_start, cudaEventDisableTiming));
    PG_CUDA(ctx, cudaEventCreateWithFlags(&sc->read_done, cudaEventDisableTiming));
  }
  // the frame's pair count (this waits for the frame)
  unsigned long long c = 0;
  PG_CUDA(ctx, cudaMemcpyAsync(&c, sc->counts.as<unsigned long long>() + sc->cur, 8, cudaMemcpyDeviceToHost, ctx->stream));
  if ((s = parrygpu_sync(ctx)) != PARRYGPU_OK) return s;
  uint64_t np = c < sc->cap ? c : sc->cap;
  if (np > cap) np = cap;
  if (n_pairs) *n_pairs = pairs || manifolds ? np : 0;
  cudaStream_t st = ctx->stream, dn = ctx->down_stream;
  // the poses change at the next frame's first kernel: copied from a snapshot
  if (poses) {
    PG_CUDA(ctx, sc->pose_snap.reserve(sc->n * 28));
    PG_CUDA(ctx, cudaMemcpyAsync(sc->pose_snap.ptr, sc->poses.ptr, sc->n * 28, cudaMemcpyDeviceToDevice, st));
  }
  PG_CUDA(ctx, cudaEventRecord(sc->read_start, st));
  PG_CUDA(ctx, cudaStreamWaitEvent(dn, sc->read_start, 0));
  if (poses) PG_CUDA(ctx, cudaMemcpyAsync(poses, sc->pose_snap.ptr, sc->n * 28, cudaMemcpyDefault, dn));
  if (pairs && np) PG_CUDA(ctx, cudaMemcpyAsync(pairs, sc->pairs[sc->cur].ptr, np * 8, cudaMemcpyDefault, dn));
  if (manifolds && np) PG_CUDA(ctx, cudaMemcpyAsync(manifolds, sc->recs[sc->cur].ptr, np * sizeof(parrygpu_manifold), cudaMemcpyDefault, dn));
  if (sc->n_rays) {
    if (ray_part) PG_CUDA(ctx, cudaMemcpyAsync(ray_part, sc->ray_part.ptr, sc->n_rays * 4, cudaMemcpyDefault, dn));
    if (ray_toi) PG_CUDA(ctx, cudaMemcpyAsync(ray_toi, sc->ray_toi.ptr, sc->n_rays * 4, cudaMemcpyDefault, dn));
    if (ray_normal) PG_CUDA(ctx, cudaMemcpyAsync(ray_normal, sc->ray_nrm.ptr, sc->n_rays * 12, cudaMemcpyDefault, dn));
  }
  PG_CUDA(ctx, cudaEventRecord(sc->read_done, dn));
  sc->read_cur = sc->cur;
  sc->read_order = true;
  sc->read_inflight = true;
  return PARRYGPU_OK;
}

parrygpu_status parrygpu_scene_read_wait(parrygpu_ctx* ctx, parrygpu_scene* sc) {
  if (!ctx || !sc) return PARRYGPU_INVALID_ARG;
  if (!sc->read_inflight) return PARRYGPU_OK;
  PG_CUDA(ctx, cudaSetDevice(ctx->device));
  sc->read_inflight = false;
  PG_CUDA(ctx, cudaEventSynchronize(sc->read_done));
  return PARRYGPU_OK;
}

parrygpu_status parrygpu_scene_stats(parrygpu_ctx* ctx, const parrygpu_scene* sc, parrygpu_gjk_stats* stats, uint64_t* seeded_pairs) {
  if (!ctx || !sc) return PARRYGPU_INVALID_ARG;
  PG_CUDA(ctx, cudaSetDevice(ctx->device));
  // the manifold counters block: [1..3] GJK iterations, EPA iterations, EPA calls; [15] seeded pairs
  unsigned long long h[16] = {};
  if (sc->frame > 0) {
    PG_CUDA(ctx, cudaMemcpyAsync(h, sc->mf.counters.ptr, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
  }
  parrygpu_status s = parrygpu_sync(ctx);
  if (stats) {
    std::memset(stats, 0, sizeof(*stats));
    stats->gjk_iterations = h[1];
    stats->epa_iterations = h[2];
    stats->epa_calls = h[3];
  }
  if (seeded_pairs) *seeded_pairs = sc->seeded ? h[15] : 0;
  return s;
}

}  // extern "C"
