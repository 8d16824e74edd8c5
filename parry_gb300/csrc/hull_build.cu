// ConvexPolyhedron::from_convex_hull for many clouds on the GPU (src/shape/convex_polyhedron.rs:
// 264-268 and :390-639, paths relative to the parry repository): one thread per cloud runs the
// shared hull_core.hpp algorithm (the host builder's, so both give the same bytes).
//
//   1. clouds ordered by point count (one radix pass over a 16-bit key) so a warp walks clouds of
//      similar size;
//   2. build pass: every cloud is built once into a staging slot sized from its point count, its
//      output sizes kept;
//   3. one exclusive scan per output array gives every cloud its offsets;
//   4. copy pass (a warp per cloud): staged outputs to their offsets, in the parrygpu_polyhedra
//      layout, into device arrays the handle owns (usable directly as parrygpu_polyhedra).
// When the staging slots would exceed a fixed budget (clouds of hundreds of points by the
// million), steps 2 and 4 become a sizes pass and an emit pass that builds every cloud again.
// The hull workspaces are per thread, interleaved across threads (element i of thread t at
// i * threads + t), and reused by each cloud a thread takes.
#include "internal.hpp"
#include "hull_core.hpp"

#include <algorithm>
#include <type_traits>

using namespace hullcore;

namespace {

constexpr int HB_THREADS = 128;
constexpr size_t HB_WS_BUDGET = size_t(16) << 30;    // bytes of per-thread workspaces at once
constexpr size_t HB_STAGE_BUDGET = size_t(12) << 30;  // staging above this: build twice instead
constexpr int NSIZES = 6;  // per-cloud output sizes: points, faces, face entries, vertex entries, edges, triangles

// Thread t's spans over the interleaved workspace (arrays laid out one after another, each holding
// capacity x threads elements).
struct WsLayout {
  HullCaps caps;
  uint32_t threads;
  char* base;
  __device__ HullWs at(uint32_t t) const {
    const size_t T = threads;
    char* p = base;
    auto take = [&](auto* tag, size_t cap) {
      using E = std::remove_pointer_t<decltype(tag)>;
      E* a = reinterpret_cast<E*>(p);
      p += ((cap * T * sizeof(E)) + 255) & ~size_t(255);
      return Span<E>{a + t, T};
    };
    const size_t n = caps.n;
    HullWs ws;
    ws.pts = take((D3*)nullptr, n);
    ws.faces = take((HFace*)nullptr, caps.faces);
    ws.visible = take((uint32_t*)nullptr, caps.faces);
    ws.horizon = take((uint32_t*)nullptr, HORIZON_WORDS * (size_t)caps.horizon);
    ws.tris = take((uint32_t*)nullptr, 3 * (size_t)caps.tris);
    ws.used = take((uint32_t*)nullptr, n);
    ws.remap = take((uint32_t*)nullptr, n);
    ws.fpts = take((F3*)nullptr, n);
    ws.edges = take((HEdge*)nullptr, caps.edges);
    ws.hkeys = take((uint64_t*)nullptr, caps.hash);
    ws.hvals = take((uint32_t*)nullptr, caps.hash);
    ws.htris = take((HTri*)nullptr, caps.tris);
    ws.frecs = take((HFaceRec*)nullptr, caps.tris);
    ws.face_edges = take((uint32_t*)nullptr, caps.entries);
    ws.face_vertices = take((uint32_t*)nullptr, caps.entries);
    ws.vertex_first = take((uint32_t*)nullptr, n);
    ws.vertex_count = take((uint32_t*)nullptr, n);
    ws.vertex_faces = take((uint32_t*)nullptr, caps.entries);
    ws.vertex_edges = take((uint32_t*)nullptr, caps.entries);
    return ws;
  }
};

size_t ws_total(const HullCaps& c, uint32_t threads) {
  const size_t T = threads, n = c.n;
  auto a = [&](size_t bytes_each, size_t cap) { return ((cap * T * bytes_each) + 255) & ~size_t(255); };
  return a(sizeof(D3), n) + a(sizeof(HFace), c.faces) + a(4, c.faces) + a(4, HORIZON_WORDS * (size_t)c.horizon) + a(4, 3 * (size_t)c.tris) +
         a(4, n) * 2 + a(sizeof(F3), n) + a(sizeof(HEdge), c.edges) + a(8, c.hash) + a(4, c.hash) + a(sizeof(HTri), c.tris) +
         a(sizeof(HFaceRec), c.tris) + a(4, c.entries) * 2 + a(4, n) * 2 + a(4, c.entries) * 2;
}

__global__ void k_hb_keys(uint64_t n_hulls, const uint32_t* __restrict__ count, uint32_t cap_points, uint32_t* __restrict__ keys,
                          uint32_t* __restrict__ vals, uint32_t* __restrict__ err) {
  const uint64_t h = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (h >= n_hulls) return;
  const uint32_t c = count[h];
  if (c > cap_points) atomicOr(err, ERR_BAD_INDEX);
  keys[h] = c < 0xffffu ? c : 0xffffu;
  vals[h] = (uint32_t)h;
}

__global__ void k_hb_max(uint64_t n_hulls, const uint32_t* __restrict__ count, uint32_t* __restrict__ out) {
  const uint64_t h = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (h >= n_hulls) return;
  atomicMax(out, count[h]);
}

// Sizes pass: per cloud, npts / faces / face entries / vertex entries / edges / triangles (SoA, 6
// arrays).
__global__ void __launch_bounds__(HB_THREADS) k_hb_sizes(WsLayout lay, uint64_t n_hulls, const uint32_t* __restrict__ order,
                                                         const float* __restrict__ pts, uint64_t n_points, const uint32_t* __restrict__ first,
                                                         const uint32_t* __restrict__ count, uint32_t* __restrict__ sizes,
                                                         uint32_t* __restrict__ err) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= lay.threads) return;
  HullWs ws = lay.at(t);
  for (uint64_t k = t; k < n_hulls; k += lay.threads) {
    const uint32_t h = order[k];
    const uint32_t n = count[h];
    HullOut r;
    if (n <= lay.caps.n && (uint64_t)first[h] + n <= n_points) r = build_one(pts + 3 * (size_t)first[h], n, lay.caps, ws);
    else atomicOr(err, ERR_BAD_INDEX);
    sizes[0 * n_hulls + h] = r.npts;
    sizes[1 * n_hulls + h] = r.ok ? r.nfaces : 0u;
    sizes[2 * n_hulls + h] = r.ok ? r.nfentries : 0u;
    sizes[3 * n_hulls + h] = r.ok ? r.nventries : 0u;
    sizes[4 * n_hulls + h] = r.ok ? r.nedges : 0u;
    sizes[5 * n_hulls + h] = r.ntris;
  }
}

// Emit pass: the same build, written at the scanned offsets (triangle ranges too).
__global__ void __launch_bounds__(HB_THREADS) k_hb_emit(WsLayout lay, uint64_t n_hulls, const uint32_t* __restrict__ order,
                                                        const float* __restrict__ pts, uint64_t n_points, const uint32_t* __restrict__ first,
                                                        const uint32_t* __restrict__ count, const uint32_t* __restrict__ offsets,
                                                        size_t off_stride, PolyOut o, uint32_t* __restrict__ tri_ranges) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= lay.threads) return;
  HullWs ws = lay.at(t);
  for (uint64_t k = t; k < n_hulls; k += lay.threads) {
    const uint32_t h = order[k];
    const uint32_t n = count[h];
    HullOut r;
    if (n <= lay.caps.n && (uint64_t)first[h] + n <= n_points) r = build_one(pts + 3 * (size_t)first[h], n, lay.caps, ws);
    emit(ws, r, h, offsets[0 * off_stride + h], offsets[1 * off_stride + h], offsets[2 * off_stride + h], offsets[3 * off_stride + h],
         offsets[4 * off_stride + h], o, offsets[5 * off_stride + h]);
    tri_ranges[2 * (size_t)h] = offsets[5 * off_stride + h];
    tri_ranges[2 * (size_t)h + 1] = r.ntris;
  }
}

// ---- one build per cloud, results staged ----
// A cloud of n points fits its outputs in a staging slot laid out from HullCaps::of(n): points
// (3n f32), vertex ranges (2n), face normals (3 per triangle bound), face ranges (2 per triangle
// bound), face vertices, face edges, vertex faces, vertex edges (an entry bound each), edge
// directions (3 per edge bound), triangles (3 per triangle bound). Slots are whole 256-byte blocks.
struct StageLayout {
  uint32_t n, tris, entries, edges;
  __host__ __device__ static StageLayout of(uint32_t count) {
    const HullCaps c = HullCaps::of(count < 4 ? 4 : count);
    return StageLayout{count, c.tris, c.entries, c.edges};
  }
  __host__ __device__ size_t words() const { return 3ull * n + 2ull * n + 8ull * tris + 4ull * entries + 3ull * edges; }
  __host__ __device__ uint32_t blocks() const { return (uint32_t)((words() * 4 + 255) / 256); }
  __device__ PolyOut view(uint32_t* base) const {
    uint32_t* p = base;
    PolyOut o;
    o.points = reinterpret_cast<float*>(p); p += 3 * (size_t)n;
    o.vertex_ranges = p; p += 2 * (size_t)n;
    o.face_normals = reinterpret_cast<float*>(p); p += 3 * (size_t)tris;
    o.face_ranges = p; p += 2 * (size_t)tris;
    o.face_vertices = p; p += entries;
    o.face_edges = p; p += entries;
    o.vertex_faces = p; p += entries;
    o.vertex_edges = p; p += entries;
    o.edge_dirs = reinterpret_cast<float*>(p); p += 3 * (size_t)edges;
    o.triangles = p;
    o.hulls = nullptr;
    return o;
  }
};

__global__ void k_hb_stage_blocks(uint64_t n_hulls, const uint32_t* __restrict__ count, uint32_t* __restrict__ blocks) {
  const uint64_t h = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (h >= n_hulls) return;
  blocks[h] = StageLayout::of(count[h]).blocks();
}

// Build pass: every cloud built once, its output written to its staging slot (hull-relative
// offsets, as the host builder keeps them) and its sizes recorded (SoA, 6 arrays of `stride`).
// 64 registers (8 blocks of 128 per SM): the build is latency-bound, more resident warps beat the
// spills this costs (measured on GB300: 136 vs 160 ms for 1 M clouds of 16-64 points).
__global__ void __launch_bounds__(HB_THREADS, 8) k_hb_build(WsLayout lay, uint64_t n_hulls, const uint32_t* __restrict__ order,
                                                         const float* __restrict__ pts, uint64_t n_points, const uint32_t* __restrict__ first,
                                                         const uint32_t* __restrict__ count, const uint32_t* __restrict__ stage_off,
                                                         uint32_t* __restrict__ stage, uint32_t* __restrict__ sizes, size_t stride,
                                                         uint32_t* __restrict__ err) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= lay.threads) return;
  HullWs ws = lay.at(t);
  for (uint64_t k = t; k < n_hulls; k += lay.threads) {
    const uint32_t h = order[k];
    const uint32_t n = count[h];
    HullOut r;
    if (n <= lay.caps.n && (uint64_t)first[h] + n <= n_points) {
      r = build_one(pts + 3 * (size_t)first[h], n, lay.caps, ws);
      const PolyOut o = StageLayout::of(n).view(stage + (size_t)stage_off[h] * 64);
      emit(ws, r, 0, 0, 0, 0, 0, 0, o);
    } else {
      atomicOr(err, ERR_BAD_INDEX);
    }
    sizes[0 * stride + h] = r.npts;
    sizes[1 * stride + h] = r.ok ? r.nfaces : 0u;
    sizes[2 * stride + h] = r.ok ? r.nfentries : 0u;
    sizes[3 * stride + h] = r.ok ? r.nventries : 0u;
    sizes[4 * stride + h] = r.ok ? r.nedges : 0u;
    sizes[5 * stride + h] = r.ntris;
  }
}

// One warp per cloud: its staged output to the final arrays at the scanned offsets (ranges
// shifted by the cloud's entry offsets), and its hull record.
__global__ void k_hb_copy(uint64_t n_hulls, const uint32_t* __restrict__ count, const uint32_t* __restrict__ stage_off,
                          const uint32_t* __restrict__ stage, const uint32_t* __restrict__ sizes, const uint32_t* __restrict__ offsets,
                          size_t stride, PolyOut o, uint32_t* __restrict__ tri_ranges) {
  const uint64_t h = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint32_t lane = threadIdx.x & 31;
  if (h >= n_hulls) return;
  const StageLayout L = StageLayout::of(count[h]);
  const PolyOut sv = L.view(const_cast<uint32_t*>(stage) + (size_t)stage_off[h] * 64);
  const uint32_t np = sizes[0 * stride + h], nf = sizes[1 * stride + h], nfe = sizes[2 * stride + h], nve = sizes[3 * stride + h],
                 ne = sizes[4 * stride + h], nt = sizes[5 * stride + h];
  const uint64_t vp = offsets[0 * stride + h], fp = offsets[1 * stride + h], fe = offsets[2 * stride + h], ve = offsets[3 * stride + h],
                 ep = offsets[4 * stride + h], tp = offsets[5 * stride + h];
  if (lane == 0) {
    uint32_t* rec = o.hulls + 8 * h;
    const bool ok = ne > 0;  // a hull with topology has at least the 6 edges of a tetrahedron
    rec[0] = (uint32_t)vp; rec[1] = np; rec[2] = (uint32_t)fp; rec[3] = nf; rec[4] = (uint32_t)ep; rec[5] = ne; rec[6] = ok ? 1u : 0u;
    rec[7] = 0;
    tri_ranges[2 * h] = (uint32_t)tp;
    tri_ranges[2 * h + 1] = nt;
  }
  for (uint32_t i = lane; i < 3 * np; i += 32) o.points[3 * vp + i] = sv.points[i];
  for (uint32_t i = lane; i < 2 * np; i += 32) o.vertex_ranges[2 * vp + i] = sv.vertex_ranges[i] + ((i & 1u) ? 0u : (uint32_t)ve);
  for (uint32_t i = lane; i < 3 * nf; i += 32) o.face_normals[3 * fp + i] = sv.face_normals[i];
  for (uint32_t i = lane; i < 2 * nf; i += 32) o.face_ranges[2 * fp + i] = sv.face_ranges[i] + ((i & 1u) ? 0u : (uint32_t)fe);
  for (uint32_t i = lane; i < nfe; i += 32) { o.face_vertices[fe + i] = sv.face_vertices[i]; o.face_edges[fe + i] = sv.face_edges[i]; }
  for (uint32_t i = lane; i < nve; i += 32) { o.vertex_faces[ve + i] = sv.vertex_faces[i]; o.vertex_edges[ve + i] = sv.vertex_edges[i]; }
  for (uint32_t i = lane; i < 3 * ne; i += 32) o.edge_dirs[3 * ep + i] = sv.edge_dirs[i];
  for (uint32_t i = lane; i < 3 * nt; i += 32) o.triangles[3 * tp + i] = sv.triangles[i];
}

}  // namespace

// Device arrays of a built batch, in the parrygpu_polyhedra layout.
struct parrygpu_polyhedra_gpu {
  uint64_t n_hulls = 0;
  uint64_t sizes[5] = {0, 0, 0, 0, 0};  // points, faces, face entries, vertex entries, edges
  uint64_t n_triangles = 0;
  DevBuf points, hulls, face_normals, face_ranges, face_vertices, face_edges, vertex_ranges, vertex_faces, vertex_edges, edge_dirs;
  DevBuf triangles, tri_ranges;  // transformation::convex_hull's triangles per cloud
};

extern "C" {

parrygpu_status parrygpu_polyhedra_build_gpu(parrygpu_ctx* ctx, const float* points, uint64_t n_points, const uint32_t* first,
                                             const uint32_t* count, uint64_t n_hulls, parrygpu_polyhedra_gpu** out) {
  if (!ctx || !out || (n_hulls && (!points || !first || !count))) return PARRYGPU_INVALID_ARG;
  *out = nullptr;
  if (n_hulls >= 0x7fffffffull) return set_error(ctx, PARRYGPU_INVALID_ARG, "too many clouds");
  PG_CUDA(ctx, cudaSetDevice(ctx->device));
  auto* g = new parrygpu_polyhedra_gpu();
  g->n_hulls = n_hulls;
  struct Guard {
    parrygpu_polyhedra_gpu* g;
    DevBuf ws, sizes, keys[2], vals[2], hist, misc, stage, stage_off;
    ~Guard() {
      for (DevBuf* d : {&ws, &sizes, &keys[0], &keys[1], &vals[0], &vals[1], &hist, &misc, &stage, &stage_off}) d->release();
      if (g) parrygpu_polyhedra_gpu_destroy(g);
    }
  } gd{g};
  if (n_hulls == 0) { *out = g; gd.g = nullptr; return PARRYGPU_OK; }
  const void *dp = nullptr, *df = nullptr, *dc = nullptr;
  parrygpu_status s = stage_input(ctx, ctx->stage_in[0], points, (size_t)n_points * 12, &dp);
  if (s != PARRYGPU_OK) return s;
  if ((s = stage_input(ctx, ctx->stage_in[1], first, (size_t)n_hulls * 4, &df)) != PARRYGPU_OK) return s;
  if ((s = stage_input(ctx, ctx->stage_in[2], count, (size_t)n_hulls * 4, &dc)) != PARRYGPU_OK) return s;
  const uint32_t nh = (uint32_t)n_hulls;
  // the largest cloud sizes the workspaces
  PG_CUDA(ctx, gd.misc.reserve(16));
  PG_CUDA(ctx, cudaMemsetAsync(gd.misc.ptr, 0, 16, ctx->stream));
  k_hb_max<<<div_up(nh, 256), 256, 0, ctx->stream>>>(n_hulls, (const uint32_t*)dc, gd.misc.as<uint32_t>());
  PG_LAUNCHED(ctx);
  uint32_t max_n = 0;
  PG_CUDA(ctx, cudaMemcpyAsync(&max_n, gd.misc.ptr, 4, cudaMemcpyDeviceToHost, ctx->stream));
  PG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (max_n > 65535) return set_error(ctx, PARRYGPU_INVALID_ARG, "clouds of more than 65535 points");
  const HullCaps caps = HullCaps::of(max_n < 4 ? 4 : max_n);
  const uint32_t sms = ctx->sm_count > 0 ? (uint32_t)ctx->sm_count : 152u;
  uint32_t threads = (uint32_t)std::min<uint64_t>(n_hulls, (uint64_t)sms * 1024);
  while (threads > 32 && ws_total(caps, threads) > HB_WS_BUDGET) threads /= 2;
  threads = std::max(threads, 1u);
  // clouds in point-count order
  PG_CUDA(ctx, gd.keys[0].reserve((size_t)nh * 4));
  PG_CUDA(ctx, gd.keys[1].reserve((size_t)nh * 4));
  PG_CUDA(ctx, gd.vals[0].reserve((size_t)nh * 4));
  PG_CUDA(ctx, gd.vals[1].reserve((size_t)nh * 4));
  PG_CUDA(ctx, gd.hist.reserve((size_t)radix_sort_hist_entries(nh) * 4));
  k_hb_keys<<<div_up(nh, 256), 256, 0, ctx->stream>>>(n_hulls, (const uint32_t*)dc, caps.n, gd.keys[0].as<uint32_t>(),
                                                      gd.vals[0].as<uint32_t>(), ctx->d_err);
  PG_LAUNCHED(ctx);
  int rb = 0;
  if ((s = radix_sort_pairs_in(ctx, nh, 16, gd.keys[0].as<uint32_t>(), gd.vals[0].as<uint32_t>(), gd.keys[1].as<uint32_t>(),
                               gd.vals[1].as<uint32_t>(), gd.hist.as<uint32_t>(), &rb)) != PARRYGPU_OK)
    return s;
  const uint32_t* order = gd.vals[rb].as<uint32_t>();
  // a device short of memory gets fewer, longer-lived threads
  for (;;) {
    const cudaError_t we = gd.ws.reserve(ws_total(caps, threads));
    if (we == cudaSuccess) break;
    cudaGetLastError();
    if (we != cudaErrorMemoryAllocation || threads <= 32) return check_cuda(ctx, we, "hull workspaces");
    threads /= 2;
  }
  WsLayout lay{caps, threads, gd.ws.as<char>()};
  // sizes (then offsets), padded per array to a multiple of 4 words for the scan
  const size_t stride = ((size_t)nh + 4) & ~size_t(3);
  PG_CUDA(ctx, gd.sizes.reserve(NSIZES * stride * 4));
  PG_CUDA(ctx, cudaMemsetAsync(gd.sizes.ptr, 0, NSIZES * stride * 4, ctx->stream));
  uint32_t* sizes = gd.sizes.as<uint32_t>();
  // staging slots (256-byte blocks) of the single-build path
  PG_CUDA(ctx, gd.stage_off.reserve(stride * 4));
  PG_CUDA(ctx, cudaMemsetAsync(gd.stage_off.ptr, 0, stride * 4, ctx->stream));
  k_hb_stage_blocks<<<div_up(nh, 256), 256, 0, ctx->stream>>>(n_hulls, (const uint32_t*)dc, gd.stage_off.as<uint32_t>());
  PG_LAUNCHED(ctx);
  uint32_t sb[2] = {0, 0};
  PG_CUDA(ctx, cudaMemcpyAsync(&sb[0], gd.stage_off.as<uint32_t>() + (nh - 1), 4, cudaMemcpyDeviceToHost, ctx->stream));
  if ((s = exclusive_scan_u32(ctx, gd.stage_off.as<uint32_t>(), nh)) != PARRYGPU_OK) return s;
  PG_CUDA(ctx, cudaMemcpyAsync(&sb[1], gd.stage_off.as<uint32_t>() + (nh - 1), 4, cudaMemcpyDeviceToHost, ctx->stream));
  PG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  const size_t stage_bytes = ((size_t)sb[0] + sb[1]) * 256;
  const bool staged = stage_bytes <= HB_STAGE_BUDGET && gd.stage.reserve(stage_bytes + 256) == cudaSuccess;
  if (!staged) cudaGetLastError();  // a refused staging allocation only selects the two-pass path
  if (staged) {
    k_hb_build<<<div_up(threads, HB_THREADS), HB_THREADS, 0, ctx->stream>>>(lay, n_hulls, order, (const float*)dp, n_points,
                                                                            (const uint32_t*)df, (const uint32_t*)dc, gd.stage_off.as<uint32_t>(),
                                                                            gd.stage.as<uint32_t>(), sizes, stride, ctx->d_err);
    PG_LAUNCHED(ctx);
    PG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  } else {
    // k_hb_sizes indexes its arrays with stride n_hulls; copy them into the padded layout after
    DevBuf raw;
    PG_CUDA(ctx, raw.reserve(NSIZES * (size_t)nh * 4));
    k_hb_sizes<<<div_up(threads, HB_THREADS), HB_THREADS, 0, ctx->stream>>>(lay, n_hulls, order, (const float*)dp, n_points,
                                                                            (const uint32_t*)df, (const uint32_t*)dc, raw.as<uint32_t>(),
                                                                            ctx->d_err);
    cudaError_t ce = cudaGetLastError();
    ctx->launches++;
    for (int a = 0; a < NSIZES && ce == cudaSuccess; ++a)
      ce = cudaMemcpyAsync(sizes + a * stride, raw.as<uint32_t>() + (size_t)a * nh, (size_t)nh * 4, cudaMemcpyDeviceToDevice, ctx->stream);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(ctx->stream);
    raw.release();
    if (ce != cudaSuccess) return check_cuda(ctx, ce, "hull sizes");
  }
  if ((s = parrygpu_sync(ctx)) != PARRYGPU_OK) return set_error(ctx, PARRYGPU_INVALID_ARG, "a cloud's points lie outside the point array");
  // totals, then offsets
  uint32_t last[NSIZES];
  for (int a = 0; a < NSIZES; ++a) PG_CUDA(ctx, cudaMemcpyAsync(&last[a], sizes + a * stride + (nh - 1), 4, cudaMemcpyDeviceToHost, ctx->stream));
  // the exclusive scans need the sizes of the single-build path twice: keep a copy
  DevBuf counts_copy;
  if (staged) {
    PG_CUDA(ctx, counts_copy.reserve(NSIZES * stride * 4));
    PG_CUDA(ctx, cudaMemcpyAsync(counts_copy.ptr, sizes, NSIZES * stride * 4, cudaMemcpyDeviceToDevice, ctx->stream));
  }
  for (int a = 0; a < NSIZES; ++a)
    if ((s = exclusive_scan_u32(ctx, sizes + a * stride, nh)) != PARRYGPU_OK) { counts_copy.release(); return s; }
  uint32_t excl[NSIZES];
  for (int a = 0; a < NSIZES; ++a)
    PG_CUDA(ctx, cudaMemcpyAsync(&excl[a], sizes + a * stride + (nh - 1), 4, cudaMemcpyDeviceToHost, ctx->stream));
  PG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  for (int a = 0; a < 5; ++a) g->sizes[a] = (uint64_t)excl[a] + last[a];
  g->n_triangles = (uint64_t)excl[5] + last[5];
  PG_CUDA(ctx, g->points.reserve(g->sizes[0] * 12 + 16));
  PG_CUDA(ctx, g->vertex_ranges.reserve(g->sizes[0] * 8 + 16));
  PG_CUDA(ctx, g->hulls.reserve((size_t)nh * 32));
  PG_CUDA(ctx, g->face_normals.reserve(g->sizes[1] * 12 + 16));
  PG_CUDA(ctx, g->face_ranges.reserve(g->sizes[1] * 8 + 16));
  PG_CUDA(ctx, g->face_vertices.reserve(g->sizes[2] * 4 + 16));
  PG_CUDA(ctx, g->face_edges.reserve(g->sizes[2] * 4 + 16));
  PG_CUDA(ctx, g->vertex_faces.reserve(g->sizes[3] * 4 + 16));
  PG_CUDA(ctx, g->vertex_edges.reserve(g->sizes[3] * 4 + 16));
  PG_CUDA(ctx, g->edge_dirs.reserve(g->sizes[4] * 12 + 16));
  PG_CUDA(ctx, g->triangles.reserve(g->n_triangles * 12 + 16));
  PG_CUDA(ctx, g->tri_ranges.reserve((size_t)nh * 8));
  PolyOut o{g->points.as<float>(), g->hulls.as<uint32_t>(), g->face_normals.as<float>(), g->face_ranges.as<uint32_t>(),
            g->face_vertices.as<uint32_t>(), g->face_edges.as<uint32_t>(), g->vertex_ranges.as<uint32_t>(),
            g->vertex_faces.as<uint32_t>(), g->vertex_edges.as<uint32_t>(), g->edge_dirs.as<float>(), g->triangles.as<uint32_t>()};
  if (staged) {
    k_hb_copy<<<(unsigned)div_up((uint64_t)nh * 32, 256), 256, 0, ctx->stream>>>(n_hulls, (const uint32_t*)dc, gd.stage_off.as<uint32_t>(),
                                                                                 gd.stage.as<uint32_t>(), counts_copy.as<uint32_t>(), sizes,
                                                                                 stride, o, g->tri_ranges.as<uint32_t>());
    cudaError_t ce = cudaGetLastError();
    ctx->launches++;
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(ctx->stream);
    counts_copy.release();
    if (ce != cudaSuccess) return check_cuda(ctx, ce, "hull copy");
  } else {
    k_hb_emit<<<div_up(threads, HB_THREADS), HB_THREADS, 0, ctx->stream>>>(lay, n_hulls, order, (const float*)dp, n_points,
                                                                           (const uint32_t*)df, (const uint32_t*)dc, sizes, stride, o,
                                                                           g->tri_ranges.as<uint32_t>());
    PG_LAUNCHED(ctx);
  }
  PG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if ((s = parrygpu_sync(ctx)) != PARRYGPU_OK) return s;
  *out = g;
  gd.g = nullptr;
  return PARRYGPU_OK;
}

parrygpu_status parrygpu_polyhedra_gpu_sizes(const parrygpu_polyhedra_gpu* g, uint64_t* sizes) {
  if (!g || !sizes) return PARRYGPU_INVALID_ARG;
  for (int a = 0; a < 5; ++a) sizes[a] = g->sizes[a];
  return PARRYGPU_OK;
}

parrygpu_status parrygpu_polyhedra_gpu_copy(parrygpu_ctx* ctx, const parrygpu_polyhedra_gpu* g, float* points, uint32_t* hulls,
                                            float* face_normals, uint32_t* face_ranges, uint32_t* face_vertices, uint32_t* face_edges,
                                            uint32_t* vertex_ranges, uint32_t* vertex_faces, uint32_t* vertex_edges, float* edge_dirs) {
  if (!ctx || !g) return PARRYGPU_INVALID_ARG;
  PG_CUDA(ctx, cudaSetDevice(ctx->device));
  auto cp = [&](void* dst, const DevBuf& src, size_t bytes) -> cudaError_t {
    if (!dst || bytes == 0) return cudaSuccess;
    return cudaMemcpyAsync(dst, src.ptr, bytes, cudaMemcpyDefault, ctx->stream);
  };
  const uint64_t* z = g->sizes;
  PG_CUDA(ctx, cp(points, g->points, z[0] * 12));
  PG_CUDA(ctx, cp(hulls, g->hulls, g->n_hulls * 32));
  PG_CUDA(ctx, cp(face_normals, g->face_normals, z[1] * 12));
  PG_CUDA(ctx, cp(face_ranges, g->face_ranges, z[1] * 8));
  PG_CUDA(ctx, cp(face_vertices, g->face_vertices, z[2] * 4));
  PG_CUDA(ctx, cp(face_edges, g->face_edges, z[2] * 4));
  PG_CUDA(ctx, cp(vertex_ranges, g->vertex_ranges, z[0] * 8));
  PG_CUDA(ctx, cp(vertex_faces, g->vertex_faces, z[3] * 4));
  PG_CUDA(ctx, cp(vertex_edges, g->vertex_edges, z[3] * 4));
  PG_CUDA(ctx, cp(edge_dirs, g->edge_dirs, z[4] * 12));
  PG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return PARRYGPU_OK;
}

parrygpu_status parrygpu_polyhedra_gpu_view(const parrygpu_polyhedra_gpu* g, const float** points, parrygpu_polyhedra* view) {
  if (!g || !view) return PARRYGPU_INVALID_ARG;
  if (points) *points = g->points.as<float>();
  const uint64_t* z = g->sizes;
  *view = parrygpu_polyhedra{g->n_hulls,
                             g->hulls.as<uint32_t>(),
                             z[1],
                             g->face_normals.as<float>(),
                             g->face_ranges.as<uint32_t>(),
                             z[2],
                             g->face_vertices.as<uint32_t>(),
                             g->face_edges.as<uint32_t>(),
                             g->vertex_ranges.as<uint32_t>(),
                             z[3],
                             g->vertex_faces.as<uint32_t>(),
                             g->vertex_edges.as<uint32_t>(),
                             z[4],
                             g->edge_dirs.as<float>()};
  return PARRYGPU_OK;
}

parrygpu_status parrygpu_polyhedra_gpu_triangles(parrygpu_ctx* ctx, const parrygpu_polyhedra_gpu* g, uint64_t* n_triangles,
                                                 uint32_t* tri_ranges, uint32_t* triangles) {
  if (!ctx || !g) return PARRYGPU_INVALID_ARG;
  if (n_triangles) *n_triangles = g->n_triangles;
  PG_CUDA(ctx, cudaSetDevice(ctx->device));
  if (tri_ranges && g->n_hulls)
    PG_CUDA(ctx, cudaMemcpyAsync(tri_ranges, g->tri_ranges.ptr, g->n_hulls * 8, cudaMemcpyDefault, ctx->stream));
  if (triangles && g->n_triangles)
    PG_CUDA(ctx, cudaMemcpyAsync(triangles, g->triangles.ptr, g->n_triangles * 12, cudaMemcpyDefault, ctx->stream));
  PG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return PARRYGPU_OK;
}

void parrygpu_polyhedra_gpu_destroy(parrygpu_polyhedra_gpu* g) {
  if (!g) return;
  for (DevBuf* d : {&g->points, &g->hulls, &g->face_normals, &g->face_ranges, &g->face_vertices, &g->face_edges, &g->vertex_ranges,
                    &g->vertex_faces, &g->vertex_edges, &g->edge_dirs, &g->triangles, &g->tri_ranges})
    d->release();
  delete g;
}

}  // extern "C"
