// Triangle pseudo-normals of a TriMesh with TriMeshFlags::FIX_INTERNAL_EDGES, computed on the
// device. Paths relative to the parry repository:
//   src/shape/trimesh.rs:748-800     TriMesh::set_flags
//   src/shape/trimesh.rs:1251-1320   merge_duplicate_vertices (FIX_INTERNAL_EDGES implies it)
//   src/shape/trimesh.rs:1348-1407   compute_pseudo_normals (the edge part; vertex pseudo-normals
//                                    only serve point-containment queries)
//   src/shape/trimesh.rs:1911-1931   triangle_normal_constraints
//
// The reference walks the triangles in order with hash maps. Here the same sums come out of sorts:
//   1. corners (3 per triangle) sorted by their coordinate bits, three stable 32-bit passes (z, y,
//      x): equal runs are one merged vertex (bit-identical coordinates; a NaN never merges, as
//      PartialEq never holds for it); a scan of the run heads numbers the merged vertices;
//   2. the three edges of every triangle that has a normal, as (min, max) merged-vertex pairs, sorted
//      stably by (min, max) with the entry number 3t + slot as value, so each edge's entries sit
//      together in ascending triangle order;
//   3. each run sums its triangles' unit normals from zero in that order (the reference's
//      `*edge_n += *n`) and hands the sum to every entry of the run;
//   4. per triangle: face normal and the three sums normalised with Unit::try_new(., 1e-6); a
//      missing piece gives None.
// The result does not depend on how the merged vertices are numbered, only on which corners merge.
#include "internal.hpp"
#include "gjk_device.cuh"
#include "pseudo_device.cuh"

#include <cstring>

using namespace pg;

namespace {

constexpr int PN_THREADS = 256;

// Corner keys (coordinate bits) and face normals per original triangle, from the sorted soup.
__global__ void k_pn_corners(const float4* __restrict__ soup, uint32_t nt, uint32_t* __restrict__ kx, uint32_t* __restrict__ ky,
                             uint32_t* __restrict__ kz, uint32_t* __restrict__ sort_k, uint32_t* __restrict__ sort_v,
                             float4* __restrict__ face) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nt) return;
  const float4 x = soup[3 * (size_t)p], y = soup[3 * (size_t)p + 1], z = soup[3 * (size_t)p + 2];
  const uint32_t t = __float_as_uint(z.y);
  const V3 a = v3(x.x, x.y, x.z), b = v3(x.w, y.x, y.y), c = v3(y.z, y.w, z.x);
  const V3 cs[3] = {a, b, c};
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const size_t i = 3 * (size_t)t + k;
    kx[i] = __float_as_uint(cs[k].x);
    ky[i] = __float_as_uint(cs[k].y);
    kz[i] = __float_as_uint(cs[k].z);
    sort_k[i] = kz[i];
    sort_v[i] = (uint32_t)i;
  }
  // Triangle::normal: Unit::try_new((b - a) x (c - a), DEFAULT_EPSILON)
  V3 n = v3(0.f, 0.f, 0.f);
  const bool has = try_normalize(cross(b - a, c - a), FLT_EPSILON, &n);
  face[t] = make_float4(n.x, n.y, n.z, has ? 1.0f : 0.0f);
}

// Next key word of an LSD pass: keys[i] = src[vals_in[i]] (values carried over).
__global__ void k_pn_gather(uint32_t n, const uint32_t* __restrict__ src, const uint32_t* vals_in, uint32_t* vals_out,
                            uint32_t* __restrict__ keys) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t v = vals_in[i];
  keys[i] = src[v];
  vals_out[i] = v;
}

__device__ __forceinline__ bool bits_nan(uint32_t b) { return (b & 0x7f800000u) == 0x7f800000u && (b & 0x007fffffu) != 0u; }

// Run heads of the sorted corners: a corner starts a new merged vertex unless it has the bits of
// the previous one and no NaN coordinate.
__global__ void k_pn_corner_heads(uint32_t n, const uint32_t* __restrict__ order, const uint32_t* __restrict__ kx,
                                  const uint32_t* __restrict__ ky, const uint32_t* __restrict__ kz, uint32_t* __restrict__ head) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t c = order[i];
  const uint32_t x = kx[c], y = ky[c], z = kz[c];
  bool h = i == 0 || bits_nan(x) || bits_nan(y) || bits_nan(z);
  if (!h) {
    const uint32_t q = order[i - 1];
    h = kx[q] != x || ky[q] != y || kz[q] != z;
  }
  head[i] = h ? 1u : 0u;
}

// Merged-vertex id of each corner: the number of run heads before its run (exclusive scan + head).
__global__ void k_pn_corner_ids(uint32_t n, const uint32_t* __restrict__ order, const uint32_t* __restrict__ scan,
                                const uint32_t* __restrict__ head_in, uint32_t* __restrict__ vid) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  vid[order[i]] = scan[i] + head_in[i] - 1u;
}

// Edge entries 3t + slot (slots: edges 01, 12, 20) as (min, max) merged-vertex pairs; triangles
// without a normal add nothing to the sums and get the key (none, none) = (nv, nv), after all real
// edges.
__global__ void k_pn_edges(uint32_t nt, uint32_t none, const uint32_t* __restrict__ vid, const float4* __restrict__ face,
                           uint32_t* __restrict__ lo, uint32_t* __restrict__ hi, uint32_t* __restrict__ sort_k,
                           uint32_t* __restrict__ sort_v) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt) return;
  const bool has = face[t].w != 0.0f;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const size_t e = 3 * (size_t)t + k;
    uint32_t a = vid[3 * (size_t)t + k], b = vid[3 * (size_t)t + (k + 1) % 3];
    uint32_t l = a < b ? a : b, h = a < b ? b : a;
    if (!has) l = h = none;
    lo[e] = l;
    hi[e] = h;
    sort_k[e] = h;
    sort_v[e] = (uint32_t)e;
  }
}

// One thread per sorted entry; the first entry of each edge run sums the run's unit normals in
// ascending triangle order, from zero, and writes the sum to every entry of the run.
__global__ void k_pn_edge_sums(uint32_t n, uint32_t none, const uint32_t* __restrict__ order, const uint32_t* __restrict__ lo,
                               const uint32_t* __restrict__ hi, const float4* __restrict__ face, float4* __restrict__ sums) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t e = order[i];
  const uint32_t l = lo[e], h = hi[e];
  if (l == none) return;
  if (i > 0) {
    const uint32_t q = order[i - 1];
    if (lo[q] == l && hi[q] == h) return;
  }
  V3 s = v3(0.f, 0.f, 0.f);
  uint32_t j = i;
  for (; j < n; ++j) {
    const uint32_t f = order[j];
    if (lo[f] != l || hi[f] != h) break;
    const float4 fn = face[f / 3];
    s = s + v3(fn.x, fn.y, fn.z);
  }
  for (uint32_t q = i; q < j; ++q) sums[order[q]] = make_float4(s.x, s.y, s.z, 0.0f);
}

// TriMesh::triangle_normal_constraints of triangle t.
__global__ void k_pn_finish(uint32_t nt, const float4* __restrict__ face, const float4* __restrict__ sums, float* __restrict__ out,
                            uint8_t* __restrict__ ok) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt) return;
  const float4 f = face[t];
  float* o = out + 12 * (size_t)t;
  bool valid = f.w != 0.0f;
  V3 e[3] = {v3(0.f, 0.f, 0.f), v3(0.f, 0.f, 0.f), v3(0.f, 0.f, 0.f)};
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    if (!valid) break;
    const float4 s = sums[3 * (size_t)t + k];
    valid = try_normalize(v3(s.x, s.y, s.z), 1.0e-6f, &e[k]);
  }
  ok[t] = valid ? 1 : 0;
  const float v[12] = {f.x, f.y, f.z, e[0].x, e[0].y, e[0].z, e[1].x, e[1].y, e[1].z, e[2].x, e[2].y, e[2].z};
#pragma unroll
  for (int k = 0; k < 12; ++k) o[k] = valid ? v[k] : 0.0f;
}

__global__ void k_project_normals(uint64_t n, const float* __restrict__ pseudo, const float* __restrict__ dirs, float* __restrict__ out,
                                  uint8_t* __restrict__ ok) {
  const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const TriPN pn = load_tri_pn(pseudo, (uint32_t)i);
  V3 d = v3(dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]);
  ok[i] = project_local_normal_mut(pn, &d) ? 1 : 0;
  out[3 * i] = d.x;
  out[3 * i + 1] = d.y;
  out[3 * i + 2] = d.z;
}

int bits_for(uint32_t v) {
  int b = 0;
  while (b < 32 && (v >> b) != 0u) ++b;
  return b;
}

// Stable LSD sort by `words` key words (least significant first) of n entries whose first key word
// and identity values are already in ctx->sort_k[0] / sort_v[0]; `next[w]` is the source of key word
// w + 1, indexed by value. Returns the buffer holding the result.
parrygpu_status sort_words(parrygpu_ctx* ctx, uint32_t n, int words, const int* bits, const uint32_t* const* next, int* result) {
  int cur = 0;
  for (int w = 0; w < words; ++w) {
    if (w > 0) {
      k_pn_gather<<<div_up(n, PN_THREADS), PN_THREADS, 0, ctx->stream>>>(n, next[w - 1], ctx->sort_v[cur].as<uint32_t>(),
                                                                         ctx->sort_v[0].as<uint32_t>(), ctx->sort_k[0].as<uint32_t>());
      PG_LAUNCHED(ctx);
    }
    parrygpu_status s = radix_sort_pairs(ctx, n, bits[w], &cur);
    if (s != PARRYGPU_OK) return s;
  }
  *result = cur;
  return PARRYGPU_OK;
}

parrygpu_status compute_pseudo_normals(parrygpu_ctx* ctx, parrygpu_trimesh* m) {
  const uint32_t nt = m->n_triangles;
  PG_CUDA(ctx, m->pseudo.reserve((size_t)nt * 48 + 16));
  PG_CUDA(ctx, m->pseudo_ok.reserve((size_t)nt + 16));
  if (nt == 0) return PARRYGPU_OK;
  if ((uint64_t)nt * 3 >= 0xffffffffull) return set_error(ctx, PARRYGPU_INVALID_ARG, "too many triangles for pseudo-normals");
  const uint32_t nc = 3 * nt;
  DevBuf kx, ky, kz, vid, head, scan, face, sums;
  auto release = [&]() {
    for (DevBuf* d : {&kx, &ky, &kz, &vid, &head, &scan, &face, &sums}) d->release();
  };
  cudaError_t e = kx.reserve((size_t)nc * 4);
  if (e == cudaSuccess) e = ky.reserve((size_t)nc * 4);
  if (e == cudaSuccess) e = kz.reserve((size_t)nc * 4);
  if (e == cudaSuccess) e = vid.reserve((size_t)nc * 4);
  if (e == cudaSuccess) e = head.reserve((size_t)nc * 4 + 16);
  if (e == cudaSuccess) e = scan.reserve((size_t)nc * 4 + 16);
  if (e == cudaSuccess) e = face.reserve((size_t)nt * 16);
  if (e == cudaSuccess) e = sums.reserve((size_t)nc * 16);
  if (e != cudaSuccess) { release(); return check_cuda(ctx, e, "pseudo-normal scratch"); }
  parrygpu_status s = radix_sort_reserve(ctx, nc);
  if (s != PARRYGPU_OK) { release(); return s; }
  // 1. merged vertices
  k_pn_corners<<<div_up(nt, PN_THREADS), PN_THREADS, 0, ctx->stream>>>(m->soup.as<float4>(), nt, kx.as<uint32_t>(), ky.as<uint32_t>(),
                                                                       kz.as<uint32_t>(), ctx->sort_k[0].as<uint32_t>(),
                                                                       ctx->sort_v[0].as<uint32_t>(), face.as<float4>());
  PG_LAUNCHED(ctx);
  const int cbits[3] = {32, 32, 32};
  const uint32_t* cnext[2] = {ky.as<uint32_t>(), kx.as<uint32_t>()};
  int cur = 0;
  if ((s = sort_words(ctx, nc, 3, cbits, cnext, &cur)) != PARRYGPU_OK) { release(); return s; }
  const uint32_t* order = ctx->sort_v[cur].as<uint32_t>();
  k_pn_corner_heads<<<div_up(nc, PN_THREADS), PN_THREADS, 0, ctx->stream>>>(nc, order, kx.as<uint32_t>(), ky.as<uint32_t>(),
                                                                            kz.as<uint32_t>(), head.as<uint32_t>());
  PG_LAUNCHED(ctx);
  e = cudaMemsetAsync(scan.ptr, 0, (size_t)nc * 4 + 16, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(scan.ptr, head.ptr, (size_t)nc * 4, cudaMemcpyDeviceToDevice, ctx->stream);
  if (e != cudaSuccess) { release(); return check_cuda(ctx, e, "pseudo-normal scan"); }
  if ((s = exclusive_scan_u32(ctx, scan.as<uint32_t>(), nc)) != PARRYGPU_OK) { release(); return s; }
  k_pn_corner_ids<<<div_up(nc, PN_THREADS), PN_THREADS, 0, ctx->stream>>>(nc, order, scan.as<uint32_t>(), head.as<uint32_t>(),
                                                                          vid.as<uint32_t>());
  PG_LAUNCHED(ctx);
  uint32_t last[2] = {0, 0};
  e = cudaMemcpyAsync(&last[0], scan.as<uint32_t>() + (nc - 1), 4, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&last[1], head.as<uint32_t>() + (nc - 1), 4, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) { release(); return check_cuda(ctx, e, "pseudo-normal vertex count"); }
  const uint32_t nv = last[0] + last[1];  // merged vertices; nv doubles as the "no edge" id
  // 2. edges, sorted by (min, max): LSD on max, then min
  k_pn_edges<<<div_up(nt, PN_THREADS), PN_THREADS, 0, ctx->stream>>>(nt, nv, vid.as<uint32_t>(), face.as<float4>(), kx.as<uint32_t>(),
                                                                     ky.as<uint32_t>(), ctx->sort_k[0].as<uint32_t>(),
                                                                     ctx->sort_v[0].as<uint32_t>());
  PG_LAUNCHED(ctx);
  const int vb = bits_for(nv);
  const int ebits[2] = {vb, vb};
  const uint32_t* enext[1] = {kx.as<uint32_t>()};
  if ((s = sort_words(ctx, nc, 2, ebits, enext, &cur)) != PARRYGPU_OK) { release(); return s; }
  // 3. edge sums, 4. constraints
  k_pn_edge_sums<<<div_up(nc, PN_THREADS), PN_THREADS, 0, ctx->stream>>>(nc, nv, ctx->sort_v[cur].as<uint32_t>(), kx.as<uint32_t>(),
                                                                         ky.as<uint32_t>(), face.as<float4>(), sums.as<float4>());
  PG_LAUNCHED(ctx);
  k_pn_finish<<<div_up(nt, PN_THREADS), PN_THREADS, 0, ctx->stream>>>(nt, face.as<float4>(), sums.as<float4>(), m->pseudo.as<float>(),
                                                                      m->pseudo_ok.as<uint8_t>());
  PG_LAUNCHED(ctx);
  e = cudaStreamSynchronize(ctx->stream);
  release();
  if (e != cudaSuccess) return check_cuda(ctx, e, "pseudo-normals");
  return PARRYGPU_OK;
}

}  // namespace

extern "C" {

parrygpu_status parrygpu_trimesh_set_flags(parrygpu_ctx* ctx, parrygpu_trimesh* mesh, uint32_t flags) {
  if (!ctx || !mesh) return PARRYGPU_INVALID_ARG;
  const uint32_t known = PARRYGPU_TRIMESH_ORIENTED | PARRYGPU_TRIMESH_FIX_INTERNAL_EDGES;
  if (flags & ~known)
    return set_error(ctx, PARRYGPU_UNSUPPORTED_PAIR, "TriMeshFlags 0x%x: only ORIENTED, MERGE_DUPLICATE_VERTICES and FIX_INTERNAL_EDGES",
                     flags);
  PG_CUDA(ctx, cudaSetDevice(ctx->device));
  const bool want = (flags & PARRYGPU_TRIMESH_FIX_INTERNAL_EDGES) == PARRYGPU_TRIMESH_FIX_INTERNAL_EDGES;
  if (want && !mesh->pseudo.ptr) {
    parrygpu_status s = compute_pseudo_normals(ctx, mesh);
    if (s != PARRYGPU_OK) {
      mesh->pseudo.release();
      mesh->pseudo_ok.release();
      return s;
    }
  }
  mesh->flags = flags;
  return PARRYGPU_OK;
}

parrygpu_status parrygpu_trimesh_normal_constraints(parrygpu_ctx* ctx, const parrygpu_trimesh* mesh, float* pseudo, uint8_t* valid) {
  if (!ctx || !mesh) return PARRYGPU_INVALID_ARG;
  PG_CUDA(ctx, cudaSetDevice(ctx->device));
  const size_t nt = mesh->n_triangles;
  if (!mesh->constrained()) {  // None for every triangle: zeros
    auto zero = [&](void* p, size_t bytes) -> cudaError_t {
      cudaPointerAttributes a{};
      if (cudaPointerGetAttributes(&a, p) == cudaSuccess && (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged))
        return cudaMemsetAsync(p, 0, bytes, ctx->stream);
      std::memset(p, 0, bytes);
      return cudaSuccess;
    };
    if (pseudo && nt) PG_CUDA(ctx, zero(pseudo, nt * 48));
    if (valid && nt) PG_CUDA(ctx, zero(valid, nt));
    return parrygpu_sync(ctx);
  }
  if (pseudo && nt) PG_CUDA(ctx, cudaMemcpyAsync(pseudo, mesh->pseudo.ptr, nt * 48, cudaMemcpyDefault, ctx->stream));
  if (valid && nt) PG_CUDA(ctx, cudaMemcpyAsync(valid, mesh->pseudo_ok.ptr, nt, cudaMemcpyDefault, ctx->stream));
  return parrygpu_sync(ctx);
}

parrygpu_status parrygpu_project_local_normals(parrygpu_ctx* ctx, const float* pseudo, const float* dirs, uint64_t n, float* out,
                                               uint8_t* ok) {
  if (!ctx || (n && (!pseudo || !dirs || !out || !ok))) return PARRYGPU_INVALID_ARG;
  if (n == 0) return PARRYGPU_OK;
  PG_CUDA(ctx, cudaSetDevice(ctx->device));
  const void *dp = nullptr, *dd = nullptr;
  parrygpu_status s = stage_input(ctx, ctx->stage_in[0], pseudo, (size_t)n * 48, &dp);
  if (s != PARRYGPU_OK) return s;
  if ((s = stage_input(ctx, ctx->stage_in[1], dirs, (size_t)n * 12, &dd)) != PARRYGPU_OK) return s;
  void *dout = nullptr, *dok = nullptr;
  bool copy_out = false, copy_ok = false;
  if ((s = stage_output(ctx, ctx->stage_out[0], out, (size_t)n * 12, &dout, &copy_out)) != PARRYGPU_OK) return s;
  if ((s = stage_output(ctx, ctx->stage_out[1], ok, (size_t)n, &dok, &copy_ok)) != PARRYGPU_OK) return s;
  k_project_normals<<<(unsigned)((n + PN_THREADS - 1) / PN_THREADS), PN_THREADS, 0, ctx->stream>>>(n, (const float*)dp, (const float*)dd,
                                                                                                   (float*)dout, (uint8_t*)dok);
  PG_LAUNCHED(ctx);
  if (copy_out) PG_CUDA(ctx, cudaMemcpyAsync(out, dout, (size_t)n * 12, cudaMemcpyDeviceToHost, ctx->stream));
  if (copy_ok) PG_CUDA(ctx, cudaMemcpyAsync(ok, dok, (size_t)n, cudaMemcpyDeviceToHost, ctx->stream));
  return parrygpu_sync(ctx);
}

}  // extern "C"
