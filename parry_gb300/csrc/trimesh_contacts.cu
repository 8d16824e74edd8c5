// Contact manifolds of shapes against a TriMesh, frame after frame: contact_manifolds_trimesh_shape
// (src/query/contact_manifolds/contact_manifolds_trimesh_shape.rs:82-228, path relative to the parry
// repository) for a whole set of shapes against one mesh, with the reference's per-pair workspace:
//   - the shape's AABB in the mesh frame, loosened by the prediction, is kept while it still
//     contains the new one; otherwise it is enlarged by min(extent / 10, 0.1) per axis and the
//     triangles whose AABBs intersect it are queried again from the mesh's BVH;
//   - one ContactManifold per interfering triangle, carried over by triangle id when the list is
//     queried again (a new triangle starts from ContactManifold::new());
//   - each (triangle, shape) manifold is DefaultQueryDispatcher::contact_manifold_convex_convex with
//     the triangle as shape 1 and, when the mesh has FIX_INTERNAL_EDGES, the triangle's
//     pseudo-normals as its normal constraints (TriMesh::triangle_normal_constraints).
// Interference lists are kept in ascending triangle order: the reference's carry-over loop walks the
// old and new lists as sorted lists, and its BVH returns them in tree order.
//
// Layout: shape s owns K slots (interference ids, manifold records, pair entries). The manifold
// kernels run over all n x K slots of a combined shape set [shapes | triangles]; an unused slot holds
// the empty pair (PARRYGPU_PAIR_NONE, PARRYGPU_PAIR_NONE), which the manifold kernels skip.
#include "internal.hpp"
#include "contact_device.cuh"
#include "lbvh_device.cuh"

#include <cstring>

using namespace pg;

struct parrygpu_trimesh_contacts {
  const parrygpu_trimesh* mesh = nullptr;
  uint32_t n = 0, k = 0, n_tris = 0;
  DevBuf tri_pool;                  // 9 floats per triangle, original order
  DevBuf aabb;                      // n x 6: the workspace's local_aabb2 (invalid at first)
  DevBuf inter[2], count[2], recs[2];
  DevBuf map;                       // n x K: source slot of each new slot in the previous buffer, or -1
  DevBuf pairs;                     // n x K pairs (triangle shape, shape)
  DevBuf types, params, poses, pool;  // combined shape set
  MfScratch mf;
  int cur = 0;
};

namespace {

constexpr int TC_THREADS = 128;
constexpr int TC_STACK = 64;
constexpr uint32_t MANIFOLD_WORDS = 8u + 10u * PARRYGPU_MANIFOLD_MAX_POINTS;

// Triangle vertices of every soup position back in the mesh's original triangle order.
__global__ void k_tri_pool(const float4* __restrict__ soup, uint32_t nt, float* __restrict__ pool) {
  uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nt) return;
  float4 x = soup[3 * (size_t)p], y = soup[3 * (size_t)p + 1], z = soup[3 * (size_t)p + 2];
  uint32_t t = __float_as_uint(z.y);
  float* o = pool + 9 * (size_t)t;
  o[0] = x.x; o[1] = x.y; o[2] = x.z; o[3] = x.w; o[4] = y.x; o[5] = y.y; o[6] = y.z; o[7] = y.w; o[8] = z.x;
}

__global__ void k_invalid_aabbs(float* __restrict__ aabb, uint32_t n) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float* a = aabb + 6 * (size_t)i;
  a[0] = a[1] = a[2] = FLT_MAX;  // Aabb::new_invalid
  a[3] = a[4] = a[5] = -FLT_MAX;
}

// The triangle part of the combined shape set: triangle t is shape n + t with its vertices at pool
// offset m + 3t, posed at the mesh pose; params word 2 = t + 1 when the triangle has normal
// constraints (row t of the mesh's pseudo-normal table; `ok` null = none).
__global__ void k_fill_triangles(uint32_t n, uint32_t nt, uint64_t m, Pose mesh, const uint8_t* __restrict__ ok,
                                 uint32_t* __restrict__ types, float4* __restrict__ params, float* __restrict__ poses) {
  uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt) return;
  uint32_t i = n + t;
  types[i] = SH_TRIANGLE;
  const uint32_t row = (ok && ok[t]) ? t + 1u : 0u;
  params[i] = make_float4(__uint_as_float((uint32_t)(m + 3ull * t)), __uint_as_float(3u), __uint_as_float(row), 0.0f);
  float* p = poses + 7 * (size_t)i;
  p[0] = mesh.qi; p[1] = mesh.qj; p[2] = mesh.qk; p[3] = mesh.qw; p[4] = mesh.t.x; p[5] = mesh.t.y; p[6] = mesh.t.z;
}

// One thread per shape: the workspace step of contact_manifolds_trimesh_shape. Writes the shape's
// new interference list (ascending), for each new slot the slot of the previous list it carries
// over (or -1), and the K pair entries of the shape.
__global__ void __launch_bounds__(TC_THREADS) k_tc_workspace(ShapeArrays sh, uint32_t n, uint32_t K, Pose mesh, float prediction,
                                                             const WideNode* __restrict__ wide, const float4* __restrict__ soup,
                                                             float* __restrict__ aabb, const uint32_t* __restrict__ old_inter,
                                                             const uint32_t* __restrict__ old_count, uint32_t* __restrict__ new_inter,
                                                             uint32_t* __restrict__ new_count, int32_t* __restrict__ map,
                                                             uint32_t* __restrict__ pairs, uint32_t* __restrict__ err) {
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const size_t base = (size_t)s * K;
  uint32_t* ni = new_inter + base;
  int32_t* mp = map + base;
  const uint32_t* oi = old_inter + base;
  const uint32_t oc = old_count[s];
  uint32_t c = 0;
  if (!valid_pair(sh, s, s)) {
    atomicOr(err, ERR_BAD_INDEX);
  } else {
    ShapeDev sd = load_shape(sh.types, sh.params, sh.pool, s);
    Pose pos12 = pose_inv_mul(mesh, load_pose(sh.poses, s));
    V3 mn, mx;
    shape_world_aabb(sd, pos12, &mn, &mx);
    if (prediction > 0.0f) {  // Aabb::loosened(prediction)
      mn = mn + v3(-prediction, -prediction, -prediction);
      mx = mx + v3(prediction, prediction, prediction);
    }
    float* a = aabb + 6 * (size_t)s;
    const bool same = a[0] <= mn.x && a[1] <= mn.y && a[2] <= mn.z && a[3] >= mx.x && a[4] >= mx.y && a[5] >= mx.z;
    if (same) {
      c = oc;
      for (uint32_t j = 0; j < c; ++j) { ni[j] = oi[j]; mp[j] = (int32_t)j; }
    } else {
      V3 e = mx - mn;
      V3 extra = v3(fminf(e.x / 10.0f, 0.1f), fminf(e.y / 10.0f, 0.1f), fminf(e.z / 10.0f, 0.1f));
      mn = mn - extra;
      mx = mx + extra;
      a[0] = mn.x; a[1] = mn.y; a[2] = mn.z; a[3] = mx.x; a[4] = mx.y; a[5] = mx.z;
      // Bvh::intersect_aabb: every leaf whose AABB intersects the query (inclusive on every axis)
      bool full = false;
      auto hits = [&](const BvhNodeDev& b) {
        return b.mins.x <= mx.x && b.mins.y <= mx.y && b.mins.z <= mx.z && b.maxs.x >= mn.x && b.maxs.y >= mn.y && b.maxs.z >= mn.z;
      };
      auto leaf = [&](uint32_t pos) {
        if (c < K) ni[c++] = __float_as_uint(soup[3 * (size_t)pos + 2].y);
        else full = true;
      };
      WideNode w;
      load_wide(wide, 0, &w);
      if ((w.r.data & 0x3fffffffu) == 0u) {
        if (hits(w.l)) leaf(w.l.children);
      } else {
        uint32_t stack[TC_STACK];
        int sp = 0;
        for (;;) {
          uint32_t next = 0xffffffffu;
          const BvhNodeDev* ch[2] = {&w.l, &w.r};
#pragma unroll
          for (int q = 0; q < 2; ++q) {
            if (!hits(*ch[q])) continue;
            if ((ch[q]->data & 0x3fffffffu) == 1u) leaf(ch[q]->children);
            else if (next == 0xffffffffu) next = ch[q]->children;
            else if (sp < TC_STACK) stack[sp++] = ch[q]->children;
            else atomicOr(err, ERR_STACK_OVERFLOW);
          }
          if (next == 0xffffffffu) {
            if (sp == 0) break;
            next = stack[--sp];
          }
          load_wide(wide, next, &w);
        }
      }
      if (full) atomicOr(err, ERR_CAPACITY);
      for (uint32_t j = 1; j < c; ++j) {  // ascending triangle order
        uint32_t v = ni[j];
        uint32_t q = j;
        while (q > 0 && ni[q - 1] > v) { ni[q] = ni[q - 1]; --q; }
        ni[q] = v;
      }
      uint32_t io = 0;  // the reference's carry-over walk over the previous (sorted) list
      for (uint32_t j = 0; j < c; ++j) {
        while (io < oc && oi[io] < ni[j]) ++io;
        if (io < oc && oi[io] == ni[j]) { mp[j] = (int32_t)io; ++io; }
        else mp[j] = -1;
      }
    }
  }
  new_count[s] = c;
  uint32_t* pr = pairs + 2 * base;
  for (uint32_t j = 0; j < K; ++j) {
    pr[2 * j] = j < c ? n + ni[j] : PARRYGPU_PAIR_NONE;
    pr[2 * j + 1] = j < c ? s : PARRYGPU_PAIR_NONE;
  }
}

// One thread per slot: the record of a new slot is its carried-over record (header and live
// points) or ContactManifold::new().
__global__ void k_tc_carry(uint32_t n, uint32_t K, const uint32_t* __restrict__ new_count, const int32_t* __restrict__ map,
                           const uint32_t* __restrict__ old_recs, uint32_t* __restrict__ new_recs) {
  const uint64_t idx = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (idx >= (uint64_t)n * K) return;
  const uint32_t s = (uint32_t)(idx / K), j = (uint32_t)(idx % K);
  if (j >= new_count[s]) return;
  uint32_t* dst = new_recs + idx * MANIFOLD_WORDS;
  const int32_t src = map[idx];
  if (src < 0) {
#pragma unroll
    for (int w = 0; w < 8; ++w) dst[w] = 0u;
    return;
  }
  const uint32_t* from = old_recs + ((uint64_t)s * K + (uint32_t)src) * MANIFOLD_WORDS;
  uint32_t np = from[0] < (uint32_t)PARRYGPU_MANIFOLD_MAX_POINTS ? from[0] : (uint32_t)PARRYGPU_MANIFOLD_MAX_POINTS;
  const uint32_t words = 8u + 10u * np;
  for (uint32_t w = 0; w < words; ++w) dst[w] = from[w];
}

}  // namespace

extern "C" {

parrygpu_status parrygpu_trimesh_contacts_create(parrygpu_ctx* ctx, const parrygpu_trimesh* mesh, uint32_t n_shapes, uint32_t max_per_shape,
                                                 parrygpu_trimesh_contacts** out) {
  if (!ctx || !mesh || !out || max_per_shape == 0) return PARRYGPU_INVALID_ARG;
  *out = nullptr;
  if ((uint64_t)n_shapes * max_per_shape > 0x7fffffffull) return set_error(ctx, PARRYGPU_INVALID_ARG, "too many slots (shapes x max_per_shape)");
  PG_CUDA(ctx, cudaSetDevice(ctx->device));
  auto* tc = new parrygpu_trimesh_contacts();
  tc->mesh = mesh;
  tc->n = n_shapes;
  tc->k = max_per_shape;
  tc->n_tris = mesh->n_triangles;
  const size_t slots = (size_t)n_shapes * max_per_shape;
  cudaError_t e = tc->tri_pool.reserve((size_t)tc->n_tris * 36 + 16);
  if (e == cudaSuccess) e = tc->aabb.reserve((size_t)n_shapes * 24 + 16);
  for (int b = 0; b < 2 && e == cudaSuccess; ++b) {
    e = tc->inter[b].reserve(slots * 4 + 16);
    if (e == cudaSuccess) e = tc->count[b].reserve((size_t)n_shapes * 4 + 16);
    if (e == cudaSuccess) e = tc->recs[b].reserve(slots * MANIFOLD_WORDS * 4 + 16);
    if (e == cudaSuccess) e = cudaMemsetAsync(tc->count[b].ptr, 0, (size_t)n_shapes * 4 + 16, ctx->stream);
  }
  if (e == cudaSuccess) e = tc->map.reserve(slots * 4 + 16);
  if (e == cudaSuccess) e = tc->pairs.reserve(slots * 8 + 16);
  if (e != cudaSuccess) { parrygpu_trimesh_contacts_destroy(tc); return check_cuda(ctx, e, "trimesh contacts buffers"); }
  if (tc->n_tris) {
    k_tri_pool<<<div_up(tc->n_tris, 256), 256, 0, ctx->stream>>>(mesh->soup.as<float4>(), tc->n_tris, tc->tri_pool.as<float>());
    PG_LAUNCHED(ctx);
  }
  if (n_shapes) {
    k_invalid_aabbs<<<div_up(n_shapes, 256), 256, 0, ctx->stream>>>(tc->aabb.as<float>(), n_shapes);
    PG_LAUNCHED(ctx);
  }
  parrygpu_status s = manifolds_reserve(ctx, slots, tc->mf);
  if (s != PARRYGPU_OK) { parrygpu_trimesh_contacts_destroy(tc); return s; }
  e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) { parrygpu_trimesh_contacts_destroy(tc); return check_cuda(ctx, e, "trimesh contacts setup"); }
  *out = tc;
  return PARRYGPU_OK;
}

void parrygpu_trimesh_contacts_destroy(parrygpu_trimesh_contacts* tc) {
  if (!tc) return;
  cudaDeviceSynchronize();
  for (DevBuf* d : {&tc->tri_pool, &tc->aabb, &tc->inter[0], &tc->inter[1], &tc->count[0], &tc->count[1], &tc->recs[0], &tc->recs[1],
                    &tc->map, &tc->pairs, &tc->types, &tc->params, &tc->poses, &tc->pool, &tc->mf.queue, &tc->mf.counters, &tc->mf.bins,
                    &tc->mf.epa_ws})
    d->release();
  delete tc;
}

parrygpu_status parrygpu_trimesh_contacts_update(parrygpu_ctx* ctx, parrygpu_trimesh_contacts* tc, const float* mesh_pose7,
                                                 const parrygpu_shapes* shapes, float prediction) {
  if (!ctx || !tc || !shapes) return PARRYGPU_INVALID_ARG;
  if (shapes->n != tc->n) return set_error(ctx, PARRYGPU_INVALID_ARG, "the workspace was created for %u shapes", tc->n);
  if (tc->n == 0) return PARRYGPU_OK;
  PG_CUDA(ctx, cudaSetDevice(ctx->device));
  Pose mesh{0.f, 0.f, 0.f, 1.f, v3(0.f, 0.f, 0.f)};
  if (mesh_pose7) mesh = Pose{mesh_pose7[0], mesh_pose7[1], mesh_pose7[2], mesh_pose7[3], v3(mesh_pose7[4], mesh_pose7[5], mesh_pose7[6])};
  ShapeArrays sh;
  parrygpu_status s = stage_shapes(ctx, shapes, &sh);
  if (s != PARRYGPU_OK) return s;
  const uint32_t n = tc->n, nt = tc->n_tris, K = tc->k;
  const uint64_t m = shapes->n_vertices, total = (uint64_t)n + nt, nv = m + 3ull * nt;
  if (total >= PARRYGPU_PAIR_NONE) return set_error(ctx, PARRYGPU_INVALID_ARG, "too many shapes and triangles");
  if (nv > 0xffffffffull) return set_error(ctx, PARRYGPU_INVALID_ARG, "too many vertices");
  PG_CUDA(ctx, tc->types.reserve(total * 4));
  PG_CUDA(ctx, tc->params.reserve(total * 16));
  PG_CUDA(ctx, tc->poses.reserve(total * 28));
  PG_CUDA(ctx, tc->pool.reserve(nv * 12 + 16));
  PG_CUDA(ctx, cudaMemcpyAsync(tc->types.ptr, sh.types, (size_t)n * 4, cudaMemcpyDeviceToDevice, ctx->stream));
  PG_CUDA(ctx, cudaMemcpyAsync(tc->params.ptr, sh.params, (size_t)n * 16, cudaMemcpyDeviceToDevice, ctx->stream));
  PG_CUDA(ctx, cudaMemcpyAsync(tc->poses.ptr, sh.poses, (size_t)n * 28, cudaMemcpyDeviceToDevice, ctx->stream));
  if (m) PG_CUDA(ctx, cudaMemcpyAsync(tc->pool.ptr, sh.pool, m * 12, cudaMemcpyDeviceToDevice, ctx->stream));
  if (nt) PG_CUDA(ctx, cudaMemcpyAsync(tc->pool.as<float>() + 3 * m, tc->tri_pool.ptr, (size_t)nt * 36, cudaMemcpyDeviceToDevice, ctx->stream));
  if (nt) {
    k_fill_triangles<<<div_up(nt, 256), 256, 0, ctx->stream>>>(n, nt, m, mesh,
                                                               tc->mesh->constrained() ? tc->mesh->pseudo_ok.as<uint8_t>() : nullptr,
                                                               tc->types.as<uint32_t>(), tc->params.as<float4>(), tc->poses.as<float>());
    PG_LAUNCHED(ctx);
  }
  ShapeArrays cs{tc->types.as<uint32_t>(), tc->params.as<float4>(), tc->poses.as<float>(), tc->pool.as<float>(), total, nv, sh.poly,
                 tc->mesh->constrained() ? tc->mesh->pseudo.as<float>() : nullptr, n};
  const int cur = tc->cur, nw = 1 - cur;
  {
    KernelTimer kt(ctx, "trimesh_contacts_workspace");
    k_tc_workspace<<<div_up(n, TC_THREADS), TC_THREADS, 0, ctx->stream>>>(
        cs, n, K, mesh, prediction, tc->mesh->bvh.wide.as<WideNode>(), tc->mesh->soup.as<float4>(), tc->aabb.as<float>(),
        tc->inter[cur].as<uint32_t>(), tc->count[cur].as<uint32_t>(), tc->inter[nw].as<uint32_t>(), tc->count[nw].as<uint32_t>(),
        tc->map.as<int32_t>(), tc->pairs.as<uint32_t>(), ctx->d_err);
    kt.stop();
    PG_LAUNCHED(ctx);
  }
  const uint64_t slots = (uint64_t)n * K;
  k_tc_carry<<<div_up(slots, 256), 256, 0, ctx->stream>>>(n, K, tc->count[nw].as<uint32_t>(), tc->map.as<int32_t>(), tc->recs[cur].as<uint32_t>(),
                                                            tc->recs[nw].as<uint32_t>());
  PG_LAUNCHED(ctx);
  {
    KernelTimer kt(ctx, "trimesh_contacts_manifolds");
    if ((s = launch_manifolds(ctx, cs, tc->pairs.as<uint32_t>(), slots, nullptr, prediction, tc->recs[nw].as<uint32_t>(), tc->mf)) != PARRYGPU_OK)
      return s;
    kt.stop();
  }
  tc->cur = nw;
  if (sh.types != shapes->types || sh.params != (const void*)shapes->params || sh.poses != shapes->poses ||
      (m && sh.pool != shapes->vertices))
    return parrygpu_sync(ctx);  // staged host inputs are reused by the next call
  return PARRYGPU_OK;
}

parrygpu_status parrygpu_trimesh_contacts_read(parrygpu_ctx* ctx, const parrygpu_trimesh_contacts* tc, uint32_t* counts, uint32_t* triangles,
                                               parrygpu_manifold* manifolds) {
  if (!ctx || !tc) return PARRYGPU_INVALID_ARG;
  PG_CUDA(ctx, cudaSetDevice(ctx->device));
  const size_t slots = (size_t)tc->n * tc->k;
  if (counts) PG_CUDA(ctx, cudaMemcpyAsync(counts, tc->count[tc->cur].ptr, (size_t)tc->n * 4, cudaMemcpyDefault, ctx->stream));
  if (triangles) PG_CUDA(ctx, cudaMemcpyAsync(triangles, tc->inter[tc->cur].ptr, slots * 4, cudaMemcpyDefault, ctx->stream));
  if (manifolds) PG_CUDA(ctx, cudaMemcpyAsync(manifolds, tc->recs[tc->cur].ptr, slots * MANIFOLD_WORDS * 4, cudaMemcpyDefault, ctx->stream));
  return parrygpu_sync(ctx);
}

}  // extern "C"
