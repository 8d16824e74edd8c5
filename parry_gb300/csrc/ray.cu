// Batched ray casts against a triangle mesh (TriMesh + RayCast replacement).
//
// Mesh layout in HBM (all L2-resident for meshes of ~10^5 triangles):
//   wide : LBVH in BvhNodeWide layout; leaf `children` = sorted position of the triangle
//   soup : per sorted position, the triangle's three vertices + original index in 3 x float4
//          (48 B), so a leaf test is three 16-byte loads from the cache line next to its
//          neighbours in Morton order.
// Rays are optionally Morton-sorted by origin first (coherent traversal); results are written to
// the ray's original slot.
//
// Per-ray algorithm: best-first descent of the reference's Bvh::find_best
// (src/partitioning/bvh/bvh_traverse.rs:335-417) with the node cost of BvhNode::cast_ray
// (src/partitioning/bvh/bvh_tree.rs:1177-1181 -> src/query/ray/ray_aabb.rs:12-49) and the leaf
// cost of Triangle::cast_local_ray_and_get_normal (src/query/ray/ray_triangle.rs:49-152). Exact toi
// ties go to the lowest triangle index: nodes whose entry time equals the best toi are still
// visited, and an equal toi replaces the best only with a smaller triangle index.
#include "internal.hpp"
#include "common.cuh"
#include "lbvh_device.cuh"
#include "tri_ray_device.cuh"

using namespace pg;

namespace {

constexpr int RAY_STACK = 64;

// Normal of the winning triangle, as ray_triangle.rs computes it (faces the ray origin).
__device__ __forceinline__ V3 ray_triangle_normal(V3 a, V3 b, V3 c, V3 o) {
  V3 ab = b - a;
  V3 ac = c - a;
  V3 n = cross(ab, ac);
  V3 ap = o - a;
  float t = dot(ap, n);
  return t < 0.0f ? -normalize(n) : normalize(n);
}

// src/query/ray/ray_aabb.rs:12-49 with solid = true; FLT_MAX on a miss.
__device__ __forceinline__ float slab(float3 mn, float3 mx, V3 o, V3 inv, uint32_t zmask, float max_toi) {
  float tmin = 0.0f, tmax = max_toi;
  bool miss = false;
  if (zmask & 1u) {
    miss |= (o.x < mn.x) | (o.x > mx.x);
  } else {
    float n = (mn.x - o.x) * inv.x, f = (mx.x - o.x) * inv.x;
    if (n > f) { float s = n; n = f; f = s; }
    tmin = fmaxf(tmin, n); tmax = fminf(tmax, f);
  }
  if (zmask & 2u) {
    miss |= (o.y < mn.y) | (o.y > mx.y);
  } else {
    float n = (mn.y - o.y) * inv.y, f = (mx.y - o.y) * inv.y;
    if (n > f) { float s = n; n = f; f = s; }
    tmin = fmaxf(tmin, n); tmax = fminf(tmax, f);
  }
  if (zmask & 4u) {
    miss |= (o.z < mn.z) | (o.z > mx.z);
  } else {
    float n = (mn.z - o.z) * inv.z, f = (mx.z - o.z) * inv.z;
    if (n > f) { float s = n; n = f; f = s; }
    tmin = fmaxf(tmin, n); tmax = fminf(tmax, f);
  }
  return (!miss && tmin <= tmax) ? tmin : FLT_MAX;
}

__device__ __forceinline__ void load_tri(const float4* __restrict__ soup, uint32_t p, V3* a, V3* b, V3* c, uint32_t* orig) {
  const float4* s = soup + 3 * (size_t)p;
  float4 x = __ldg(s), y = __ldg(s + 1), z = __ldg(s + 2);
  *a = v3(x.x, x.y, x.z);
  *b = v3(x.w, y.x, y.y);
  *c = v3(y.z, y.w, z.x);
  *orig = __float_as_uint(z.y);
}

// Per-ray traversal state: the ray in mesh space and its best hit so far.
struct RayState {
  V3 o, dir, inv;
  uint32_t zmask;
  float best;
  uint32_t best_orig, best_pos;
  bool have;
};

template <bool HAS_POSE>
__device__ __forceinline__ void ray_init(const float* __restrict__ rays, uint32_t r, float max_toi, const Pose& pose, RayState* st) {
  const float* rp = rays + 6 * (size_t)r;
  V3 o = v3(rp[0], rp[1], rp[2]);
  V3 dir = v3(rp[3], rp[4], rp[5]);
  if (HAS_POSE) {
    o = pose_inv_point(pose, o);
    dir = pose_inv_rotate(pose, dir);
  }
  st->o = o;
  st->dir = dir;
  st->zmask = (dir.x == 0.0f ? 1u : 0u) | (dir.y == 0.0f ? 2u : 0u) | (dir.z == 0.0f ? 4u : 0u);
  st->inv = v3(dir.x != 0.0f ? 1.0f / dir.x : 0.0f, dir.y != 0.0f ? 1.0f / dir.y : 0.0f, dir.z != 0.0f ? 1.0f / dir.z : 0.0f);
  st->best = max_toi;
  st->best_orig = 0xffffffffu;
  st->best_pos = 0xffffffffu;
  st->have = false;
}

// Triangle::cast_local_ray_and_get_normal on soup triangle `pos` (accepts toi <= best); exact
// toi ties keep the lowest original triangle index.
__device__ __forceinline__ void ray_try_leaf(const float4* __restrict__ soup, uint32_t pos, RayState* st) {
  V3 a, b, c;
  uint32_t orig;
  load_tri(soup, pos, &a, &b, &c, &orig);
  TriHit h;
  if (!ray_triangle_toi(a, b, c, st->o, st->dir, &h)) return;
  if (!(h.toi <= st->best)) return;
  if (h.toi < st->best || (st->have && h.toi == st->best && orig < st->best_orig)) {
    st->best = h.toi; st->best_orig = orig; st->best_pos = pos; st->have = true;
  }
}

// One traversal step at wide node `w`: both children's slab tests, leaf children tested at once,
// the nearer internal child returned (the farther one pushed), or the next stack entry; returns
// 0xffffffff when the traversal is over (or the stack overflowed, with the error flag raised).
__device__ __forceinline__ uint32_t ray_step(const WideNode& w, const float4* __restrict__ soup, RayState* st, uint32_t* stack, int* sp,
                                             uint32_t* __restrict__ err) {
  float ls = slab(w.l.mins, w.l.maxs, st->o, st->inv, st->zmask, st->best);
  float rs = slab(w.r.mins, w.r.maxs, st->o, st->inv, st->zmask, st->best);
  const BvhNodeDev* nearn = &w.l;
  const BvhNodeDev* farn = &w.r;
  if (ls > rs) { float t = ls; ls = rs; rs = t; nearn = &w.r; farn = &w.l; }
  uint32_t next = 0xffffffffu;
  if (ls != FLT_MAX && (ls < st->best || (st->have && ls == st->best))) {
    if ((nearn->data & 0x3fffffffu) == 1u) ray_try_leaf(soup, nearn->children, st);
    else next = nearn->children;
  }
  if (rs != FLT_MAX && (rs < st->best || (st->have && rs == st->best))) {
    if ((farn->data & 0x3fffffffu) == 1u) {
      ray_try_leaf(soup, farn->children, st);
    } else if (next != 0xffffffffu) {
      if (*sp >= RAY_STACK) { atomicOr(err, ERR_STACK_OVERFLOW); return 0xffffffffu; }
      stack[(*sp)++] = farn->children;
    } else {
      next = farn->children;
    }
  }
  if (next == 0xffffffffu && *sp > 0) next = stack[--(*sp)];
  return next;
}

// Writes ray r's answer (feature, toi, normal facing the origin) from its final state.
template <bool HAS_POSE, bool WANT_NORMAL>
__device__ __forceinline__ void ray_finish(const float4* __restrict__ soup, uint32_t n_tris, const Pose& pose, const RayState& st, uint32_t r,
                                           uint32_t* __restrict__ feat, float* __restrict__ toi_out, float* __restrict__ normal_out) {
  if (st.have) {
    V3 a, b, c;
    uint32_t orig;
    load_tri(soup, st.best_pos, &a, &b, &c, &orig);
    TriHit h;
    ray_triangle_toi(a, b, c, st.o, st.dir, &h);
    feat[r] = h.fid == 1u ? st.best_orig + n_tris : st.best_orig;
    toi_out[r] = st.best;
    if (WANT_NORMAL) {
      V3 nrm = ray_triangle_normal(a, b, c, st.o);
      if (HAS_POSE) nrm = pose_rotate(pose, nrm);
      normal_out[3 * (size_t)r + 0] = nrm.x;
      normal_out[3 * (size_t)r + 1] = nrm.y;
      normal_out[3 * (size_t)r + 2] = nrm.z;
    }
  } else {
    feat[r] = 0xffffffffu;
    toi_out[r] = 0.0f;
    if (WANT_NORMAL) {
      normal_out[3 * (size_t)r + 0] = 0.0f;
      normal_out[3 * (size_t)r + 1] = 0.0f;
      normal_out[3 * (size_t)r + 2] = 0.0f;
    }
  }
}

// One ray per thread: the whole traversal of ray order[k] (or k) in thread k.
template <bool HAS_POSE, bool WANT_NORMAL>
__global__ void k_trimesh_rays(const WideNode* __restrict__ wide, const float4* __restrict__ soup, uint32_t n_tris,
                               const float* __restrict__ rays, const uint32_t* __restrict__ order, uint32_t n, float max_toi,
                               Pose pose, uint32_t* __restrict__ feat, float* __restrict__ toi_out, float* __restrict__ normal_out,
                               uint32_t* __restrict__ err) {
  uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  uint32_t r = order ? order[k] : k;
  RayState st;
  ray_init<HAS_POSE>(rays, r, max_toi, pose, &st);
  WideNode w;
  load_wide(wide, 0, &w);
  if ((w.r.data & 0x3fffffffu) == 0u) {
    // Partial root (single triangle), bvh_traverse.rs:354-362.
    float s0 = slab(w.l.mins, w.l.maxs, st.o, st.inv, st.zmask, max_toi);
    if (s0 < max_toi) ray_try_leaf(soup, w.l.children, &st);
  } else {
    uint32_t stack[RAY_STACK];
    int sp = 0;
    for (;;) {
      uint32_t next = ray_step(w, soup, &st, stack, &sp, err);
      if (next == 0xffffffffu) break;
      load_wide(wide, next, &w);
    }
  }
  ray_finish<HAS_POSE, WANT_NORMAL>(soup, n_tris, pose, st, r, feat, toi_out, normal_out);
}

// Postponed leaves ("while-while" traversal): a lane that meets a leaf child keeps it (up to two)
// and goes on stepping through nodes while some lane of its warp has still found no leaf; then the
// whole warp tests its pending triangles together. Triangle tests - the divergent part of a step -
// run with most lanes active, at the price of node steps pruned by a best hit that is not yet
// lowered. A pending leaf is tested only if its box entry still passes the acceptance test of the
// moment; the answer (nearest hit, lowest index on exact ties) does not depend on the order.
template <bool HAS_POSE, bool WANT_NORMAL>
__global__ void k_trimesh_rays_ww(const WideNode* __restrict__ wide, const float4* __restrict__ soup, uint32_t n_tris,
                                  const float* __restrict__ rays, const uint32_t* __restrict__ order, uint32_t n, float max_toi, Pose pose,
                                  uint32_t* __restrict__ feat, float* __restrict__ toi_out, float* __restrict__ normal_out,
                                  uint32_t* __restrict__ err) {
  const unsigned FULL = 0xffffffffu;
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  const bool live = k < n;
  uint32_t r = 0;
  RayState st;
  uint32_t cur = 0xffffffffu;  // next wide node to step, none when ~0
  uint32_t p0 = 0xffffffffu, p1 = 0xffffffffu;  // pending leaves (soup positions)
  float e0 = 0.f, e1 = 0.f;                    // their box entries
  uint32_t stack[RAY_STACK];
  int sp = 0;
  if (live) {
    r = order ? order[k] : k;
    ray_init<HAS_POSE>(rays, r, max_toi, pose, &st);
    cur = 0;
  }
  auto accept = [&](float t) { return t != FLT_MAX && (t < st.best || (st.have && t == st.best)); };
  for (;;) {
    // node phase: step while some lane has nodes left and no pending leaf
    while (__any_sync(FULL, cur != 0xffffffffu && p0 == 0xffffffffu)) {
      if (cur == 0xffffffffu || p1 != 0xffffffffu) continue;  // nothing to step, or both leaf slots full
      WideNode w;
      load_wide(wide, cur, &w);
      float ls = slab(w.l.mins, w.l.maxs, st.o, st.inv, st.zmask, st.best);
      float rs = slab(w.r.mins, w.r.maxs, st.o, st.inv, st.zmask, st.best);
      const BvhNodeDev* nearn = &w.l;
      const BvhNodeDev* farn = &w.r;
      if (ls > rs) { float t = ls; ls = rs; rs = t; nearn = &w.r; farn = &w.l; }
      uint32_t next = 0xffffffffu;
      const float ts[2] = {ls, rs};
      const BvhNodeDev* cs[2] = {nearn, farn};
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        if (!accept(ts[c])) continue;
        if ((cs[c]->data & 0x3fffffffu) == 1u) {
          if (p0 == 0xffffffffu) { p0 = cs[c]->children; e0 = ts[c]; }
          else if (p1 == 0xffffffffu) { p1 = cs[c]->children; e1 = ts[c]; }
          else ray_try_leaf(soup, cs[c]->children, &st);  // third leaf of a speculative step: tested now
        } else if (next == 0xffffffffu) {
          next = cs[c]->children;
        } else if (sp >= RAY_STACK) {
          atomicOr(err, ERR_STACK_OVERFLOW);
          next = 0xffffffffu;
          sp = 0;
          break;
        } else {
          stack[sp++] = cs[c]->children;
        }
      }
      if (next == 0xffffffffu && sp > 0) next = stack[--sp];
      cur = next;
    }
    // leaf phase: every lane tests its pending triangles
    if (p0 != 0xffffffffu) {
      if (accept(e0)) ray_try_leaf(soup, p0, &st);
      p0 = 0xffffffffu;
    }
    if (p1 != 0xffffffffu) {
      if (accept(e1)) ray_try_leaf(soup, p1, &st);
      p1 = 0xffffffffu;
    }
    if (!__any_sync(FULL, cur != 0xffffffffu)) break;
  }
  if (live) ray_finish<HAS_POSE, WANT_NORMAL>(soup, n_tris, pose, st, r, feat, toi_out, normal_out);
}

// Persistent warps with dynamic ray fetch: every lane runs one traversal step per loop turn, and
// once at least `refill` lanes of the warp have finished their rays, the warp takes that many new
// ray slots from a global counter with one atomicAdd. Lanes whose rays end early pick up new rays
// instead of idling until the warp's longest traversal ends. The per-ray work and answers are
// those of k_trimesh_rays. Requires a non-leaf root (two or more triangles).
template <bool HAS_POSE, bool WANT_NORMAL>
__global__ void __launch_bounds__(128) k_trimesh_rays_fetch(const WideNode* __restrict__ wide, const float4* __restrict__ soup,
                                                            uint32_t n_tris, const float* __restrict__ rays,
                                                            const uint32_t* __restrict__ order, uint32_t n, float max_toi, Pose pose,
                                                            uint32_t* __restrict__ feat, float* __restrict__ toi_out,
                                                            float* __restrict__ normal_out, uint32_t* __restrict__ err,
                                                            uint32_t* __restrict__ next_ray, uint32_t refill) {
  const unsigned FULL = 0xffffffffu;
  const uint32_t lane = threadIdx.x & 31u;
  uint32_t stack[RAY_STACK];
  int sp = 0;
  bool active = false, exhausted = false;
  uint32_t r = 0, cur = 0;
  RayState st;
  for (;;) {
    const unsigned idle = __ballot_sync(FULL, !active);
    const uint32_t n_idle = (uint32_t)__popc(idle);
    if (!exhausted && n_idle >= refill) {  // warp-uniform
      uint32_t base = 0;
      if (lane == 0) base = atomicAdd(next_ray, n_idle);
      base = __shfl_sync(FULL, base, 0);
      if (base >= n || n - base <= n_idle) exhausted = true;
      if (!active) {
        uint32_t k = base + (uint32_t)__popc(idle & ((1u << lane) - 1u));
        if (k < n) {
          r = order ? order[k] : k;
          ray_init<HAS_POSE>(rays, r, max_toi, pose, &st);
          sp = 0;
          cur = 0;
          active = true;
        }
      }
    }
    if (__ballot_sync(FULL, active) == 0u) break;  // only once the counter is exhausted
    if (active) {
      WideNode w;
      load_wide(wide, cur, &w);
      cur = ray_step(w, soup, &st, stack, &sp, err);
      if (cur == 0xffffffffu) {
        ray_finish<HAS_POSE, WANT_NORMAL>(soup, n_tris, pose, st, r, feat, toi_out, normal_out);
        active = false;
      }
    }
  }
}

__global__ void k_tri_aabbs(const float* __restrict__ verts, const uint32_t* __restrict__ idx, uint32_t nt, uint32_t nv,
                            float* __restrict__ aabbs, uint32_t* __restrict__ err) {
  uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt) return;
  uint32_t i0 = idx[3 * (size_t)t], i1 = idx[3 * (size_t)t + 1], i2 = idx[3 * (size_t)t + 2];
  if (i0 >= nv || i1 >= nv || i2 >= nv) { atomicOr(err, ERR_CAPACITY); i0 = i1 = i2 = 0; }
  float* out = aabbs + 6 * (size_t)t;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    float a = verts[3 * (size_t)i0 + d], b = verts[3 * (size_t)i1 + d], c = verts[3 * (size_t)i2 + d];
    // aabb_triangle.rs:25-27: a.min(b).min(c), a.max(b).max(c)
    out[d] = fminf(fminf(a, b), c);
    out[3 + d] = fmaxf(fmaxf(a, b), c);
  }
}

__global__ void k_tri_soup(const float* __restrict__ verts, const uint32_t* __restrict__ idx, const uint32_t* __restrict__ leaf_index,
                           uint32_t nt, uint32_t nv, float4* __restrict__ soup) {
  uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nt) return;
  uint32_t t = leaf_index[p];
  uint32_t i0 = idx[3 * (size_t)t], i1 = idx[3 * (size_t)t + 1], i2 = idx[3 * (size_t)t + 2];
  if (i0 >= nv || i1 >= nv || i2 >= nv) i0 = i1 = i2 = 0;
  const float* a = verts + 3 * (size_t)i0;
  const float* b = verts + 3 * (size_t)i1;
  const float* c = verts + 3 * (size_t)i2;
  soup[3 * (size_t)p + 0] = make_float4(a[0], a[1], a[2], b[0]);
  soup[3 * (size_t)p + 1] = make_float4(b[1], b[2], c[0], c[1]);
  soup[3 * (size_t)p + 2] = make_float4(c[2], __uint_as_float(t), 0.0f, 0.0f);
}

// Bounds of the ray origins: warp shuffles, then a shared-memory reduction, then one atomic per
// block and component (order-preserving float encoding).
__global__ void __launch_bounds__(256) k_ray_bounds(const float* __restrict__ rays, uint32_t n, uint32_t* __restrict__ bounds) {
  __shared__ float smn[3][8], smx[3][8];
  float mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, mx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      float v = rays[6 * (size_t)i + d];
      mn[d] = fminf(mn[d], v);
      mx[d] = fmaxf(mx[d], v);
    }
  }
#pragma unroll
  for (int d = 0; d < 3; ++d) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      mn[d] = fminf(mn[d], __shfl_xor_sync(0xffffffffu, mn[d], o));
      mx[d] = fmaxf(mx[d], __shfl_xor_sync(0xffffffffu, mx[d], o));
    }
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) {
#pragma unroll
    for (int d = 0; d < 3; ++d) { smn[d][w] = mn[d]; smx[d][w] = mx[d]; }
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    int d = threadIdx.x;
    float a = smn[d][0], b = smx[d][0];
    for (int k = 1; k < (int)(blockDim.x >> 5); ++k) { a = fminf(a, smn[d][k]); b = fmaxf(b, smx[d][k]); }
    atomicMin(&bounds[d], float_flip(a));
    atomicMax(&bounds[3 + d], float_flip(b));
  }
}

__global__ void k_ray_keys(const float* __restrict__ rays, uint32_t n, const uint32_t* __restrict__ bounds, uint32_t* __restrict__ keys,
                           uint32_t* __restrict__ vals, uint32_t key_mode) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float ext = 0.0f;  // one scale for all axes: cubic Morton cells
#pragma unroll
  for (int d = 0; d < 3; ++d) ext = fmaxf(ext, float_unflip(bounds[3 + d]) - float_unflip(bounds[d]));
  float u[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) u[d] = ext > 0.0f ? (rays[6 * (size_t)i + d] - float_unflip(bounds[d])) / ext : 0.5f;
  uint32_t key = morton30(u[0], u[1], u[2]);
  if (key_mode == 1) {
    const float* d = rays + 6 * (size_t)i + 3;
    uint32_t oct = (d[0] < 0.0f ? 4u : 0u) | (d[1] < 0.0f ? 2u : 0u) | (d[2] < 0.0f ? 1u : 0u);
    key = (oct << 27) | (key >> 3);
  } else if (key_mode == 2) {
    key >>= 14;  // the top 16 bits of the Morton code: a two-pass sort
  } else if (key_mode == 3) {
    // direction class: octant and dominant axis (5 bits) above the top 25 bits of the Morton code
    const float* d = rays + 6 * (size_t)i + 3;
    const uint32_t oct = (d[0] < 0.0f ? 4u : 0u) | (d[1] < 0.0f ? 2u : 0u) | (d[2] < 0.0f ? 1u : 0u);
    const float ax = fabsf(d[0]), ay = fabsf(d[1]), az = fabsf(d[2]);
    const uint32_t dom = (ax >= ay && ax >= az) ? 0u : (ay >= az ? 1u : 2u);
    key = ((oct * 3u + dom) << 25) | (key >> 5);
  }
  keys[i] = key;
  vals[i] = i;
}

}  // namespace

extern "C" {

parrygpu_status parrygpu_trimesh_create(parrygpu_ctx* ctx, const float* vertices, uint32_t n_vertices, const uint32_t* indices,
                                        uint32_t n_triangles, parrygpu_trimesh** out) {
  if (!ctx || !out) return PARRYGPU_INVALID_ARG;
  *out = nullptr;
  if (n_triangles > 0 && (!vertices || !indices || n_vertices == 0))
    return set_error(ctx, PARRYGPU_INVALID_ARG, "trimesh needs vertices and indices");
  PG_CUDA(ctx, cudaSetDevice(ctx->device));
  const void* dv = nullptr;
  const void* di = nullptr;
  parrygpu_status s = stage_input(ctx, ctx->stage_in[0], vertices, (size_t)n_vertices * 12, &dv);
  if (s != PARRYGPU_OK) return s;
  s = stage_input(ctx, ctx->stage_in[1], indices, (size_t)n_triangles * 12, &di);
  if (s != PARRYGPU_OK) return s;
  parrygpu_trimesh* m = new parrygpu_trimesh();
  m->n_vertices = n_vertices;
  m->n_triangles = n_triangles;
  if (n_triangles > 0) {
    DevBuf aabbs;
    cudaError_t e = aabbs.reserve((size_t)n_triangles * 24);
    if (e == cudaSuccess) e = m->soup.reserve((size_t)n_triangles * 48);
    if (e != cudaSuccess) { aabbs.release(); parrygpu_trimesh_destroy(m); return check_cuda(ctx, e, "trimesh alloc"); }
    k_tri_aabbs<<<div_up(n_triangles, 256), 256, 0, ctx->stream>>>((const float*)dv, (const uint32_t*)di, n_triangles, n_vertices,
                                                                   aabbs.as<float>(), ctx->d_err);
    ctx->launches++;
    s = lbvh_build(ctx, &m->bvh, aabbs.as<float>(), n_triangles, true);
    if (s == PARRYGPU_OK) {
      k_tri_soup<<<div_up(n_triangles, 256), 256, 0, ctx->stream>>>((const float*)dv, (const uint32_t*)di, m->bvh.leaf_index.as<uint32_t>(),
                                                                     n_triangles, n_vertices, m->soup.as<float4>());
      ctx->launches++;
    }
    cudaError_t se = cudaStreamSynchronize(ctx->stream);
    aabbs.release();
    if (s != PARRYGPU_OK) { parrygpu_trimesh_destroy(m); return s; }
    if (se != cudaSuccess) { parrygpu_trimesh_destroy(m); return check_cuda(ctx, se, "trimesh build"); }
    s = parrygpu_sync(ctx);
    if (s != PARRYGPU_OK) {
      parrygpu_trimesh_destroy(m);
      return set_error(ctx, PARRYGPU_INVALID_ARG, "triangle index out of range of the vertex buffer");
    }
  }
  *out = m;
  return PARRYGPU_OK;
}

void parrygpu_trimesh_destroy(parrygpu_trimesh* m) {
  if (!m) return;
  for (DevBuf* d : {&m->bvh.wide, &m->bvh.leaf_parent, &m->bvh.node_parent, &m->bvh.leaf_index, &m->bvh.flags, &m->bvh.root_aabb,
                    &m->bvh.info, &m->soup, &m->pseudo, &m->pseudo_ok})
    d->release();
  delete m;
}

// Host-buffer calls without a ray ordering run in chunks alternating between the context stream
// and a second stream: the host<->device copies of one chunk overlap the traversal of the other
// (each chunk's upload, traversal and download stay in order on its stream). Answers are those of
// the single-shot call: every ray is independent.
constexpr uint32_t PIPE_MIN_CHUNK = 65536;

static parrygpu_status cast_rays_pipelined(parrygpu_ctx* ctx, const parrygpu_trimesh* mesh, const float* pose_host, const float* rays,
                                           uint32_t n, float max_toi, uint32_t* feature, float* toi, float* normal, bool host_in,
                                           bool h_feat, bool h_toi, bool h_nrm) {
  if (!ctx->aux_stream) {
    PG_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->aux_stream, cudaStreamNonBlocking));
    PG_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming));
    PG_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming));
  }
  const float* d_rays = rays;
  uint32_t* d_feat = feature;
  float *d_toi = toi, *d_nrm = normal;
  if (host_in) { PG_CUDA(ctx, ctx->stage_in[2].reserve((size_t)n * 24)); d_rays = ctx->stage_in[2].as<float>(); }
  if (h_feat) { PG_CUDA(ctx, ctx->stage_out[1].reserve((size_t)n * 4)); d_feat = ctx->stage_out[1].as<uint32_t>(); }
  if (h_toi) { PG_CUDA(ctx, ctx->stage_out[2].reserve((size_t)n * 4)); d_toi = ctx->stage_out[2].as<float>(); }
  if (h_nrm) { PG_CUDA(ctx, ctx->stage_out[3].reserve((size_t)n * 12)); d_nrm = ctx->stage_out[3].as<float>(); }
  PG_CUDA(ctx, ctx->misc.reserve(128));
  uint32_t* counters = ctx->misc.as<uint32_t>() + 16;  // one fetch counter per stream
  cudaStream_t main = ctx->stream;
  cudaStream_t lanes[2] = {main, ctx->aux_stream};
  PG_CUDA(ctx, cudaEventRecord(ctx->ev_fork, main));
  PG_CUDA(ctx, cudaStreamWaitEvent(ctx->aux_stream, ctx->ev_fork, 0));
  // Every chunk costs about 40 us of host-side issue (measured on GB300: 1M rays in 0.78 ms unchunked,
  // 0.67 ms in 2 or 4 chunks, 0.77 / 1.12 / 1.78 ms in 8 / 16 / 32): by default 2 to 4 chunks of at
  // least 262,144 rays.
  uint32_t chunks = ctx->cfg.ray_chunks;
  if (chunks == 0) {
    chunks = n / (4 * PIPE_MIN_CHUNK);
    if (chunks > 4) chunks = 4;
    if (chunks < 2) chunks = 2;
  }
  const uint32_t chunk = ((n + chunks - 1) / chunks + 255u) & ~255u;
  parrygpu_status s = PARRYGPU_OK;
  cudaError_t e = cudaSuccess;
  for (uint32_t c = 0, off = 0; off < n && s == PARRYGPU_OK && e == cudaSuccess; ++c, off += chunk) {
    const uint32_t m = n - off < chunk ? n - off : chunk;
    cudaStream_t st = lanes[c & 1];
    ctx->stream = st;
    if (host_in) e = cudaMemcpyAsync((void*)(d_rays + 6 * (size_t)off), rays + 6 * (size_t)off, (size_t)m * 24, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
      s = launch_trimesh_rays(ctx, mesh, pose_host, d_rays + 6 * (size_t)off, nullptr, m, max_toi, d_feat + off, d_toi + off,
                              d_nrm ? d_nrm + 3 * (size_t)off : nullptr, counters + (c & 1));
    if (s == PARRYGPU_OK && e == cudaSuccess && h_feat) e = cudaMemcpyAsync(feature + off, d_feat + off, (size_t)m * 4, cudaMemcpyDeviceToHost, st);
    if (s == PARRYGPU_OK && e == cudaSuccess && h_toi) e = cudaMemcpyAsync(toi + off, d_toi + off, (size_t)m * 4, cudaMemcpyDeviceToHost, st);
    if (s == PARRYGPU_OK && e == cudaSuccess && h_nrm)
      e = cudaMemcpyAsync(normal + 3 * (size_t)off, d_nrm + 3 * (size_t)off, (size_t)m * 12, cudaMemcpyDeviceToHost, st);
  }
  ctx->stream = main;
  cudaError_t je = cudaEventRecord(ctx->ev_join, ctx->aux_stream);
  if (je == cudaSuccess) je = cudaStreamWaitEvent(main, ctx->ev_join, 0);
  if (s != PARRYGPU_OK) return s;
  if (e != cudaSuccess) return check_cuda(ctx, e, "pipelined ray cast");
  if (je != cudaSuccess) return check_cuda(ctx, je, "pipelined ray cast join");
  return parrygpu_sync(ctx);
}

parrygpu_status parrygpu_trimesh_cast_rays(parrygpu_ctx* ctx, const parrygpu_trimesh* mesh, const float* pose7, const float* rays,
                                           uint32_t n, float max_toi, int solid, uint32_t* feature, float* toi, float* normal) {
  (void)solid;
  if (!ctx || !mesh) return PARRYGPU_INVALID_ARG;
  if (n == 0) return PARRYGPU_OK;
  if (!rays || !feature || !toi) return set_error(ctx, PARRYGPU_INVALID_ARG, "rays, feature and toi are required");
  PG_CUDA(ctx, cudaSetDevice(ctx->device));
  Pose pose{0.f, 0.f, 0.f, 1.f, v3(0.f, 0.f, 0.f)};
  bool has_pose = pose7 != nullptr;
  if (has_pose) {
    float p[7];
    if (is_device_ptr(pose7)) {
      PG_CUDA(ctx, cudaMemcpyAsync(p, pose7, 28, cudaMemcpyDeviceToHost, ctx->stream));
      PG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    } else {
      for (int i = 0; i < 7; ++i) p[i] = pose7[i];
    }
    pose = Pose{p[0], p[1], p[2], p[3], v3(p[4], p[5], p[6])};
  }
  {
    const bool host_in = !is_device_ptr(rays), h_feat = !is_device_ptr(feature), h_toi = !is_device_ptr(toi);
    const bool h_nrm = normal && !is_device_ptr(normal);
    const bool in_place = ctx->cfg.ray_host_access == 1 || (ctx->cfg.ray_host_access == 0 && ctx->coherent_host);
    if ((host_in || h_feat || h_toi || h_nrm) && mesh->n_triangles > 0 && !ctx->cfg.sort_rays && in_place &&
        is_addressable(rays) && is_addressable(feature) && is_addressable(toi) && (!normal || is_addressable(normal))) {
      // every buffer is device memory or page-locked host memory the device addresses in place:
      // the traversal reads the rays and writes its results over the host link, no staging copies
      PG_CUDA(ctx, ctx->misc.reserve(128));
      float p7[7] = {pose.qi, pose.qj, pose.qk, pose.qw, pose.t.x, pose.t.y, pose.t.z};
      KernelTimer kt(ctx, "trimesh_rays");
      parrygpu_status s = launch_trimesh_rays(ctx, mesh, has_pose ? p7 : nullptr, device_view(rays), nullptr, n, max_toi,
                                              device_view(feature), device_view(toi), normal ? device_view(normal) : nullptr,
                                              ctx->misc.as<uint32_t>() + 16);
      kt.stop();
      if (s != PARRYGPU_OK) return s;
      return parrygpu_sync(ctx);
    }
    if ((host_in || h_feat || h_toi || h_nrm) && mesh->n_triangles > 0 && !ctx->cfg.sort_rays && ctx->cfg.ray_chunks != 1 &&
        n >= 2 * PIPE_MIN_CHUNK) {
      float p7[7] = {pose.qi, pose.qj, pose.qk, pose.qw, pose.t.x, pose.t.y, pose.t.z};
      return cast_rays_pipelined(ctx, mesh, has_pose ? p7 : nullptr, rays, n, max_toi, feature, toi, normal, host_in, h_feat, h_toi, h_nrm);
    }
  }
  const void* d_rays = nullptr;
  parrygpu_status s = stage_input(ctx, ctx->stage_in[2], rays, (size_t)n * 24, &d_rays);
  if (s != PARRYGPU_OK) return s;
  void *d_feat, *d_toi, *d_nrm;
  bool c_feat, c_toi, c_nrm;
  if ((s = stage_output(ctx, ctx->stage_out[1], feature, (size_t)n * 4, &d_feat, &c_feat)) != PARRYGPU_OK) return s;
  if ((s = stage_output(ctx, ctx->stage_out[2], toi, (size_t)n * 4, &d_toi, &c_toi)) != PARRYGPU_OK) return s;
  if ((s = stage_output(ctx, ctx->stage_out[3], normal, (size_t)n * 12, &d_nrm, &c_nrm)) != PARRYGPU_OK) return s;

  if (mesh->n_triangles == 0) {
    PG_CUDA(ctx, cudaMemsetAsync(d_feat, 0xff, (size_t)n * 4, ctx->stream));
    PG_CUDA(ctx, cudaMemsetAsync(d_toi, 0, (size_t)n * 4, ctx->stream));
    if (d_nrm) PG_CUDA(ctx, cudaMemsetAsync(d_nrm, 0, (size_t)n * 12, ctx->stream));
  } else {
    const uint32_t* order = nullptr;
    if (ctx->cfg.sort_rays && n > 4096) {
      s = radix_sort_reserve(ctx, n);
      if (s != PARRYGPU_OK) return s;
      PG_CUDA(ctx, ctx->misc.reserve(64));
      uint32_t* bounds = ctx->misc.as<uint32_t>() + 8;
      PG_CUDA(ctx, cudaMemsetAsync(bounds, 0xff, 12, ctx->stream));
      PG_CUDA(ctx, cudaMemsetAsync(bounds + 3, 0x00, 12, ctx->stream));
      k_ray_bounds<<<div_up(n, 256 * 8), 256, 0, ctx->stream>>>((const float*)d_rays, n, bounds);
      PG_LAUNCHED(ctx);
      k_ray_keys<<<div_up(n, 256), 256, 0, ctx->stream>>>((const float*)d_rays, n, bounds, ctx->sort_k[0].as<uint32_t>(),
                                                          ctx->sort_v[0].as<uint32_t>(), ctx->cfg.ray_sort_key);
      PG_LAUNCHED(ctx);
      int rb;
      KernelTimer kt(ctx, "ray_sort");
      s = radix_sort_pairs(ctx, n, ray_sort_bits(ctx), &rb);
      kt.stop();
      if (s != PARRYGPU_OK) return s;
      order = ctx->sort_v[rb].as<uint32_t>();
    }
    PG_CUDA(ctx, ctx->misc.reserve(128));
    float p7[7] = {pose.qi, pose.qj, pose.qk, pose.qw, pose.t.x, pose.t.y, pose.t.z};
    KernelTimer kt(ctx, "trimesh_rays");
    s = launch_trimesh_rays(ctx, mesh, has_pose ? p7 : nullptr, (const float*)d_rays, order, n, max_toi, (uint32_t*)d_feat, (float*)d_toi,
                            (float*)d_nrm, ctx->misc.as<uint32_t>() + 16);
    kt.stop();
    if (s != PARRYGPU_OK) return s;
  }
  if (c_feat) PG_CUDA(ctx, cudaMemcpyAsync(feature, d_feat, (size_t)n * 4, cudaMemcpyDeviceToHost, ctx->stream));
  if (c_toi) PG_CUDA(ctx, cudaMemcpyAsync(toi, d_toi, (size_t)n * 4, cudaMemcpyDeviceToHost, ctx->stream));
  if (c_nrm) PG_CUDA(ctx, cudaMemcpyAsync(normal, d_nrm, (size_t)n * 12, cudaMemcpyDeviceToHost, ctx->stream));
  if (c_feat || c_toi || c_nrm || d_rays != rays) return parrygpu_sync(ctx);
  return PARRYGPU_OK;
}

}  // extern "C"

// Launches the ray-ordering keys (origin bounds into `bounds`, 6 words, then Morton keys) on
// caller-provided device buffers. Allocates nothing.
parrygpu_status launch_ray_keys(parrygpu_ctx* ctx, const float* d_rays, uint32_t n, uint32_t* bounds, uint32_t* keys, uint32_t* vals,
                                uint32_t key_mode) {
  PG_CUDA(ctx, cudaMemsetAsync(bounds, 0xff, 12, ctx->stream));
  PG_CUDA(ctx, cudaMemsetAsync(bounds + 3, 0x00, 12, ctx->stream));
  k_ray_bounds<<<div_up(n, 256 * 8), 256, 0, ctx->stream>>>(d_rays, n, bounds);
  PG_LAUNCHED(ctx);
  k_ray_keys<<<div_up(n, 256), 256, 0, ctx->stream>>>(d_rays, n, bounds, keys, vals, key_mode);
  PG_LAUNCHED(ctx);
  return PARRYGPU_OK;
}

// Launches the traversal kernel of the context's configuration on device buffers (order may be
// NULL; `counter` = one device word for the dynamic-fetch traversal's ray counter, zeroed here).
// Allocates nothing.
parrygpu_status launch_trimesh_rays(parrygpu_ctx* ctx, const parrygpu_trimesh* mesh, const float* pose7_host, const float* d_rays,
                                    const uint32_t* order, uint32_t n, float max_toi, uint32_t* d_feat, float* d_toi, float* d_nrm,
                                    uint32_t* counter) {
  Pose pose{0.f, 0.f, 0.f, 1.f, v3(0.f, 0.f, 0.f)};
  bool has_pose = pose7_host != nullptr;
  if (has_pose) pose = Pose{pose7_host[0], pose7_host[1], pose7_host[2], pose7_host[3], v3(pose7_host[4], pose7_host[5], pose7_host[6])};
  const WideNode* w = mesh->bvh.wide.as<WideNode>();
  const float4* soup = mesh->soup.as<float4>();
  // the fetch traversal needs an internal root (two or more triangles) and headroom in its counter
  if (ctx->cfg.ray_traversal == 2 && mesh->n_triangles >= 2 && n <= 0xF0000000u) {
    uint32_t refill = ctx->cfg.ray_refill ? ctx->cfg.ray_refill : 16;
    auto kern = has_pose ? (d_nrm ? k_trimesh_rays_fetch<true, true> : k_trimesh_rays_fetch<true, false>)
                         : (d_nrm ? k_trimesh_rays_fetch<false, true> : k_trimesh_rays_fetch<false, false>);
    int per_sm = 0;
    PG_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 128, 0));
    if (per_sm < 1) per_sm = 1;
    uint32_t blocks = (uint32_t)(ctx->sm_count > 0 ? ctx->sm_count : 152) * (uint32_t)per_sm;
    uint32_t need = div_up(n, 128);
    if (blocks > need) blocks = need;
    PG_CUDA(ctx, cudaMemsetAsync(counter, 0, 4, ctx->stream));
    kern<<<blocks, 128, 0, ctx->stream>>>(w, soup, mesh->n_triangles, d_rays, order, n, max_toi, pose, d_feat, d_toi, d_nrm, ctx->d_err,
                                          counter, refill);
    PG_LAUNCHED(ctx);
    return PARRYGPU_OK;
  }
  uint32_t bs = ctx->cfg.ray_block ? ctx->cfg.ray_block : 128;
  if (ctx->cfg.ray_traversal == 3 && mesh->n_triangles >= 2) {
    auto kern = has_pose ? (d_nrm ? k_trimesh_rays_ww<true, true> : k_trimesh_rays_ww<true, false>)
                         : (d_nrm ? k_trimesh_rays_ww<false, true> : k_trimesh_rays_ww<false, false>);
    kern<<<div_up(n, bs), bs, 0, ctx->stream>>>(w, soup, mesh->n_triangles, d_rays, order, n, max_toi, pose, d_feat, d_toi, d_nrm,
                                                ctx->d_err);
    PG_LAUNCHED(ctx);
    return PARRYGPU_OK;
  }
  auto kern = has_pose ? (d_nrm ? k_trimesh_rays<true, true> : k_trimesh_rays<true, false>)
                       : (d_nrm ? k_trimesh_rays<false, true> : k_trimesh_rays<false, false>);
  kern<<<div_up(n, bs), bs, 0, ctx->stream>>>(w, soup, mesh->n_triangles, d_rays, order, n, max_toi, pose, d_feat, d_toi, d_nrm, ctx->d_err);
  PG_LAUNCHED(ctx);
  return PARRYGPU_OK;
}
