// Batched ray casts against a shape set (the reference's Compound: parts with poses under one BVH).
//
// Per ray: best-first descent of Bvh::find_best (src/partitioning/bvh/bvh_traverse.rs:335-417)
// over the LBVH of the parts' world AABBs, leaf cost = the part's RayCast::cast_ray_and_get_normal
// (ray moved into the part frame, src/query/ray/ray.rs:393-403) with max_toi = best so far:
//   ball      src/query/ray/ray_ball.rs:33-98
//   cuboid    src/query/ray/ray_cuboid.rs:6-25 -> ray_aabb.rs:51-92 -> clip/clip_aabb_line.rs:79-185
//   capsule, convex polyhedron
//             src/query/ray/ray_support_map.rs:19-71 -> gjk.rs:519-534, 660-795 (GJK ray cast)
//   triangle  src/query/ray/ray_triangle.rs:49-152
// Compound semantics: src/query/ray/ray_composite_shape.rs:86-105, src/shape/compound.rs:113-144.
// Exact toi ties resolve to the lowest part index (as for triangle meshes).
#include "internal.hpp"
#include "gjk_device.cuh"
#include "lbvh_device.cuh"
#include "gjk_reg.cuh"

#include <cooperative_groups.h>
#include <algorithm>
#include <cmath>

using namespace pg;

namespace {

constexpr int CRAY_STACK = 64;

__device__ __forceinline__ bool ray_ball(float r, V3 o, V3 d, bool solid, float max_toi, float* toi, V3* n) {
  float a = dot(d, d), b = dot(o, d), c = dot(o, o) - r * r;
  bool inside;
  float t;
  if (a == 0.0f) {
    if (c > 0.0f) return false;
    inside = true; t = 0.0f;
  } else {
    if (c > 0.0f && b > 0.0f) return false;
    float delta = b * b - a * c;
    if (delta < 0.0f) return false;
    t = (-b - sqrtf(delta)) / a;
    if (t <= 0.0f) { inside = true; t = solid ? 0.0f : (-b + sqrtf(delta)) / a; }
    else inside = false;
  }
  V3 nn = normalize(o + d * t);
  if (!(t <= max_toi)) return false;
  *toi = t;
  *n = inside ? -nn : nn;
  return true;
}

__device__ __forceinline__ float cmp3(V3 v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }

// clip_aabb_line + ray_aabb on [-h, h]
__device__ __forceinline__ bool ray_cuboid(V3 h, V3 o, V3 d, bool solid, float max_toi, float* toi, V3* n) {
  float tmax = FLT_MAX, tmin = -FLT_MAX;
  int near_side = 0, far_side = 0;
  bool near_diag = false, far_diag = false;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    float di = cmp3(d, i), oi = cmp3(o, i), hi = cmp3(h, i);
    if (di == 0.0f) {
      if (oi < -hi || oi > hi) return false;
    } else {
      float denom = 1.0f / di;
      float a = (-hi - oi) * denom, b = (hi - oi) * denom;
      bool flip = a > b;
      if (flip) { float s = a; a = b; b = s; }
      if (a > tmin) { tmin = a; near_side = flip ? -(i + 1) : (i + 1); near_diag = false; }
      else if (a == tmin) near_diag = true;
      if (b < tmax) { tmax = b; far_side = !flip ? -(i + 1) : (i + 1); far_diag = false; }
      else if (b == tmax) far_diag = true;
      if (tmax < 0.0f || tmin > tmax) return false;
    }
  }
  float tn, tf;
  V3 nn, nf;
  bool contains = !(o.x < -h.x || o.x > h.x || o.y < -h.y || o.y > h.y || o.z < -h.z || o.z > h.z);
  bool degenerate = false;
  if (near_diag) { tn = tmin; nn = -normalize(d); }
  else if (near_side == 0) { degenerate = true; }
  else {
    float c[3] = {0.f, 0.f, 0.f};
    if (near_side < 0) c[-near_side - 1] = 1.0f; else c[near_side - 1] = -1.0f;
    tn = tmin; nn = v3(c[0], c[1], c[2]);
  }
  if (!degenerate) {
    if (far_diag) { tf = tmax; nf = -normalize(d); }
    else if (far_side == 0) { degenerate = true; }
    else {
      float c[3] = {0.f, 0.f, 0.f};
      if (far_side < 0) c[-far_side - 1] = -1.0f; else c[far_side - 1] = 1.0f;
      tf = tmax; nf = v3(c[0], c[1], c[2]);
    }
  }
  if (degenerate) {
    if (!contains) return false;
    tn = 0.0f; nn = v3(0.f, 0.f, 0.f); tf = 0.0f; nf = nn;
  }
  if (tn < 0.0f) {
    if (solid) { *toi = 0.0f; *n = v3(0.f, 0.f, 0.f); return true; }
    if (tf <= max_toi) { *toi = tf; *n = nf; return true; }
    return false;
  }
  if (tn <= max_toi) { *toi = tn; *n = nn; return true; }
  return false;
}

__device__ __forceinline__ bool ray_halfspace(V3 center, V3 normal, V3 o, V3 d, float* t) {
  V3 dpos = center - o;
  float denom = dot(normal, d);
  if (fabsf(denom) <= EPS) return false;
  float tt = dot(normal, dpos) / denom;
  if (tt >= 0.0f) { *t = tt; return true; }
  return false;
}

// gjk.rs:660-795 minkowski_ray_cast with the identity pose and the constant origin.
__device__ __noinline__ bool gjk_cast_local_ray(const ShapeDev& shape, V3 ro, V3 rd, float max_toi, float* toi_out, V3* n_out) {
  const float eps_tol = GJK_EPS_TOL;
  const float eps_rel = sqrtf(eps_tol);
  float ray_length = norm(rd);
  if (fabsf(ray_length) <= EPS) return false;
  float ltoi = 0.0f;
  V3 co = ro, cd = rd / ray_length;
  V3 dir = -cd;
  V3 ldir = dir;
  Pose id{0.f, 0.f, 0.f, 1.f, v3(0.f, 0.f, 0.f)};
  ShapeDev origin;
  origin.type = SH_ORIGIN;
  Simplex s;
  CSO sp = cso_from_shapes(id, shape, origin, dir);
  simplex_reset(s, CSO{sp.p - co, sp.o1, sp.o2});
  V3 proj = simplex_project_origin_and_reduce(s);
  float max_bound = FLT_MAX;
  int niter = 0;
  bool last_chance = false;
  for (;;) {
    float old_max_bound = max_bound;
    float nb;
    V3 u;
    if (try_normalize(-proj, eps_tol, &u, &nb)) { dir = u; max_bound = nb; }
    else { *toi_out = ltoi / ray_length; *n_out = ldir; return true; }
    CSO support;
    if (max_bound >= old_max_bound) {
      last_chance = true;
      V3 p = proj + co;
      support = CSO{p, p, v3(0.f, 0.f, 0.f)};
    } else {
      support = cso_from_shapes(id, shape, origin, dir);
    }
    if (last_chance && ltoi > 0.0f) { *toi_out = ltoi / ray_length; *n_out = ldir; return true; }
    float t;
    if (ray_halfspace(support.p, dir, co, cd, &t)) {
      if (dot(dir, cd) < 0.0f && t > 0.0f) {
        ldir = dir;
        ltoi += t;
        if (ltoi / ray_length > max_toi) return false;
        V3 shift = cd * t;
        co = co + shift;
        max_bound = FLT_MAX;
        for (int i = 0; i <= s.dim; ++i) s.v[i].p = s.v[i].p + (-shift);
        last_chance = false;
      }
    } else {
      if (dot(dir, cd) > eps_tol) return false;
    }
    if (last_chance) return false;
    float min_bound = -dot(dir, support.p - co);
    if (max_bound - min_bound <= eps_rel * max_bound) return false;
    simplex_add(s, CSO{support.p - co, support.o1, support.o2});
    proj = simplex_project_origin_and_reduce(s);
    if (s.dim == 3) {
      if (min_bound >= eps_tol) return false;
      *toi_out = ltoi / ray_length; *n_out = ldir; return true;
    }
    niter += 1;
    if (niter == 100) return false;
  }
}

// ray_support_map.rs:19-71
__device__ __forceinline__ bool ray_support_map(const ShapeDev& shape, V3 o, V3 d, bool solid, float max_toi, float* toi, V3* n) {
  float t;
  V3 nn;
  if (!gjk_cast_local_ray(shape, o, d, max_toi, &t, &nn)) return false;
  if (solid || t != 0.0f) { *toi = t; *n = nn; return true; }
  V3 ndir = normalize(d);
  V3 supp = local_support(shape, ndir);
  float eps = 0.001f;
  float shift = dot(supp - o, ndir) + eps;
  float t2;
  V3 n2;
  if (!gjk_cast_local_ray(shape, o + ndir * shift, -d, shift + eps, &t2, &n2)) return false;
  float tt = shift - t2;
  if (!(tt <= max_toi)) return false;
  *toi = tt;
  *n = -n2;
  return true;
}

// ---- the GJK ray cast with its simplex in registers, for one support-map kind ----
// gjk_cast_local_ray keeps its Voronoi simplex in an array indexed at run time (local memory, and
// witness points the ray cast never reads). The candidate kernels run one shape kind per launch,
// so the cast below is inlined with that kind's support function over a positions-only
// RegSimplex (gjk_reg.cuh); every value is computed as in gjk_cast_local_ray, so the answers are
// the same.
// Support of one kind: TY = SH_CAPSULE (O(1)) or SH_CONVEX (vertex scan).
template <uint32_t TY>
__device__ __forceinline__ V3 kind_support(const ShapeDev& s, V3 dir) {
  if constexpr (TY == SH_CAPSULE) {
    V3 d;
    if (!try_normalize(dir, 0.0f, &d)) d = v3(0.f, 1.f, 0.f);
    V3 a = v3(0.f, -s.a, 0.f), b = v3(0.f, s.a, 0.f);
    if (dot(d, a) > dot(d, b)) return a + d * s.b;
    return b + d * s.b;
  } else {
    return convex_support(s.pts, s.npts, dir);
  }
}

// gjk.rs:660-795 minkowski_ray_cast, as gjk_cast_local_ray, for one support kind.
template <uint32_t TY>
__device__ __forceinline__ bool gjk_cast_local_ray_kind(const ShapeDev& shape, V3 ro, V3 rd, float max_toi, float* toi_out, V3* n_out) {
  const float eps_tol = GJK_EPS_TOL;
  const float eps_rel = sqrtf(eps_tol);
  float ray_length = norm(rd);
  if (fabsf(ray_length) <= EPS) return false;
  float ltoi = 0.0f;
  V3 co = ro, cd = rd / ray_length;
  V3 dir = -cd;
  V3 ldir = dir;
  RegSimplex<false> s;
  {
    const V3 sp = kind_support<TY>(shape, dir) - co;
    rs_reset(s, CSO{sp, sp, sp});
  }
  V3 proj = rs_project_origin_and_reduce(s);
  float max_bound = FLT_MAX;
  int niter = 0;
  bool last_chance = false;
  for (;;) {
    float old_max_bound = max_bound;
    float nb;
    V3 u;
    if (try_normalize(-proj, eps_tol, &u, &nb)) { dir = u; max_bound = nb; }
    else { *toi_out = ltoi / ray_length; *n_out = ldir; return true; }
    V3 sp;
    if (max_bound >= old_max_bound) {
      last_chance = true;
      sp = proj + co;
    } else {
      sp = kind_support<TY>(shape, dir);
    }
    if (last_chance && ltoi > 0.0f) { *toi_out = ltoi / ray_length; *n_out = ldir; return true; }
    float t;
    if (ray_halfspace(sp, dir, co, cd, &t)) {
      if (dot(dir, cd) < 0.0f && t > 0.0f) {
        ldir = dir;
        ltoi += t;
        if (ltoi / ray_length > max_toi) return false;
        V3 shift = cd * t;
        co = co + shift;
        max_bound = FLT_MAX;
        rs_translate(s, -shift);
        last_chance = false;
      }
    } else {
      if (dot(dir, cd) > eps_tol) return false;
    }
    if (last_chance) return false;
    float min_bound = -dot(dir, sp - co);
    if (max_bound - min_bound <= eps_rel * max_bound) return false;
    {
      const V3 q = sp - co;
      rs_add(s, CSO{q, q, q});
    }
    proj = rs_project_origin_and_reduce(s);
    if (s.dim == 3) {
      if (min_bound >= eps_tol) return false;
      *toi_out = ltoi / ray_length; *n_out = ldir; return true;
    }
    niter += 1;
    if (niter == 100) return false;
  }
}

// ray_support_map.rs:19-71 for one support kind, in the part's frame after the pose, as part_cast_ray.
template <uint32_t TY>
__device__ __forceinline__ bool part_cast_ray_kind(const ShapeDev& shape, const Pose& pose, V3 wo, V3 wd, float max_toi, bool solid, float* toi,
                                                   V3* n) {
  V3 o = pose_inv_point(pose, wo), d = pose_inv_rotate(pose, wd);
  float t;
  V3 nn;
  if (!gjk_cast_local_ray_kind<TY>(shape, o, d, max_toi, &t, &nn)) return false;
  if (!(solid || t != 0.0f)) {
    V3 ndir = normalize(d);
    V3 supp = kind_support<TY>(shape, ndir);
    float eps = 0.001f;
    float shift = dot(supp - o, ndir) + eps;
    float t2;
    V3 n2;
    if (!gjk_cast_local_ray_kind<TY>(shape, o + ndir * shift, -d, shift + eps, &t2, &n2)) return false;
    float tt = shift - t2;
    if (!(tt <= max_toi)) return false;
    t = tt;
    nn = -n2;
  }
  *toi = t;
  *n = pose_rotate(pose, nn);
  return true;
}

// ray_triangle.rs:49-152 (toi <= max_toi filter), normal facing the ray origin
__device__ __forceinline__ bool ray_triangle(V3 a, V3 b, V3 c, V3 o, V3 dir, float max_toi, float* toi, V3* nrm) {
  V3 ab = b - a, ac = c - a;
  V3 n = cross(ab, ac);
  float d = dot(n, dir);
  if (d == 0.0f) return false;
  V3 ap = o - a;
  float t = dot(ap, n);
  if ((t < 0.0f && d < 0.0f) || (t > 0.0f && d > 0.0f)) return false;
  d = fabsf(d);
  V3 e = -cross(dir, ap);
  float v, w, tt;
  V3 normal;
  if (t < 0.0f) {
    v = -dot(ac, e);
    if (v < 0.0f || v > d) return false;
    w = dot(ab, e);
    if (w < 0.0f || v + w > d) return false;
    float invd = 1.0f / d;
    tt = -t * invd;
    normal = -normalize(n);
  } else {
    v = dot(ac, e);
    if (v < 0.0f || v > d) return false;
    w = -dot(ab, e);
    if (w < 0.0f || v + w > d) return false;
    float invd = 1.0f / d;
    tt = t * invd;
    normal = normalize(n);
  }
  if (!(tt <= max_toi)) return false;
  *toi = tt;
  *nrm = normal;
  return true;
}

// RayCast::cast_ray_and_get_normal(pose, ray, max_toi, solid) for one part.
__device__ __noinline__ bool part_cast_ray(const ShapeDev& s, const Pose& pose, V3 wo, V3 wd, float max_toi, bool solid, float* toi, V3* n) {
  V3 o = pose_inv_point(pose, wo), d = pose_inv_rotate(pose, wd);
  V3 ln;
  bool ok;
  switch (s.type) {
    case SH_BALL: ok = ray_ball(s.a, o, d, solid, max_toi, toi, &ln); break;
    case SH_CUBOID: ok = ray_cuboid(v3(s.a, s.b, s.c), o, d, solid, max_toi, toi, &ln); break;
    case SH_TRIANGLE: ok = ray_triangle(ldv(s.pts), ldv(s.pts + 3), ldv(s.pts + 6), o, d, max_toi, toi, &ln); break;
    default: ok = ray_support_map(s, o, d, solid, max_toi, toi, &ln); break;
  }
  if (ok) *n = pose_rotate(pose, ln);
  return ok;
}

// Ray vs AABB slab (ray_aabb.rs:12-49, solid), FLT_MAX on a miss.
__device__ __forceinline__ float slab(float3 mn, float3 mx, V3 o, V3 inv, uint32_t zmask, float max_toi) {
  float tmin = 0.0f, tmax = max_toi;
  bool miss = false;
  float oo[3] = {o.x, o.y, o.z}, iv[3] = {inv.x, inv.y, inv.z}, lo[3] = {mn.x, mn.y, mn.z}, hi[3] = {mx.x, mx.y, mx.z};
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    if (zmask & (1u << i)) {
      miss |= (oo[i] < lo[i]) | (oo[i] > hi[i]);
    } else {
      float a = (lo[i] - oo[i]) * iv[i], b = (hi[i] - oo[i]) * iv[i];
      if (a > b) { float t = a; a = b; b = t; }
      tmin = fmaxf(tmin, a);
      tmax = fminf(tmax, b);
    }
  }
  return (!miss && tmin <= tmax) ? tmin : FLT_MAX;
}

struct CompoundDev {
  const uint32_t* types;
  const float4* params;
  const float* poses;
  const float* pool;
  const float4* hull_box;  // per shape: local vertex bounds of a convex hull (min, max); may be null
};

// Local vertex bounds of every convex shape (one thread per shape); other shapes and invalid
// vertex ranges get an unbounded box, which filters nothing.
__global__ void k_hull_local_boxes(const uint32_t* __restrict__ types, const float4* __restrict__ params, const float* __restrict__ pool,
                                   uint32_t n, uint64_t n_vertices, float4* __restrict__ box) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float4 lo = make_float4(-FLT_MAX, -FLT_MAX, -FLT_MAX, 0.f), hi = make_float4(FLT_MAX, FLT_MAX, FLT_MAX, 0.f);
  if (types[i] == SH_CONVEX) {
    float4 p = params[i];
    uint64_t first = __float_as_uint(p.x), count = __float_as_uint(p.y);
    if (count > 0 && first + count <= n_vertices) {
      const float* v = pool + 3 * first;
      lo = make_float4(v[0], v[1], v[2], 0.f);
      hi = lo;
      for (uint64_t k = 1; k < count; ++k) {
        float x = v[3 * k], y = v[3 * k + 1], z = v[3 * k + 2];
        lo.x = fminf(lo.x, x); lo.y = fminf(lo.y, y); lo.z = fminf(lo.z, z);
        hi.x = fmaxf(hi.x, x); hi.y = fmaxf(hi.y, y); hi.z = fmaxf(hi.z, z);
      }
    }
  }
  box[2 * (size_t)i] = lo;
  box[2 * (size_t)i + 1] = hi;
}

// How far outside a shape the GJK ray cast (gjk.rs:660-795) may report a hit, as a margin for the
// pre-tests below: the cast stops when its distance bounds agree within sqrt(eps) relative, and on a
// rounded shape it was measured reporting hits for rays passing up to 0.41 % of a capsule's radius
// outside it (800,000 grazing rays against the f32 oracle); 3 % of the shape's extent keeps a wide
// safety factor. Plus 1e-4 of the coordinates' magnitude for the rounding of the transform.
__device__ __forceinline__ float gjk_ray_margin(float ext, V3 ol) {
  return 0.03f * ext + 1e-4f * (1.0f + ext + fmaxf(fmaxf(fabsf(ol.x), fabsf(ol.y)), fabsf(ol.z)));
}

// Conservative pre-test of a capsule / hull candidate: can the ray (world o, dir) reach the shape's
// local box (capsule: its exact bounds; hull: its vertex bounds), inflated by gjk_ray_margin, before
// `tlim`? A false answer proves the GJK ray cast cannot return a hit at toi <= tlim, so the
// candidate is dropped without changing any answer. *t_in receives a lower bound of the entry time.
__device__ __forceinline__ bool local_box_may_hit(const CompoundDev& cd, uint32_t part, uint32_t ty, V3 o, V3 dir, float tlim, float* t_in) {
  float3 lo, hi;
  float4 prm = cd.params[part];
  if (ty == SH_CAPSULE) {
    lo = make_float3(-prm.y, -prm.x - prm.y, -prm.y);
    hi = make_float3(prm.y, prm.x + prm.y, prm.y);
  } else if (cd.hull_box) {
    float4 a = cd.hull_box[2 * (size_t)part], b = cd.hull_box[2 * (size_t)part + 1];
    lo = make_float3(a.x, a.y, a.z);
    hi = make_float3(b.x, b.y, b.z);
  } else {
    *t_in = 0.0f;
    return true;
  }
  Pose p = load_pose(cd.poses, part);
  V3 ol = pose_inv_point(p, o), dl = pose_inv_rotate(p, dir);
  float ext = fmaxf(fmaxf(fmaxf(fabsf(lo.x), fabsf(hi.x)), fmaxf(fabsf(lo.y), fabsf(hi.y))), fmaxf(fabsf(lo.z), fabsf(hi.z)));
  if (!(ext < 1e30f)) { *t_in = 0.0f; return true; }  // unbounded box: no filter
  const float m = gjk_ray_margin(ext, ol);
  float tmin = 0.0f, tmax = tlim + fabsf(tlim) * 1e-5f;
  const float oo[3] = {ol.x, ol.y, ol.z}, dd[3] = {dl.x, dl.y, dl.z};
  const float lov[3] = {lo.x - m, lo.y - m, lo.z - m}, hiv[3] = {hi.x + m, hi.y + m, hi.z + m};
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    if (fabsf(dd[i]) < 1e-30f) {
      if (oo[i] < lov[i] || oo[i] > hiv[i]) return false;
    } else {
      // fast division (within 2 ulp): the inflated box and the padded tmax absorb it
      float a = __fdividef(lov[i] - oo[i], dd[i]), b = __fdividef(hiv[i] - oo[i], dd[i]);
      if (a > b) { float t = a; a = b; b = t; }
      tmin = fmaxf(tmin, a);
      tmax = fminf(tmax, b);
    }
  }
  *t_in = tmin;
  return tmin <= tmax;
}

// Conservative pre-test of a capsule candidate after the box test: can the ray's line come within
// radius + margin of the capsule's axis line? The line-to-line distance is a lower bound of the
// distance from the ray to the capsule's axis segment, so a ray farther than that misses the
// capsule. Computed in double precision in the capsule's frame (axis = y) with the box test's
// margin (gjk_ray_margin). A false answer proves the GJK ray cast returns no hit.
__device__ __forceinline__ bool capsule_may_hit(const CompoundDev& cd, uint32_t part, V3 o, V3 dir) {
  const float4 prm = cd.params[part];
  const Pose p = load_pose(cd.poses, part);
  const V3 ol = pose_inv_point(p, o), dl = pose_inv_rotate(p, dir);
  const double rad = prm.y;
  const double lim = rad + (double)gjk_ray_margin(prm.x + prm.y, ol);
  const double ex = dl.x, ez = dl.z, px = ol.x, pz = ol.z;
  const double den2 = ex * ex + ez * ez;
  if (den2 == 0.0) return px * px + pz * pz <= lim * lim;  // along the axis: a constant distance
  const double num = px * ez - pz * ex;                      // |P x E| in the x-z plane
  return num * num <= lim * lim * den2;
}

// Thread k handles ray r = order[k] (order may be null: r = k), read from slot k when the rays were
// already permuted into that order (rays_permuted), else from slot r; results go to slot r.
__global__ void __launch_bounds__(128) k_compound_rays(const WideNode* __restrict__ wide, CompoundDev cd, const float* __restrict__ rays,
                                                       uint32_t n, float max_toi, int solid, int has_pose, Pose cpose,
                                                       uint32_t* __restrict__ part_out, float* __restrict__ toi_out,
                                                       float* __restrict__ normal_out, uint32_t* __restrict__ err,
                                                       const uint32_t* __restrict__ order, int rays_permuted,
                                                       const uint8_t* __restrict__ only) {
  uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  uint32_t r = order ? order[k] : k;
  if (only && !only[r]) return;
  const float* rp = rays + 6 * (size_t)(rays_permuted ? k : r);
  V3 o = v3(rp[0], rp[1], rp[2]), dir = v3(rp[3], rp[4], rp[5]);
  if (has_pose) { o = pose_inv_point(cpose, o); dir = pose_inv_rotate(cpose, dir); }
  uint32_t zmask = (dir.x == 0.0f ? 1u : 0u) | (dir.y == 0.0f ? 2u : 0u) | (dir.z == 0.0f ? 4u : 0u);
  V3 inv = v3(dir.x != 0.0f ? 1.0f / dir.x : 0.0f, dir.y != 0.0f ? 1.0f / dir.y : 0.0f, dir.z != 0.0f ? 1.0f / dir.z : 0.0f);
  float best = max_toi;
  uint32_t best_part = 0xffffffffu;
  V3 best_n = v3(0.f, 0.f, 0.f);
  bool have = false;
  auto try_leaf = [&](uint32_t part) {
    ShapeDev s = load_shape(cd.types, cd.params, cd.pool, part);
    Pose p = load_pose(cd.poses, part);
    float t;
    V3 nn;
    if (!part_cast_ray(s, p, o, dir, best, solid != 0, &t, &nn)) return;
    if (t < best || (have && t == best && part < best_part)) { best = t; best_part = part; best_n = nn; have = true; }
  };
  WideNode w;
  load_wide(wide, 0, &w);
  if ((w.r.data & 0x3fffffffu) == 0u) {
    float s = slab(w.l.mins, w.l.maxs, o, inv, zmask, max_toi);
    if (s < max_toi) try_leaf(w.l.children);
  } else {
    uint32_t stack[CRAY_STACK];
    int sp = 0;
    for (;;) {
      float ls = slab(w.l.mins, w.l.maxs, o, inv, zmask, best);
      float rs = slab(w.r.mins, w.r.maxs, o, inv, zmask, best);
      const BvhNodeDev* nearn = &w.l;
      const BvhNodeDev* farn = &w.r;
      if (ls > rs) { float t = ls; ls = rs; rs = t; nearn = &w.r; farn = &w.l; }
      uint32_t next = 0xffffffffu;
      uint32_t far_child = farn->children, far_data = farn->data;
      if (ls != FLT_MAX && (ls < best || (have && ls == best))) {
        if ((nearn->data & 0x3fffffffu) == 1u) try_leaf(nearn->children);
        else next = nearn->children;
      }
      if (rs != FLT_MAX && (rs < best || (have && rs == best))) {
        if ((far_data & 0x3fffffffu) == 1u) try_leaf(far_child);
        else if (next != 0xffffffffu) {
          if (sp >= CRAY_STACK) { atomicOr(err, ERR_STACK_OVERFLOW); break; }
          stack[sp++] = far_child;
        } else next = far_child;
      }
      if (next == 0xffffffffu) {
        if (sp == 0) break;
        next = stack[--sp];
      }
      load_wide(wide, next, &w);
    }
  }
  if (has_pose && have) best_n = pose_rotate(cpose, best_n);
  part_out[r] = have ? best_part : 0xffffffffu;
  toi_out[r] = have ? best : 0.0f;
  if (normal_out) {
    normal_out[3 * (size_t)r] = best_n.x;
    normal_out[3 * (size_t)r + 1] = best_n.y;
    normal_out[3 * (size_t)r + 2] = best_n.z;
  }
}

// ---- wavefront shape-set rays ----
// The single-kernel traversal above carries the GJK ray cast's state (155 registers), which caps
// the occupancy of the whole, latency-bound traversal. The wavefront form splits it:
//   k_rays_wave     traversal + the analytic leaves (balls, cuboids, triangles) in few registers.
//                   A support-map leaf (capsule, hull) whose box the ray enters before the best
//                   analytic hit becomes a candidate with its box entry time: the ray's nearest
//                   candidate goes to list A, the others to list B (both compacted by
//                   warp-aggregated appends, so the GJK kernels run on dense lists).
//                   The ray's best hit so far is published as the 64-bit key (toi bits, index).
//   k_rays_cand_kind<capsule | hull>  GJK ray casts (their toi does not depend on the max_toi
//                   bound, which only accepts or rejects) for list A, then for list B skipping
//                   candidates whose box entry lies beyond the ray's current best; atomicMin of
//                   (toi, index).
//   k_rays_finish   the candidate holding its ray's minimum key writes the ray's result.
// The frame pipeline replaces k_rays_wave by the grid walk k_rays_walk (below), which lists the
// analytic leaves too (list C, tested by k_rays_cand_analytic before the GJK candidates).
// The minimum of (toi, index) over every hit with toi < max_toi is the single-kernel answer (nearest
// hit, lowest index on exact ties). Rays whose candidates did not fit a list are redone by the
// single kernel (mask `only`).
struct RayCand {
  uint32_t k, r, part, hit;
  float tmin, t, nx, ny, nz, pad;
};

__device__ __forceinline__ unsigned long long hit_key(float t, uint32_t part) {
  return ((unsigned long long)__float_as_uint(t + 0.0f) << 32) | part;
}
__device__ __forceinline__ float key_toi(unsigned long long key) {
  return key == ~0ull ? FLT_MAX : __uint_as_float((uint32_t)(key >> 32));
}

__device__ __forceinline__ bool analytic_type(uint32_t t) { return t == SH_BALL || t == SH_CUBOID || t == SH_TRIANGLE; }

// part_cast_ray for the analytic shapes only.
__device__ __forceinline__ bool part_cast_ray_analytic(const ShapeDev& s, const Pose& pose, V3 wo, V3 wd, float max_toi, bool solid, float* toi,
                                                       V3* n) {
  V3 o = pose_inv_point(pose, wo), d = pose_inv_rotate(pose, wd);
  V3 ln;
  bool ok;
  if (s.type == SH_BALL) ok = ray_ball(s.a, o, d, solid, max_toi, toi, &ln);
  else if (s.type == SH_CUBOID) ok = ray_cuboid(v3(s.a, s.b, s.c), o, d, solid, max_toi, toi, &ln);
  else ok = ray_triangle(ldv(s.pts), ldv(s.pts + 3), ldv(s.pts + 6), o, d, max_toi, toi, &ln);
  if (ok) *n = pose_rotate(pose, ln);
  return ok;
}

__device__ __forceinline__ void ray_of(const float* rays, const uint32_t* order, int permuted, uint32_t k, int has_pose, const Pose& cpose,
                                       uint32_t* r, V3* o, V3* dir) {
  *r = order ? order[k] : k;
  const float* rp = rays + 6 * (size_t)(permuted ? k : *r);
  *o = v3(rp[0], rp[1], rp[2]);
  *dir = v3(rp[3], rp[4], rp[5]);
  if (has_pose) { *o = pose_inv_point(cpose, *o); *dir = pose_inv_rotate(cpose, *dir); }
}

// Candidate lists are two-ended: capsule candidates fill a list from the front, hull candidates
// from the back, so each kind's entries are contiguous and the GJK kernels run warps of one kind
// (a capsule's support is O(1), a hull's a vertex scan). A list's 64-bit counter holds the front
// count (low half) and the back count (high half).
struct WaveBufs {
  RayCand* a;            // nearest candidate of each ray that has one (capacity n)
  RayCand* b;            // the other candidates (capacity cap)
  unsigned long long cap;
  unsigned long long* count;    // [0] list B counter, [1] list A counter, [2] list B first-failure snapshot,
                                // [8] list C counter, [9] list C snapshot
  unsigned long long* keys;  // per ray (index r)
  uint8_t* ovf;              // per ray (index r)
  RayCand* c;                // the grid walk's analytic candidates: balls at the front, the others at the back
                             // (capacity cap)
};

// Appends one slot per calling thread to a two-ended list of `cap` entries (kind 0 at the front,
// kind 1 at the back) with one atomicAdd per group of converged threads. A group whose slots do
// not all fit gets none (returns ~0), and its leader records the counter value it found in *fail
// (atomicMin): counters only grow, so every later group fails too, and the first failure's value
// is the count of slots actually written at each end.
__device__ __forceinline__ unsigned long long append_slot2(unsigned long long* counter, unsigned long long cap, uint32_t kind,
                                                           unsigned long long* fail) {
  namespace cg = cooperative_groups;
  cg::coalesced_group g = cg::coalesced_threads();
  const unsigned back = g.ballot(kind != 0);
  const uint32_t n1 = (uint32_t)__popc(back), n0 = g.size() - n1;
  unsigned long long base = 0;
  if (g.thread_rank() == 0) base = atomicAdd(counter, (unsigned long long)n0 | ((unsigned long long)n1 << 32));
  base = g.shfl(base, 0);
  const unsigned long long lo = base & 0xffffffffull, hi = base >> 32;
  if (lo + hi + n0 + n1 > cap) {
    if (fail && g.thread_rank() == 0) atomicMin(fail, base);
    return ~0ull;
  }
  const uint32_t below = (uint32_t)__popc(back & ((1u << g.thread_rank()) - 1u));  // back-kind threads of lower rank
  return kind ? cap - 1ull - (hi + below) : lo + (g.thread_rank() - below);
}

// Entries of a two-ended list: [0, front) and [cap - back, cap), as one index space.
__device__ __forceinline__ void list_extent(const unsigned long long* counter, const unsigned long long* fail, unsigned long long* front,
                                            unsigned long long* back) {
  unsigned long long c = *counter;
  if (fail && *fail != ~0ull) c = *fail;
  *front = c & 0xffffffffull;
  *back = c >> 32;
}
__device__ __forceinline__ unsigned long long list_slot(unsigned long long i, unsigned long long front, unsigned long long cap) {
  return i < front ? i : cap - 1ull - (i - front);
}

// ---- uniform grid over the shapes (the frame pipeline's rays) ----
// Each frame the grid is placed on the BVH root box (which holds every shape's loosened AABB),
// widened by `delta`; its resolution is fixed. A shape is entered in every cell its AABB, widened by
// delta, overlaps. A ray clipped to the grid box walks its cells in order (3-D DDA) and tests the
// entries' AABBs as the BVH traversal tests its leaf boxes. A point of the ray lies within delta of
// a cell the walk visits (delta is far above the walk's rounding), so every shape the ray reaches
// is met; the walk stops once the next cell starts beyond the best hit (with a margin). The leaves
// met are those the BVH traversal meets (possibly more, and some twice), and the answer - the
// minimum (toi, index) - is the same. When the entries outgrow their capacity the grid reports
// itself unusable (ok = 0) and the BVH kernel casts the rays of that frame instead.
struct GridDev {
  float lo[3], cell[3], inv[3], delta;
  uint32_t res[3], ok;
  unsigned long long total;  // entries counted this frame
};

// One entry of a cell: the shape's AABB with its index and type (two 16-byte loads, no second
// lookup).
struct __align__(16) GridEntry {
  float mn[3];
  uint32_t part;
  float mx[3];
  uint32_t type;
};

__global__ void k_grid_setup(const float* __restrict__ root, GridDev* __restrict__ g, uint32_t rx, uint32_t ry, uint32_t rz) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  float m = 0.0f;
  for (int i = 0; i < 6; ++i) m = fmaxf(m, fabsf(root[i]));
  const float delta = 1e-3f + 4e-6f * m;
  const uint32_t res[3] = {rx, ry, rz};
  for (int i = 0; i < 3; ++i) {
    const float lo = root[i] - delta, hi = root[3 + i] + delta;
    float c = (hi - lo) / (float)res[i];
    if (!(c > 0.0f) || !isfinite(c)) c = 1.0f;
    g->lo[i] = lo;
    g->cell[i] = c;
    g->inv[i] = 1.0f / c;
    g->res[i] = res[i];
  }
  g->delta = delta;
  g->ok = isfinite(m) ? 1u : 0u;
  g->total = 0ull;
}

__device__ __forceinline__ uint32_t grid_coord(const GridDev& g, int axis, float x) {
  const float f = floorf((x - g.lo[axis]) * g.inv[axis]);
  if (!(f > 0.0f)) return 0u;  // (NaN too)
  const float top = (float)(g.res[axis] - 1u);
  return f >= top ? g.res[axis] - 1u : (uint32_t)f;
}

// Cell range of shape i's AABB widened by delta; false for an empty range.
__device__ __forceinline__ void grid_range(const GridDev& g, const float* __restrict__ aabbs, uint32_t i, uint32_t* a, uint32_t* b) {
  const float* bx = aabbs + 6 * (size_t)i;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    a[k] = grid_coord(g, k, bx[k] - g.delta);
    b[k] = grid_coord(g, k, bx[3 + k] + g.delta);
  }
}

__global__ void k_grid_count(const float* __restrict__ aabbs, uint32_t n, GridDev* __restrict__ g, uint32_t* __restrict__ counts) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const GridDev gd = *g;
  unsigned long long mine = 0;
  if (i < n && gd.ok) {
    uint32_t a[3], b[3];
    grid_range(gd, aabbs, i, a, b);
    mine = (unsigned long long)(b[0] - a[0] + 1) * (b[1] - a[1] + 1) * (b[2] - a[2] + 1);
    if (mine <= 4096ull) {
      for (uint32_t z = a[2]; z <= b[2]; ++z)
        for (uint32_t y = a[1]; y <= b[1]; ++y)
          for (uint32_t x = a[0]; x <= b[0]; ++x) atomicAdd(&counts[((size_t)z * gd.res[1] + y) * gd.res[0] + x], 1u);
    }
  }
  // a shape over more than 4096 cells is not entered, and the grid is not used this frame
  if (mine > 4096ull) {
    g->ok = 0u;
    mine = 0;
  }
  const uint32_t w = __reduce_add_sync(0xffffffffu, (uint32_t)mine);
  if ((threadIdx.x & 31) == 0 && w) atomicAdd(&g->total, (unsigned long long)w);
}

__global__ void k_grid_check(GridDev* __restrict__ g, unsigned long long cap) {
  if (threadIdx.x == 0 && blockIdx.x == 0 && g->total > cap) g->ok = 0u;
}

__global__ void k_grid_fill(const float* __restrict__ aabbs, const uint32_t* __restrict__ types, uint32_t n, const GridDev* __restrict__ g,
                            const uint32_t* __restrict__ starts, uint32_t* __restrict__ cursor, GridEntry* __restrict__ entries,
                            unsigned long long cap) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const GridDev gd = *g;
  if (i >= n || !gd.ok) return;
  uint32_t a[3], b[3];
  grid_range(gd, aabbs, i, a, b);
  const float* bx = aabbs + 6 * (size_t)i;
  const GridEntry e{{bx[0], bx[1], bx[2]}, i, {bx[3], bx[4], bx[5]}, types[i]};
  for (uint32_t z = a[2]; z <= b[2]; ++z)
    for (uint32_t y = a[1]; y <= b[1]; ++y)
      for (uint32_t x = a[0]; x <= b[0]; ++x) {
        const size_t c = ((size_t)z * gd.res[1] + y) * gd.res[0] + x;
        const unsigned long long slot = (unsigned long long)starts[c] + atomicAdd(&cursor[c], 1u);
        if (slot < cap) entries[slot] = e;
      }
}

__global__ void __launch_bounds__(128) k_rays_wave(const WideNode* __restrict__ wide, CompoundDev cd, const float* __restrict__ rays, uint32_t n,
                                                   float max_toi, int solid, int has_pose, Pose cpose, uint32_t* __restrict__ part_out,
                                                   float* __restrict__ toi_out, float* __restrict__ normal_out, uint32_t* __restrict__ err,
                                                   const uint32_t* __restrict__ order, int permuted, WaveBufs wb,
                                                   const GridDev* __restrict__ grid) {
  uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  // with a usable grid the walk (k_rays_walk) casts the rays instead
  if (grid && grid->ok != 0u) return;
  uint32_t r;
  V3 o, dir;
  ray_of(rays, order, permuted, k, has_pose, cpose, &r, &o, &dir);
  uint32_t zmask = (dir.x == 0.0f ? 1u : 0u) | (dir.y == 0.0f ? 2u : 0u) | (dir.z == 0.0f ? 4u : 0u);
  V3 inv = v3(dir.x != 0.0f ? 1.0f / dir.x : 0.0f, dir.y != 0.0f ? 1.0f / dir.y : 0.0f, dir.z != 0.0f ? 1.0f / dir.z : 0.0f);
  float best = max_toi;
  uint32_t best_part = 0xffffffffu;
  V3 best_n = v3(0.f, 0.f, 0.f);
  bool have = false, overflow = false;
  uint32_t near_part = 0xffffffffu;
  float near_tmin = FLT_MAX;
  auto defer = [&](uint32_t part, float tmin) {
    if (overflow) return;  // this ray is recast by the single kernel anyway
    unsigned long long slot = append_slot2(wb.count, wb.cap, cd.types[part] == SH_CAPSULE ? 0u : 1u, wb.count + 2);
    if (slot != ~0ull) wb.b[slot] = RayCand{k, r, part, 0u, tmin, 0.f, 0.f, 0.f, 0.f, 0.f};
    else overflow = true;
  };
  auto visit_leaf = [&](uint32_t part, float tmin) {
    uint32_t ty = cd.types[part];
    if (!analytic_type(ty)) {
      float t_box;
      if (!local_box_may_hit(cd, part, ty, o, dir, best, &t_box)) return;
      tmin = fmaxf(tmin, t_box);
      if (tmin < near_tmin) {
        if (near_part != 0xffffffffu) defer(near_part, near_tmin);
        near_part = part;
        near_tmin = tmin;
      } else {
        defer(part, tmin);
      }
      return;
    }
    ShapeDev s = load_shape(cd.types, cd.params, cd.pool, part);
    Pose p = load_pose(cd.poses, part);
    float t;
    V3 nn;
    if (!part_cast_ray_analytic(s, p, o, dir, best, solid != 0, &t, &nn)) return;
    if (t < best || (have && t == best && part < best_part)) { best = t; best_part = part; best_n = nn; have = true; }
  };
  {
  WideNode w;
  load_wide(wide, 0, &w);
  if ((w.r.data & 0x3fffffffu) == 0u) {
    float s0 = slab(w.l.mins, w.l.maxs, o, inv, zmask, max_toi);
    if (s0 < max_toi) visit_leaf(w.l.children, s0);
  } else {
    uint32_t stack[CRAY_STACK];
    int sp = 0;
    for (;;) {
      float ls = slab(w.l.mins, w.l.maxs, o, inv, zmask, best);
      float rs = slab(w.r.mins, w.r.maxs, o, inv, zmask, best);
      const BvhNodeDev* nearn = &w.l;
      const BvhNodeDev* farn = &w.r;
      if (ls > rs) { float t = ls; ls = rs; rs = t; nearn = &w.r; farn = &w.l; }
      uint32_t next = 0xffffffffu;
      uint32_t far_child = farn->children, far_data = farn->data;
      if (ls != FLT_MAX && (ls < best || (have && ls == best))) {
        if ((nearn->data & 0x3fffffffu) == 1u) visit_leaf(nearn->children, ls);
        else next = nearn->children;
      }
      if (rs != FLT_MAX && (rs < best || (have && rs == best))) {
        if ((far_data & 0x3fffffffu) == 1u) visit_leaf(far_child, rs);
        else if (next != 0xffffffffu) {
          if (sp >= CRAY_STACK) { atomicOr(err, ERR_STACK_OVERFLOW); break; }
          stack[sp++] = far_child;
        } else next = far_child;
      }
      if (next == 0xffffffffu) {
        if (sp == 0) break;
        next = stack[--sp];
      }
      load_wide(wide, next, &w);
    }
  }
  }  // BVH traversal
  if (near_part != 0xffffffffu) {
    // at most one entry per ray: list A (n entries) never fills
    unsigned long long slot = append_slot2(wb.count + 1, n, cd.types[near_part] == SH_CAPSULE ? 0u : 1u, nullptr);
    wb.a[slot] = RayCand{k, r, near_part, 0u, near_tmin, 0.f, 0.f, 0.f, 0.f, 0.f};
  }
  wb.keys[r] = have ? hit_key(best, best_part) : ~0ull;
  wb.ovf[r] = overflow ? 1 : 0;
  if (has_pose && have) best_n = pose_rotate(cpose, best_n);
  part_out[r] = have ? best_part : 0xffffffffu;
  toi_out[r] = have ? best : 0.0f;
  if (normal_out) {
    normal_out[3 * (size_t)r] = best_n.x;
    normal_out[3 * (size_t)r + 1] = best_n.y;
    normal_out[3 * (size_t)r + 2] = best_n.z;
  }
}

// The grid walk alone (frame pipeline rays): every shape whose AABB the ray enters below max_toi
// becomes a candidate - an analytic shape in list C (balls at the front), a capsule / hull that
// passes the local-box pre-test in list A (the ray's nearest) or B - and the leaf tests run in their
// own kernels afterwards, each over one shape kind. Walking without a best hit costs the walk the
// cells behind a ray's first hit, but keeps the warp's lanes on one code path: walking leaf tests
// inline left fewer than 5 of 32 lanes active. The ray's outputs start as "no hit"; the candidate
// kernels publish hits through the per-ray key and k_rays_finish writes the winners. A ray whose
// candidates overflow a list is marked for the single-kernel cast. Does nothing when the grid is
// unusable (the BVH wave kernel casts the rays then).
// Per-warp staging of the grid walk's appends to a two-ended list: a warp's entries gather in shared
// memory (front kind from slot 0 up, back kind from the last slot down) and reach the global list in
// batches of up to WALK_STAGE, one counter update per batch. The lanes of a walk rarely append in
// the same loop turn, so appending one group of lanes at a time cost one contended atomic on the
// list's counter per 1-5 entries. Every live lane of the warp takes part in each put and flush, so
// the held counts (n0, n1) and the overflow bits are the same in all of them.
constexpr uint32_t WALK_STAGE = 32;
struct WalkStage {
  RayCand* e;      // this warp's WALK_STAGE shared-memory slots
  uint32_t n0, n1;  // front / back entries held
};

// Writes the held entries to the list and empties the stage. A batch that does not fit is not
// written: its first-failure snapshot is kept (as by append_slot2) and the owners of its entries
// (lane = k mod 32) are returned as overflow bits.
__device__ __forceinline__ uint32_t walk_stage_flush(WalkStage& st, unsigned live, unsigned long long* counter, unsigned long long cap,
                                                     unsigned long long* fail, RayCand* __restrict__ list) {
  const uint32_t n0 = st.n0, n1 = st.n1;
  if (n0 + n1 == 0u) return 0u;
  const uint32_t lane = threadIdx.x & 31u, leader = (uint32_t)__ffs(live) - 1u;
  const uint32_t rank = (uint32_t)__popc(live & ((1u << lane) - 1u)), size = (uint32_t)__popc(live);
  unsigned long long base = 0;
  if (lane == leader) base = atomicAdd(counter, (unsigned long long)n0 | ((unsigned long long)n1 << 32));
  base = __shfl_sync(live, base, leader);
  const unsigned long long lo = base & 0xffffffffull, hi = base >> 32;
  uint32_t bits = 0u;
  if (lo + hi + n0 + n1 > cap) {
    if (lane == leader) atomicMin(fail, base);
    for (uint32_t i = rank; i < n0; i += size) bits |= 1u << (st.e[i].k & 31u);
    for (uint32_t i = rank; i < n1; i += size) bits |= 1u << (st.e[WALK_STAGE - 1u - i].k & 31u);
  } else {
    for (uint32_t i = rank; i < n0; i += size) list[lo + i] = st.e[i];
    for (uint32_t i = rank; i < n1; i += size) list[cap - 1ull - (hi + i)] = st.e[WALK_STAGE - 1u - i];
  }
  __syncwarp(live);  // the slots are read before they are refilled
  st.n0 = 0u;
  st.n1 = 0u;
  return __reduce_or_sync(live, bits);
}

// Adds the entry of each lane with `add` (kind 0 front, 1 back); flushes first if they do not fit.
__device__ __forceinline__ uint32_t walk_stage_put(WalkStage& st, unsigned live, bool add, uint32_t kind, const RayCand& c,
                                                   unsigned long long* counter, unsigned long long cap, unsigned long long* fail,
                                                   RayCand* __restrict__ list) {
  const unsigned want = __ballot_sync(live, add), back = __ballot_sync(live, add && kind != 0u);
  const uint32_t m1 = (uint32_t)__popc(back), m0 = (uint32_t)__popc(want) - m1;
  uint32_t bits = 0u;
  if (st.n0 + st.n1 + m0 + m1 > WALK_STAGE) bits = walk_stage_flush(st, live, counter, cap, fail, list);
  if (add) {
    const unsigned lt = (1u << (threadIdx.x & 31u)) - 1u;
    const uint32_t idx = kind ? WALK_STAGE - 1u - (st.n1 + (uint32_t)__popc(back & lt)) : st.n0 + (uint32_t)__popc(want & ~back & lt);
    st.e[idx] = c;
  }
  __syncwarp(live);  // the entries are in place before any lane flushes them
  st.n0 += m0;
  st.n1 += m1;
  return bits;
}

__global__ void __launch_bounds__(128) k_rays_walk(CompoundDev cd, const float* __restrict__ rays, uint32_t n, float max_toi, int has_pose,
                                                   Pose cpose, uint32_t* __restrict__ part_out, float* __restrict__ toi_out,
                                                   float* __restrict__ normal_out, const uint32_t* __restrict__ order, int permuted,
                                                   WaveBufs wb, const GridDev* __restrict__ grid, const uint32_t* __restrict__ starts,
                                                   const GridEntry* __restrict__ entries) {
  __shared__ RayCand stage_mem[2][4][WALK_STAGE];  // lists B and C, per warp of the 128-thread block
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  const bool mine = k < n && grid->ok != 0u;
  const unsigned live = __ballot_sync(0xffffffffu, mine);
  if (!mine) return;
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
  WalkStage st_b{stage_mem[0][warp], 0u, 0u}, st_c{stage_mem[1][warp], 0u, 0u};
  uint32_t ovf_bits = 0u;
  uint32_t r;
  V3 o, dir;
  ray_of(rays, order, permuted, k, has_pose, cpose, &r, &o, &dir);
  const uint32_t zmask = (dir.x == 0.0f ? 1u : 0u) | (dir.y == 0.0f ? 2u : 0u) | (dir.z == 0.0f ? 4u : 0u);
  const V3 inv = v3(dir.x != 0.0f ? 1.0f / dir.x : 0.0f, dir.y != 0.0f ? 1.0f / dir.y : 0.0f, dir.z != 0.0f ? 1.0f / dir.z : 0.0f);
  uint32_t near_part = 0xffffffffu, near_ty = 0u;
  float near_tmin = FLT_MAX;
  const GridDev g = *grid;
  const float3 glo = make_float3(g.lo[0], g.lo[1], g.lo[2]);
  const float3 ghi = make_float3(g.lo[0] + g.cell[0] * (float)g.res[0], g.lo[1] + g.cell[1] * (float)g.res[1], g.lo[2] + g.cell[2] * (float)g.res[2]);
  const float t0 = slab(glo, ghi, o, inv, zmask, max_toi);
  bool walking = t0 != FLT_MAX;
  uint32_t cx = 0u, cy = 0u, cz = 0u, j = 0u, e1 = 0u;
  uint32_t s0 = 0xffffffffu, s1 = 0xffffffffu, s2 = 0xffffffffu, s3 = 0xffffffffu;  // the last parts met
  auto cross_t = [&](int a, uint32_t ci, float oa, float da, float ia) {
    if (zmask & (1u << a)) return FLT_MAX;
    const float b = g.lo[a] + g.cell[a] * (float)(da > 0.0f ? ci + 1u : ci);
    return (b - oa) * ia;
  };
  if (walking) {
    cx = grid_coord(g, 0, o.x + dir.x * t0);
    cy = grid_coord(g, 1, o.y + dir.y * t0);
    cz = grid_coord(g, 2, o.z + dir.z * t0);
    const size_t cell = ((size_t)cz * g.res[1] + cy) * g.res[0] + cx;
    j = starts[cell];
    e1 = starts[cell + 1];
  }
  // One loop turn tests one entry of the current cell, or steps to the next cell: lanes whose cells
  // hold different numbers of entries stay in step. Each turn ends at a point all live lanes reach,
  // where the entries chosen in the turn go to the warp's stages.
  for (;;) {
    bool add_b = false, add_c = false;
    uint32_t kind = 0u;
    RayCand cand;
    const bool overflow = (ovf_bits >> lane) & 1u;
    if (walking) {
      if (j < e1) {
        do {
          const float4 ea = __ldg(reinterpret_cast<const float4*>(entries + j));
          const float4 eb = __ldg(reinterpret_cast<const float4*>(entries + j) + 1);
          ++j;
          const uint32_t part = __float_as_uint(ea.w);
          if (part == s0 || part == s1 || part == s2 || part == s3) break;  // met in an earlier cell
          s3 = s2;
          s2 = s1;
          s1 = s0;
          s0 = part;
          float ts = slab(make_float3(ea.x, ea.y, ea.z), make_float3(eb.x, eb.y, eb.z), o, inv, zmask, max_toi);
          if (ts == FLT_MAX || !(ts < max_toi) || overflow) break;
          const uint32_t ty = __float_as_uint(eb.w);
          if (analytic_type(ty)) {
            add_c = true;
            kind = ty == SH_BALL ? 0u : 1u;
            cand = RayCand{k, r, part, 0u, ts, 0.f, 0.f, 0.f, 0.f, 0.f};
            break;
          }
          float t_box;
          if (!local_box_may_hit(cd, part, ty, o, dir, max_toi, &t_box)) break;
          ts = fmaxf(ts, t_box);
          uint32_t dpart = part, dty = ty;
          float dt = ts;
          if (ts < near_tmin) {
            dpart = near_part;
            dty = near_ty;
            dt = near_tmin;
            near_part = part;
            near_ty = ty;
            near_tmin = ts;
          }
          if (dpart != 0xffffffffu) {
            add_b = true;
            kind = dty == SH_CAPSULE ? 0u : 1u;
            cand = RayCand{k, r, dpart, 0u, dt, 0.f, 0.f, 0.f, 0.f, 0.f};
          }
        } while (false);
      } else {
        const float tx = cross_t(0, cx, o.x, dir.x, inv.x), ty = cross_t(1, cy, o.y, dir.y, inv.y), tz = cross_t(2, cz, o.z, dir.z, inv.z);
        const float tn = fminf(tx, fminf(ty, tz));
        bool out = tn >= FLT_MAX || !(tn <= max_toi);
        if (!out) {
          if (tn == tx) {
            if (dir.x > 0.0f) out = ++cx >= g.res[0];
            else if (cx == 0u) out = true;
            else --cx;
          } else if (tn == ty) {
            if (dir.y > 0.0f) out = ++cy >= g.res[1];
            else if (cy == 0u) out = true;
            else --cy;
          } else {
            if (dir.z > 0.0f) out = ++cz >= g.res[2];
            else if (cz == 0u) out = true;
            else --cz;
          }
        }
        if (out) {
          walking = false;
        } else {
          const size_t cell = ((size_t)cz * g.res[1] + cy) * g.res[0] + cx;
          j = starts[cell];
          e1 = starts[cell + 1];
        }
      }
    }
    if (__any_sync(live, add_c)) ovf_bits |= walk_stage_put(st_c, live, add_c, kind, cand, wb.count + 8, wb.cap, wb.count + 9, wb.c);
    if (__any_sync(live, add_b)) ovf_bits |= walk_stage_put(st_b, live, add_b, kind, cand, wb.count, wb.cap, wb.count + 2, wb.b);
    if (!__any_sync(live, walking)) break;
  }
  ovf_bits |= walk_stage_flush(st_c, live, wb.count + 8, wb.cap, wb.count + 9, wb.c);
  ovf_bits |= walk_stage_flush(st_b, live, wb.count, wb.cap, wb.count + 2, wb.b);
  const bool overflow = (ovf_bits >> lane) & 1u;
  if (near_part != 0xffffffffu && !overflow) {
    const unsigned long long slot = append_slot2(wb.count + 1, n, near_ty == SH_CAPSULE ? 0u : 1u, nullptr);
    wb.a[slot] = RayCand{k, r, near_part, 0u, near_tmin, 0.f, 0.f, 0.f, 0.f, 0.f};
  }
  wb.keys[r] = ~0ull;
  wb.ovf[r] = overflow ? 1 : 0;
  part_out[r] = 0xffffffffu;
  toi_out[r] = 0.0f;
  if (normal_out) {
    normal_out[3 * (size_t)r] = 0.0f;
    normal_out[3 * (size_t)r + 1] = 0.0f;
    normal_out[3 * (size_t)r + 2] = 0.0f;
  }
}

// The analytic candidates of list C: FRONT = the balls, else the cuboids and triangles. A candidate
// whose box entry lies beyond the ray's current best is skipped.
template <bool FRONT>
__global__ void __launch_bounds__(128) k_rays_cand_analytic(CompoundDev cd, const float* __restrict__ rays, float max_toi, int solid,
                                                            int has_pose, Pose cpose, const uint32_t* __restrict__ order, int permuted,
                                                            RayCand* __restrict__ list, unsigned long long cap,
                                                            const unsigned long long* __restrict__ count,
                                                            const unsigned long long* __restrict__ fail, unsigned long long* __restrict__ keys) {
  unsigned long long front, back;
  list_extent(count, fail, &front, &back);
  const unsigned long long m = FRONT ? front : back;
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < m;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    RayCand* e = list + (FRONT ? i : cap - 1ull - i);
    const RayCand c = *e;
    if (c.tmin > key_toi(keys[c.r])) continue;
    uint32_t r;
    V3 o, dir;
    ray_of(rays, order, permuted, c.k, has_pose, cpose, &r, &o, &dir);
    const ShapeDev sh = load_shape(cd.types, cd.params, cd.pool, c.part);
    const Pose p = load_pose(cd.poses, c.part);
    float t;
    V3 nn;
    // composite casts keep hits strictly below max_toi (CompositeShapeRef::cast_local_ray)
    if (!part_cast_ray_analytic(sh, p, o, dir, max_toi, solid != 0, &t, &nn) || !(t < max_toi)) continue;
    if (has_pose) nn = pose_rotate(cpose, nn);
    e->hit = 1u;
    e->t = t;
    e->nx = nn.x;
    e->ny = nn.y;
    e->nz = nn.z;
    atomicMin(&keys[r], hit_key(t, c.part));
  }
}

// One end of a two-ended list: TY = SH_CAPSULE runs the front (capsule candidates), SH_CONVEX the
// back (the other support-map kinds; a part that is not a convex hull takes part_cast_ray).
template <uint32_t TY>
__global__ void __launch_bounds__(128, 4) k_rays_cand_kind(CompoundDev cd, const float* __restrict__ rays, float max_toi, int solid, int has_pose,
                                                        Pose cpose, const uint32_t* __restrict__ order, int permuted,
                                                        RayCand* __restrict__ list, unsigned long long cap,
                                                        const unsigned long long* __restrict__ count,
                                                        const unsigned long long* __restrict__ fail, unsigned long long* __restrict__ keys) {
  unsigned long long front, back;
  list_extent(count, fail, &front, &back);
  const unsigned long long m = TY == SH_CAPSULE ? front : back;
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < m;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    RayCand* e = list + (TY == SH_CAPSULE ? i : cap - 1ull - i);
    RayCand c = *e;
    if (c.part == 0xffffffffu) continue;
    const float best = key_toi(keys[c.r]);
    if (c.tmin > best) continue;
    uint32_t r;
    V3 o, dir;
    ray_of(rays, order, permuted, c.k, has_pose, cpose, &r, &o, &dir);
    // (the candidate passed the local-box pre-test when it was listed); a capsule's axis distance
    if (TY == SH_CAPSULE && !capsule_may_hit(cd, c.part, o, dir)) continue;
    ShapeDev sh = load_shape(cd.types, cd.params, cd.pool, c.part);
    Pose p = load_pose(cd.poses, c.part);
    float t;
    V3 nn;
    bool ok;
    if (TY == SH_CAPSULE || sh.type == SH_CONVEX) ok = part_cast_ray_kind<TY>(sh, p, o, dir, max_toi, solid != 0, &t, &nn);
    else ok = part_cast_ray(sh, p, o, dir, max_toi, solid != 0, &t, &nn);
    // composite casts keep hits strictly below max_toi (CompositeShapeRef::cast_local_ray)
    if (!ok || !(t < max_toi)) continue;
    if (has_pose) nn = pose_rotate(cpose, nn);
    e->hit = 1u;
    e->t = t;
    e->nx = nn.x;
    e->ny = nn.y;
    e->nz = nn.z;
    atomicMin(&keys[r], hit_key(t, c.part));
  }
}

__global__ void __launch_bounds__(128) k_rays_finish(const RayCand* __restrict__ list, unsigned long long cap,
                                                     const unsigned long long* __restrict__ count, const unsigned long long* __restrict__ fail,
                                                     const unsigned long long* __restrict__ keys, uint32_t* __restrict__ part_out,
                                                     float* __restrict__ toi_out, float* __restrict__ normal_out) {
  unsigned long long front, back;
  list_extent(count, fail, &front, &back);
  const unsigned long long m = front + back;
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < m;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    RayCand e = list[list_slot(i, front, cap)];
    if (!e.hit || keys[e.r] != hit_key(e.t, e.part)) continue;
    part_out[e.r] = e.part;
    toi_out[e.r] = e.t;
    if (normal_out) {
      normal_out[3 * (size_t)e.r] = e.nx;
      normal_out[3 * (size_t)e.r + 1] = e.ny;
      normal_out[3 * (size_t)e.r + 2] = e.nz;
    }
  }
}

}  // namespace

static parrygpu_status compound_copy_in(parrygpu_ctx* ctx, DevBuf& dst, const void* src, size_t bytes) {
  PG_CUDA(ctx, dst.reserve(bytes ? bytes : 16));
  if (bytes) PG_CUDA(ctx, cudaMemcpyAsync(dst.ptr, src, bytes, cudaMemcpyDefault, ctx->stream));
  return PARRYGPU_OK;
}

parrygpu_status shape_rays_reserve(parrygpu_ctx* ctx, RayWaveScratch& sc, uint32_t n) {
  if (n > (1u << 30)) return set_error(ctx, PARRYGPU_INVALID_ARG, "shape-set ray casts take at most 2^30 rays per call");
  uint64_t cap = 4ull * n + 1024;  // below 2^32: the list counters pack two 32-bit counts
  PG_CUDA(ctx, sc.cands.reserve((2 * cap + n) * sizeof(RayCand)));  // list A (n slots), list B (cap), list C (cap)
  PG_CUDA(ctx, sc.counter.reserve(96));  // [0..2] lists A / B, [8..9] list C
  PG_CUDA(ctx, sc.keys.reserve((size_t)n * 8 + 16));
  PG_CUDA(ctx, sc.ovf.reserve((size_t)n + 16));
  sc.cap = cap;
  return PARRYGPU_OK;
}

parrygpu_status shape_ray_grid_reserve(parrygpu_ctx* ctx, RayGridScratch& g, uint64_t n_shapes, const float* root) {
  double ext[3], vol = 1.0;
  for (int i = 0; i < 3; ++i) {
    ext[i] = (double)root[3 + i] - (double)root[i];
    if (!(ext[i] > 0.0) || !std::isfinite(ext[i])) ext[i] = 0.0;
    vol *= ext[i] > 0.0 ? ext[i] : 1.0;
  }
  double c = std::cbrt(vol / (4.0 * (double)(n_shapes ? n_shapes : 1)));
  uint64_t cells = 0;
  for (int it = 0; it < 64; ++it) {
    cells = 1;
    for (int i = 0; i < 3; ++i) {
      double r = ext[i] > 0.0 && c > 0.0 ? std::ceil(ext[i] / c) : 1.0;
      g.res[i] = (uint32_t)std::min(1024.0, std::max(1.0, r));
      cells *= g.res[i];
    }
    if (cells <= (1ull << 22)) break;
    c *= 1.25;
  }
  g.cells = cells;
  g.cap = 16ull * n_shapes + 4096ull;
  PG_CUDA(ctx, g.dev.reserve(sizeof(GridDev)));
  PG_CUDA(ctx, g.starts.reserve(((cells + 1 + 3) & ~3ull) * 4 + 16));
  PG_CUDA(ctx, g.cursor.reserve(cells * 4 + 16));
  PG_CUDA(ctx, g.entries.reserve(g.cap * sizeof(GridEntry)));
  PG_CUDA(ctx, g.sums.reserve((size_t)exclusive_scan_u32_sums((uint32_t)(cells + 1)) * 4 + 16));
  return PARRYGPU_OK;
}

// The grid of this frame from the shapes' AABBs and the BVH root box: placement, counts, starts
// (exclusive scan), capacity check, fill.
static parrygpu_status build_grid(parrygpu_ctx* ctx, RayGridScratch& g, const float* root, const float* aabbs, const uint32_t* types,
                                  uint32_t n_shapes) {
  GridDev* gd = g.dev.as<GridDev>();
  const uint32_t m = (uint32_t)((g.cells + 1 + 3) & ~3ull);
  k_grid_setup<<<1, 32, 0, ctx->stream>>>(root, gd, g.res[0], g.res[1], g.res[2]);
  PG_LAUNCHED(ctx);
  PG_CUDA(ctx, cudaMemsetAsync(g.starts.ptr, 0, (size_t)m * 4, ctx->stream));
  PG_CUDA(ctx, cudaMemsetAsync(g.cursor.ptr, 0, g.cells * 4, ctx->stream));
  k_grid_count<<<div_up(n_shapes, 256), 256, 0, ctx->stream>>>(aabbs, n_shapes, gd, g.starts.as<uint32_t>());
  PG_LAUNCHED(ctx);
  k_grid_check<<<1, 32, 0, ctx->stream>>>(gd, g.cap);
  PG_LAUNCHED(ctx);
  parrygpu_status s = exclusive_scan_u32_wide(ctx, g.starts.as<uint32_t>(), m, g.sums.as<uint32_t>());
  if (s != PARRYGPU_OK) return s;
  k_grid_fill<<<div_up(n_shapes, 256), 256, 0, ctx->stream>>>(aabbs, types, n_shapes, gd, g.starts.as<uint32_t>(), g.cursor.as<uint32_t>(),
                                                              g.entries.as<GridEntry>(), g.cap);
  PG_LAUNCHED(ctx);
  return PARRYGPU_OK;
}

// The wavefront cast of n rays (see k_rays_wave). No allocation, no host synchronisation. With a
// grid (and the shapes' AABBs and the BVH root box), the grid is rebuilt and walked; the BVH kernel
// still launches and casts the rays itself only if the grid reports itself unusable.
static parrygpu_status launch_wave(parrygpu_ctx* ctx, const WideNode* wide, CompoundDev cd, const float* d_rays, const uint32_t* order,
                                   int permuted, uint32_t n, float max_toi, int solid, int has_pose, Pose pose, uint32_t* d_part,
                                   float* d_toi, float* d_nrm, RayWaveScratch& sc, RayGridScratch* rg = nullptr, const float* aabbs = nullptr,
                                   const float* root = nullptr, uint32_t n_shapes = 0) {
  unsigned long long* cnt = sc.counter.as<unsigned long long>();
  WaveBufs wb{sc.cands.as<RayCand>(), sc.cands.as<RayCand>() + n, sc.cap, cnt, sc.keys.as<unsigned long long>(), sc.ovf.as<uint8_t>(),
              sc.cands.as<RayCand>() + n + sc.cap};
  uint32_t grid = (uint32_t)(ctx->sm_count > 0 ? ctx->sm_count : 152) * 16;
  PG_CUDA(ctx, cudaMemsetAsync(cnt, 0, 16, ctx->stream));
  PG_CUDA(ctx, cudaMemsetAsync(cnt + 2, 0xff, 8, ctx->stream));
  PG_CUDA(ctx, cudaMemsetAsync(cnt + 8, 0, 8, ctx->stream));
  PG_CUDA(ctx, cudaMemsetAsync(cnt + 9, 0xff, 8, ctx->stream));
  const bool use_grid = rg && rg->cells && aabbs && root;
  const GridDev* gd = nullptr;
  if (use_grid) {
    parrygpu_status s = build_grid(ctx, *rg, root, aabbs, cd.types, n_shapes);
    if (s != PARRYGPU_OK) return s;
    gd = rg->dev.as<GridDev>();
    k_rays_walk<<<div_up(n, 128), 128, 0, ctx->stream>>>(cd, d_rays, n, max_toi, has_pose, pose, d_part, d_toi, d_nrm, order, permuted, wb, gd,
                                                         rg->starts.as<uint32_t>(), rg->entries.as<GridEntry>());
    PG_LAUNCHED(ctx);
  }
  k_rays_wave<<<div_up(n, 128), 128, 0, ctx->stream>>>(wide, cd, d_rays, n, max_toi, solid, has_pose, pose, d_part, d_toi, d_nrm,
                                                       ctx->d_err, order, permuted, wb, gd);
  PG_LAUNCHED(ctx);
  if (use_grid) {  // the walk's analytic candidates first: their hits prune the GJK candidates
    k_rays_cand_analytic<true><<<grid, 128, 0, ctx->stream>>>(cd, d_rays, max_toi, solid, has_pose, pose, order, permuted, wb.c, sc.cap,
                                                              cnt + 8, cnt + 9, wb.keys);
    PG_LAUNCHED(ctx);
    k_rays_cand_analytic<false><<<grid, 128, 0, ctx->stream>>>(cd, d_rays, max_toi, solid, has_pose, pose, order, permuted, wb.c, sc.cap,
                                                               cnt + 8, cnt + 9, wb.keys);
    PG_LAUNCHED(ctx);
  }
  // list A, then list B; capsules and hulls of each in their own launches
  k_rays_cand_kind<SH_CAPSULE><<<grid, 128, 0, ctx->stream>>>(cd, d_rays, max_toi, solid, has_pose, pose, order, permuted, wb.a, n, cnt + 1,
                                                              nullptr, wb.keys);
  PG_LAUNCHED(ctx);
  k_rays_cand_kind<SH_CONVEX><<<grid, 128, 0, ctx->stream>>>(cd, d_rays, max_toi, solid, has_pose, pose, order, permuted, wb.a, n, cnt + 1,
                                                             nullptr, wb.keys);
  PG_LAUNCHED(ctx);
  k_rays_cand_kind<SH_CAPSULE><<<grid, 128, 0, ctx->stream>>>(cd, d_rays, max_toi, solid, has_pose, pose, order, permuted, wb.b, sc.cap, cnt,
                                                              cnt + 2, wb.keys);
  PG_LAUNCHED(ctx);
  k_rays_cand_kind<SH_CONVEX><<<grid, 128, 0, ctx->stream>>>(cd, d_rays, max_toi, solid, has_pose, pose, order, permuted, wb.b, sc.cap, cnt,
                                                             cnt + 2, wb.keys);
  PG_LAUNCHED(ctx);
  k_rays_finish<<<grid, 128, 0, ctx->stream>>>(wb.a, n, cnt + 1, nullptr, wb.keys, d_part, d_toi, d_nrm);
  PG_LAUNCHED(ctx);
  k_rays_finish<<<grid, 128, 0, ctx->stream>>>(wb.b, sc.cap, cnt, cnt + 2, wb.keys, d_part, d_toi, d_nrm);
  PG_LAUNCHED(ctx);
  if (use_grid) {
    k_rays_finish<<<grid, 128, 0, ctx->stream>>>(wb.c, sc.cap, cnt + 8, cnt + 9, wb.keys, d_part, d_toi, d_nrm);
    PG_LAUNCHED(ctx);
  }
  // rays whose candidates overflowed list B: the single-kernel cast, for them only
  k_compound_rays<<<div_up(n, 128), 128, 0, ctx->stream>>>(wide, cd, d_rays, n, max_toi, solid, has_pose, pose, d_part, d_toi, d_nrm,
                                                           ctx->d_err, order, permuted, sc.ovf.as<uint8_t>());
  PG_LAUNCHED(ctx);
  return PARRYGPU_OK;
}

parrygpu_status launch_hull_boxes(parrygpu_ctx* ctx, const uint32_t* types, const float* params, const float* pool, uint32_t n,
                                  uint64_t n_vertices, float* box) {
  if (n == 0) return PARRYGPU_OK;
  k_hull_local_boxes<<<div_up(n, 256), 256, 0, ctx->stream>>>(types, (const float4*)params, pool, n, n_vertices, (float4*)box);
  PG_LAUNCHED(ctx);
  return PARRYGPU_OK;
}

parrygpu_status launch_shape_rays(parrygpu_ctx* ctx, const parrygpu_bvh* bvh, const uint32_t* types, const float* params,
                                  const float* poses, const float* pool, const float* hull_box, const float* d_rays, const uint32_t* order,
                                  uint32_t n, float max_toi, uint32_t* d_part, float* d_toi, float* d_nrm, RayWaveScratch& scratch,
                                  RayGridScratch* grid, const float* d_aabbs) {
  if (n == 0 || bvh->n_leaves == 0) return PARRYGPU_OK;
  CompoundDev cd{types, (const float4*)params, poses, pool, (const float4*)hull_box};
  Pose pose{0.f, 0.f, 0.f, 1.f, v3(0.f, 0.f, 0.f)};
  return launch_wave(ctx, bvh->wide.as<WideNode>(), cd, d_rays, order, order ? 1 : 0, n, max_toi, 1, 0, pose, d_part, d_toi, d_nrm, scratch,
                     grid, d_aabbs, grid ? bvh->root_aabb.as<float>() : nullptr, bvh->n_leaves);
}

extern "C" {

parrygpu_status parrygpu_compound_create(parrygpu_ctx* ctx, const parrygpu_shapes* shapes, parrygpu_compound** out) {
  if (!ctx || !shapes || !out) return PARRYGPU_INVALID_ARG;
  *out = nullptr;
  if (shapes->n > 0xffffffffull) return set_error(ctx, PARRYGPU_INVALID_ARG, "too many parts");
  PG_CUDA(ctx, cudaSetDevice(ctx->device));
  parrygpu_compound* c = new parrygpu_compound();
  c->n = shapes->n;
  c->n_vertices = shapes->n_vertices;
  parrygpu_status s;
  if ((s = compound_copy_in(ctx, c->types, shapes->types, c->n * 4)) != PARRYGPU_OK ||
      (s = compound_copy_in(ctx, c->params, shapes->params, c->n * 16)) != PARRYGPU_OK ||
      (s = compound_copy_in(ctx, c->poses, shapes->poses, c->n * 28)) != PARRYGPU_OK ||
      (s = compound_copy_in(ctx, c->pool, shapes->vertices, c->n_vertices * 12)) != PARRYGPU_OK ||
      (s = compound_copy_in(ctx, c->aabbs, nullptr, 0)) != PARRYGPU_OK) {
    parrygpu_compound_destroy(c);
    return s;
  }
  if (c->n > 0) {
    if ((s = check_cuda(ctx, c->aabbs.reserve(c->n * 24), "compound aabbs")) != PARRYGPU_OK ||
        (s = check_cuda(ctx, c->hull_box.reserve(c->n * 32), "compound hull boxes")) != PARRYGPU_OK ||
        (s = launch_hull_boxes(ctx, c->types.as<uint32_t>(), c->params.as<float>(), c->pool.as<float>(), (uint32_t)c->n, c->n_vertices,
                               c->hull_box.as<float>())) != PARRYGPU_OK ||
        (s = compound_part_aabbs(ctx, c, c->aabbs.as<float>())) != PARRYGPU_OK ||
        (s = lbvh_build(ctx, &c->bvh, c->aabbs.as<float>(), (uint32_t)c->n, false)) != PARRYGPU_OK) {
      parrygpu_compound_destroy(c);
      return s;
    }
  }
  PG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if ((s = parrygpu_sync(ctx)) != PARRYGPU_OK) {
    parrygpu_compound_destroy(c);
    return set_error(ctx, PARRYGPU_INVALID_ARG, "invalid shape description (type or vertex range)");
  }
  *out = c;
  return PARRYGPU_OK;
}

void parrygpu_compound_destroy(parrygpu_compound* c) {
  if (!c) return;
  for (DevBuf* d : {&c->types, &c->params, &c->poses, &c->pool, &c->aabbs, &c->hull_box, &c->bvh.wide, &c->bvh.leaf_parent, &c->bvh.node_parent,
                    &c->bvh.leaf_index, &c->bvh.flags, &c->bvh.root_aabb, &c->bvh.info})
    d->release();
  delete c;
}

parrygpu_status parrygpu_compound_set_poses(parrygpu_ctx* ctx, parrygpu_compound* c, const float* poses) {
  if (!ctx || !c) return PARRYGPU_INVALID_ARG;
  if (c->n == 0) return PARRYGPU_OK;
  if (!poses) return set_error(ctx, PARRYGPU_INVALID_ARG, "poses is null");
  PG_CUDA(ctx, cudaSetDevice(ctx->device));
  PG_CUDA(ctx, cudaMemcpyAsync(c->poses.ptr, poses, c->n * 28, cudaMemcpyDefault, ctx->stream));
  parrygpu_status s = compound_part_aabbs(ctx, c, c->aabbs.as<float>());
  if (s != PARRYGPU_OK) return s;
  s = lbvh_refit(ctx, &c->bvh, c->aabbs.as<float>());
  if (s != PARRYGPU_OK) return s;
  if (!is_device_ptr(poses)) PG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return PARRYGPU_OK;
}

parrygpu_status parrygpu_compound_cast_rays(parrygpu_ctx* ctx, const parrygpu_compound* c, const float* pose7, const float* rays, uint32_t n,
                                            float max_toi, int solid, uint32_t* part, float* toi, float* normal) {
  if (!ctx || !c) return PARRYGPU_INVALID_ARG;
  if (n == 0) return PARRYGPU_OK;
  if (!rays || !part || !toi) return set_error(ctx, PARRYGPU_INVALID_ARG, "rays, part and toi are required");
  PG_CUDA(ctx, cudaSetDevice(ctx->device));
  Pose pose{0.f, 0.f, 0.f, 1.f, v3(0.f, 0.f, 0.f)};
  if (pose7) {
    float p[7];
    PG_CUDA(ctx, cudaMemcpyAsync(p, pose7, 28, cudaMemcpyDefault, ctx->stream));
    PG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    pose = Pose{p[0], p[1], p[2], p[3], v3(p[4], p[5], p[6])};
  }
  const void* d_rays;
  parrygpu_status s = stage_input(ctx, ctx->stage_in[6], rays, (size_t)n * 24, &d_rays);
  if (s != PARRYGPU_OK) return s;
  void *d_part, *d_toi, *d_nrm;
  bool c1, c2, c3;
  if ((s = stage_output(ctx, ctx->stage_out[1], part, (size_t)n * 4, &d_part, &c1)) != PARRYGPU_OK) return s;
  if ((s = stage_output(ctx, ctx->stage_out[2], toi, (size_t)n * 4, &d_toi, &c2)) != PARRYGPU_OK) return s;
  if ((s = stage_output(ctx, ctx->stage_out[3], normal, (size_t)n * 12, &d_nrm, &c3)) != PARRYGPU_OK) return s;
  if (c->n == 0) {
    PG_CUDA(ctx, cudaMemsetAsync(d_part, 0xff, (size_t)n * 4, ctx->stream));
    PG_CUDA(ctx, cudaMemsetAsync(d_toi, 0, (size_t)n * 4, ctx->stream));
    if (d_nrm) PG_CUDA(ctx, cudaMemsetAsync(d_nrm, 0, (size_t)n * 12, ctx->stream));
  } else {
    CompoundDev cd{c->types.as<uint32_t>(), c->params.as<float4>(), c->poses.as<float>(), c->pool.as<float>(), c->hull_box.as<float4>()};
    const uint32_t* order = nullptr;
    if (ctx->cfg.sort_rays && n > 4096) {  // Morton order of the origins: coherent traversal
      if ((s = radix_sort_reserve(ctx, n)) != PARRYGPU_OK) return s;
      PG_CUDA(ctx, ctx->misc.reserve(64));
      uint32_t* bounds = ctx->misc.as<uint32_t>() + 8;
      if ((s = launch_ray_keys(ctx, (const float*)d_rays, n, bounds, ctx->sort_k[0].as<uint32_t>(), ctx->sort_v[0].as<uint32_t>(),
                               ctx->cfg.ray_sort_key)) != PARRYGPU_OK)
        return s;
      int rb;
      if ((s = radix_sort_pairs(ctx, n, ray_sort_bits(ctx), &rb)) != PARRYGPU_OK) return s;
      order = ctx->sort_v[rb].as<uint32_t>();
    }
    if ((s = shape_rays_reserve(ctx, ctx->ray_wave, n)) != PARRYGPU_OK) return s;
    KernelTimer kt(ctx, "compound_rays");
    s = launch_wave(ctx, c->bvh.wide.as<WideNode>(), cd, (const float*)d_rays, order, 0, n, max_toi, solid, pose7 ? 1 : 0, pose,
                    (uint32_t*)d_part, (float*)d_toi, (float*)d_nrm, ctx->ray_wave);
    kt.stop();
    if (s != PARRYGPU_OK) return s;
  }
  if (c1) PG_CUDA(ctx, cudaMemcpyAsync(part, d_part, (size_t)n * 4, cudaMemcpyDeviceToHost, ctx->stream));
  if (c2) PG_CUDA(ctx, cudaMemcpyAsync(toi, d_toi, (size_t)n * 4, cudaMemcpyDeviceToHost, ctx->stream));
  if (c3) PG_CUDA(ctx, cudaMemcpyAsync(normal, d_nrm, (size_t)n * 12, cudaMemcpyDeviceToHost, ctx->stream));
  if (c1 || c2 || c3 || d_rays != rays) return parrygpu_sync(ctx);
  return PARRYGPU_OK;
}

}  // extern "C"
