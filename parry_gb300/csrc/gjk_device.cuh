// Device-side convex queries: support maps, Voronoi-simplex projections and GJK.
//
// Every function follows the reference step for step (same branch tests, same evaluation order;
// the translation unit is compiled with --fmad=false), so hit/miss decisions, simplex reductions and
// EPA face choices are identical to the f32 reference on the same inputs. Paths are relative to the
// parry repository:
//   support maps  src/shape/{ball.rs:242-249, cuboid.rs:454-456, capsule.rs:407-418, triangle.rs:697-715},
//                 src/utils/point_cloud_support_point.rs:5-19 (first index wins ties)
//   CSOPoint      src/query/gjk/cso_point.rs:69-78
//   projections   src/query/point/point_segment.rs:49-84, point_triangle.rs:58-291, point_tetrahedron.rs:32-340
//   simplex       src/query/gjk/voronoi_simplex3.rs:57-279
//   GJK           src/query/gjk/gjk.rs:353-453, 797-818
#pragma once
#include "common.cuh"

namespace pg {

// SH_SEGMENT is a capsule's axis segment (its polygonal feature map, shape.rs:855-857): only
// built on the device, never a type of the C ABI.
enum : uint32_t { SH_BALL = 0, SH_CUBOID = 1, SH_CAPSULE = 2, SH_CONVEX = 3, SH_TRIANGLE = 4, SH_SEGMENT = 5, SH_ORIGIN = 255 };

constexpr float EPS = 1.1920929e-7f;         // f32::EPSILON
constexpr float GJK_EPS_TOL = EPS * 10.0f;   // gjk::eps_tol()

struct ShapeDev {
  uint32_t type;
  float a, b, c;               // ball: r; cuboid: hx hy hz; capsule: half_height, radius
  const float* __restrict__ pts;  // convex / triangle vertices (x, y, z) in the pool
  uint32_t npts;
};

__device__ __forceinline__ ShapeDev load_shape(const uint32_t* __restrict__ types, const float4* __restrict__ params,
                                               const float* __restrict__ pool, uint32_t i) {
  ShapeDev s;
  s.type = types[i];
  float4 p = params[i];
  s.a = p.x; s.b = p.y; s.c = p.z;
  s.pts = nullptr;
  s.npts = 0;
  if (s.type == SH_CONVEX || s.type == SH_TRIANGLE) {
    s.pts = pool + 3 * (size_t)__float_as_uint(p.x);
    s.npts = __float_as_uint(p.y);
  }
  return s;
}

__device__ __forceinline__ Pose load_pose(const float* __restrict__ poses, uint32_t i) {
  const float* p = poses + 7 * (size_t)i;
  return Pose{p[0], p[1], p[2], p[3], v3(p[4], p[5], p[6])};
}

__device__ __forceinline__ V3 ldv(const float* p) { return v3(__ldg(p), __ldg(p + 1), __ldg(p + 2)); }

// Unit::try_new(v, min_norm) / try_new_and_get
__device__ __forceinline__ bool try_normalize(V3 v, float min_norm, V3* out, float* n_out = nullptr) {
  float sq = dot(v, v);
  if (sq > min_norm * min_norm) {
    float n = sqrtf(sq);
    *out = v / n;
    if (n_out) *n_out = n;
    return true;
  }
  return false;
}

// Pose composition helpers (nalgebra Isometry / UnitQuaternion formulas).
__device__ __forceinline__ void quat_mul(float ai, float aj, float ak, float aw, float bi, float bj, float bk, float bw, float* ri,
                                         float* rj, float* rk, float* rw) {
  *ri = aw * bi + ai * bw + aj * bk - ak * bj;
  *rj = aw * bj - ai * bk + aj * bw + ak * bi;
  *rk = aw * bk + ai * bj - aj * bi + ak * bw;
  *rw = aw * bw - ai * bi - aj * bj - ak * bk;
}
// self^-1 * o  (Isometry::inv_mul)
__device__ __forceinline__ Pose pose_inv_mul(const Pose& s, const Pose& o) {
  Pose r;
  quat_mul(-s.qi, -s.qj, -s.qk, s.qw, o.qi, o.qj, o.qk, o.qw, &r.qi, &r.qj, &r.qk, &r.qw);
  r.t = quat_rotate(-s.qi, -s.qj, -s.qk, s.qw, o.t - s.t);
  return r;
}
// Isometry::inverse: rotation conj, translation conj * (-t)
__device__ __forceinline__ Pose pose_inverse(const Pose& s) {
  Pose r{-s.qi, -s.qj, -s.qk, s.qw, v3(0.f, 0.f, 0.f)};
  r.t = quat_rotate(r.qi, r.qj, r.qk, r.qw, -s.t);
  return r;
}

// Support point of a vertex cloud (point_cloud_support_point). Kept out of line: it is called
// from every support evaluation of every kernel, and one shared copy keeps the large GJK / EPA /
// manifold kernels within the instruction cache.
// Unroll factor of the support scan's loop over 4-vertex groups (0: the compiler's choice). A
// translation unit may define it before including this header. 2 keeps twice the loads in flight
// per thread (shape casts +9 %, manifolds +3 %, TriMesh contacts +2 % on the bench workloads); the
// fused contact kernel's GJK ran 3.2 ms per 1M hull pairs with the compiler's choice and 4.7-4.8 ms
// with any explicit factor (1, 2 or 4), so contact.cu builds with 0.
#ifndef PG_SCAN_UNROLL
#define PG_SCAN_UNROLL 2
#endif
#define PG_PRAGMA(x) _Pragma(#x)
#define PG_UNROLL(n) PG_PRAGMA(unroll n)

static __device__ __noinline__ V3 convex_support(const float* __restrict__ pts, uint32_t npts, V3 dir) {
  // First index of the maximum dot product (point_cloud_support_point: best = 0, then strict
  // `>`). Four partial scans, each seeded with vertex 0, keep four independent compare chains;
  // each keeps the first index of its own maximum (its indices increase), and the merge prefers
  // the larger value, then the smaller index - the sequential answer (NaN dot products never
  // replace, as in the sequential scan). Vertices are 12 bytes; from the first vertex whose
  // address is 16-byte aligned, groups of four are read as three 16-byte loads, one vertex per
  // chain; the vertices before and after those groups go to chain 0.
  const uint32_t n = npts;
  const float d0 = dot(ldv(pts), dir);
  uint32_t bi[4] = {0u, 0u, 0u, 0u};
  float bd[4] = {d0, d0, d0, d0};
  uint32_t h = 0;
  const uintptr_t addr = reinterpret_cast<uintptr_t>(pts);
  while (h < 4 && ((addr + 12u * h) & 15u) != 0) ++h;
  uint32_t i = 1;
  if (h < 4 && h + 4 <= n) {
    for (; i < h; ++i) {  // leading vertices: chain 0 (indices below the body's)
      float d = dot(ldv(pts + 3 * i), dir);
      if (d > bd[0]) { bd[0] = d; bi[0] = i; }
    }
    const float4* q = reinterpret_cast<const float4*>(pts + 3 * h);
#if PG_SCAN_UNROLL > 0
    PG_UNROLL(PG_SCAN_UNROLL)
#endif
    for (i = h; i + 4 <= n; i += 4, q += 3) {
      float4 a = __ldg(q), b = __ldg(q + 1), c = __ldg(q + 2);
      float e0 = dot(v3(a.x, a.y, a.z), dir), e1 = dot(v3(a.w, b.x, b.y), dir);
      float e2 = dot(v3(b.z, b.w, c.x), dir), e3 = dot(v3(c.y, c.z, c.w), dir);
      if (e0 > bd[0]) { bd[0] = e0; bi[0] = i; }
      if (e1 > bd[1]) { bd[1] = e1; bi[1] = i + 1; }
      if (e2 > bd[2]) { bd[2] = e2; bi[2] = i + 2; }
      if (e3 > bd[3]) { bd[3] = e3; bi[3] = i + 3; }
    }
  }
  for (; i < n; ++i) {  // trailing vertices (or all of a short / unaligned cloud): chain 0
    float d = dot(ldv(pts + 3 * i), dir);
    if (d > bd[0]) { bd[0] = d; bi[0] = i; }
  }
  uint32_t best = bi[0];
  float bv = bd[0];
#pragma unroll
  for (int l = 1; l < 4; ++l) {
    if (bd[l] > bv || (bd[l] == bv && bi[l] < best)) { bv = bd[l]; best = bi[l]; }
  }
  return ldv(pts + 3 * best);
}

// SupportMap::local_support_point
__device__ __forceinline__ V3 local_support(const ShapeDev& s, V3 dir) {
  switch (s.type) {
    case SH_BALL: return normalize(dir) * s.a;
    case SH_CUBOID: return v3(copysignf(s.a, dir.x), copysignf(s.b, dir.y), copysignf(s.c, dir.z));
    case SH_CAPSULE: {
      V3 d;
      if (!try_normalize(dir, 0.0f, &d)) d = v3(0.f, 1.f, 0.f);
      V3 a = v3(0.f, -s.a, 0.f), b = v3(0.f, s.a, 0.f);
      if (dot(d, a) > dot(d, b)) return a + d * s.b;
      return b + d * s.b;
    }
    case SH_SEGMENT: {
      // segment.rs:461-467
      V3 a = v3(0.f, -s.a, 0.f), b = v3(0.f, s.a, 0.f);
      return dot(a, dir) > dot(b, dir) ? a : b;
    }
    case SH_TRIANGLE: {
      V3 p0 = ldv(s.pts), p1 = ldv(s.pts + 3), p2 = ldv(s.pts + 6);
      float d1 = dot(p0, dir), d2 = dot(p1, dir), d3 = dot(p2, dir);
      if (d1 > d2) return d1 > d3 ? p0 : p2;
      return d2 > d3 ? p1 : p2;
    }
    case SH_CONVEX: return convex_support(s.pts, s.npts, dir);
    default: return v3(0.f, 0.f, 0.f);  // ConstantOrigin
  }
}

// SupportMap::support_point(m, dir) (support_map.rs:380-383); ConstantOrigin -> m.translation.
__device__ __forceinline__ V3 world_support(const ShapeDev& s, const Pose& m, V3 dir) {
  if (s.type == SH_ORIGIN) return m.t;
  return pose_point(m, local_support(s, pose_inv_rotate(m, dir)));
}

struct CSO {
  V3 p, o1, o2;
};

__device__ __forceinline__ CSO cso_from_shapes(const Pose& pos12, const ShapeDev& g1, const ShapeDev& g2, V3 dir) {
  V3 sp1 = local_support(g1, dir);
  V3 sp2 = world_support(g2, pos12, -dir);
  return CSO{sp1 - sp2, sp1, sp2};
}

// ---------------- point projections with location (solid) ----------------

enum : int { LOC_VERTEX = 0, LOC_EDGE = 1, LOC_FACE = 2, LOC_SOLID = 3 };
struct Loc {
  int kind, id;
  float bc[3];
};

__device__ __forceinline__ V3 project_segment(V3 a, V3 b, V3 pt, Loc* loc) {
  V3 ab = b - a, ap = pt - a;
  float ab_ap = dot(ab, ap), sqnab = dot(ab, ab);
  if (ab_ap <= 0.0f) { *loc = Loc{LOC_VERTEX, 0, {1.f, 0.f, 0.f}}; return a; }
  if (ab_ap >= sqnab) { *loc = Loc{LOC_VERTEX, 1, {0.f, 1.f, 0.f}}; return b; }
  float u = ab_ap / sqnab;
  *loc = Loc{LOC_EDGE, 0, {1.0f - u, u, 0.f}};
  return a + ab * u;
}

// The triangle and tetrahedron projections have an inline body for kernels that keep their simplex
// in registers, and an out-of-line copy that the other kernels share.
// The Voronoi region of pt against triangle (a, b, c), with the quantities its projection needs.
// The region tests are evaluated in full and the first that holds selected, instead of returning
// at the first region that holds: lanes of a warp that project onto different regions then stay on
// one path. Every value is the expression the early-return form computes (same operands, same
// operations), so the answer is the same bits.
struct TriRegion {
  V3 ab, ac, bc, ap, bp, n;
  float ab_ap, ac_ap, va, vb, vc;
  int region;  // 0-2 vertex a / b / c, 3 edge ab, 4 edge ac, 5 edge bc, 6 face, 7 solid
};

__device__ __forceinline__ TriRegion tri_region(V3 a, V3 b, V3 c, V3 pt) {
  TriRegion r;
  r.ab = b - a; r.ac = c - a; r.ap = pt - a;
  r.ab_ap = dot(r.ab, r.ap); r.ac_ap = dot(r.ac, r.ap);
  r.bp = pt - b;
  const float ab_bp = dot(r.ab, r.bp), ac_bp = dot(r.ac, r.bp);
  const V3 cp = pt - c;
  const float ab_cp = dot(r.ab, cp), ac_cp = dot(r.ac, cp);
  r.bc = c - b;
  r.n = cross(r.ab, r.ac);
  r.vc = dot(r.n, cross(r.ab, r.ap));
  r.vb = -dot(r.n, cross(r.ac, cp));
  r.va = dot(r.n, cross(r.bc, r.bp));
  if (r.ab_ap <= 0.0f && r.ac_ap <= 0.0f) r.region = 0;
  else if (ab_bp >= 0.0f && ac_bp <= ab_bp) r.region = 1;
  else if (ac_cp >= 0.0f && ab_cp <= ac_cp) r.region = 2;
  else if (r.vc < 0.0f && r.ab_ap >= 0.0f && ab_bp <= 0.0f) r.region = 3;
  else if (r.vb < 0.0f && r.ac_ap >= 0.0f && ac_cp <= 0.0f) r.region = 4;
  else if (r.va < 0.0f && ac_bp - ab_bp >= 0.0f && ab_cp - ac_cp >= 0.0f) r.region = 5;
  else if (r.va + r.vb + r.vc != 0.0f) r.region = 6;
  else r.region = 7;
  return r;
}

// The edge projection of a region 3-5: base + dir * t, t = num / |dir|^2.
__device__ __forceinline__ V3 tri_edge_point(const TriRegion& r, V3 a, V3 b, float* t_out) {
  const V3 base = r.region == 5 ? b : a;
  const V3 dir = r.region == 3 ? r.ab : (r.region == 4 ? r.ac : r.bc);
  const float num = r.region == 3 ? r.ab_ap : (r.region == 4 ? r.ac_ap : dot(r.bc, r.bp));
  const float t = num / dot(dir, dir);
  *t_out = t;
  return base + dir * t;
}

__device__ __forceinline__ V3 project_triangle_inl(V3 a, V3 b, V3 c, V3 pt, Loc* loc) {
  const TriRegion r = tri_region(a, b, c, pt);
  const int region = r.region;
  if (region < 3) {
    *loc = Loc{LOC_VERTEX, region, {region == 0 ? 1.f : 0.f, region == 1 ? 1.f : 0.f, region == 2 ? 1.f : 0.f}};
    return region == 0 ? a : (region == 1 ? b : c);
  }
  if (region < 6) {
    float t;
    const V3 p = tri_edge_point(r, a, b, &t);
    *loc = Loc{LOC_EDGE, region == 3 ? 0 : (region == 4 ? 2 : 1), {1.0f - t, t, 0.f}};
    return p;
  }
  if (region == 6) {
    const int side = dot(r.n, r.ap) >= 0.0f ? 0 : 1;
    const float denom = 1.0f / ((r.va + r.vb) + r.vc);
    const float v = r.vb * denom, w = r.vc * denom;
    *loc = Loc{LOC_FACE, side, {(1.0f - v) - w, v, w}};
    return (a + r.ab * v) + r.ac * w;
  }
  *loc = Loc{LOC_SOLID, 0, {0.f, 0.f, 0.f}};
  return pt;
}

static __device__ __noinline__ V3 project_triangle(V3 a, V3 b, V3 c, V3 pt, Loc* loc) { return project_triangle_inl(a, b, c, pt, loc); }

__device__ __forceinline__ bool tet_edge(int i, V3 a, V3 nabc, V3 nabd, V3 ap, V3 ab, float ap_ab, float bp_ab, float* dabc,
                                         float* dabd, V3* res, Loc* loc) {
  float ab_ab = ap_ab - bp_ab;
  V3 x = cross(ap, ab);
  *dabc = dot(x, nabc);
  *dabd = dot(x, nabd);
  if (ab_ab != 0.0f && *dabc >= 0.0f && *dabd >= 0.0f && ap_ab >= 0.0f && ap_ab <= ab_ab) {
    float u = ap_ab / ab_ab;
    *loc = Loc{LOC_EDGE, i, {1.0f - u, u, 0.f}};
    *res = a + ab * u;
    return true;
  }
  return false;
}

__device__ __forceinline__ bool tet_face(int i, V3 a, V3 b, V3 c, V3 ap, V3 bp, V3 cp, V3 ab, V3 ac, V3 ad, float dabc, float dbca,
                                         float dacb, V3* res, Loc* loc) {
  if (dabc < 0.0f && dbca < 0.0f && dacb < 0.0f) {
    V3 n = cross(ab, ac);
    if (dot(n, ad) * dot(n, ap) < 0.0f) {
      float nn = norm(n);
      if (nn <= EPS) return false;
      V3 normal = n / nn;
      float vc = dot(normal, cross(ap, bp));
      float va = dot(normal, cross(bp, cp));
      float vb = dot(normal, cross(cp, ap));
      float denom = va + vb + vc;
      float inv = 1.0f / denom;
      float b0 = va * inv, b1 = vb * inv, b2 = vc * inv;
      *loc = Loc{LOC_FACE, i, {b0, b1, b2}};
      *res = (a * b0 + b * b1) + c * b2;
      return true;
    }
  }
  return false;
}

__device__ __forceinline__ V3 project_tetrahedron_inl(V3 a, V3 b, V3 c, V3 d, V3 pt, Loc* loc) {
  V3 ab = b - a, ac = c - a, ad = d - a, ap = pt - a;
  float ap_ab = dot(ap, ab), ap_ac = dot(ap, ac), ap_ad = dot(ap, ad);
  if (ap_ab <= 0.0f && ap_ac <= 0.0f && ap_ad <= 0.0f) { *loc = Loc{LOC_VERTEX, 0, {1.f, 0.f, 0.f}}; return a; }
  V3 bc = c - b, bd = d - b, bp = pt - b;
  float bp_bc = dot(bp, bc), bp_bd = dot(bp, bd), bp_ab = dot(bp, ab);
  if (bp_bc <= 0.0f && bp_bd <= 0.0f && bp_ab >= 0.0f) { *loc = Loc{LOC_VERTEX, 1, {1.f, 0.f, 0.f}}; return b; }
  V3 cd = d - c, cp = pt - c;
  float cp_ac = dot(cp, ac), cp_bc = dot(cp, bc), cp_cd = dot(cp, cd);
  if (cp_cd <= 0.0f && cp_bc >= 0.0f && cp_ac >= 0.0f) { *loc = Loc{LOC_VERTEX, 2, {1.f, 0.f, 0.f}}; return c; }
  V3 dp = pt - d;
  float dp_cd = dot(dp, cd), dp_bd = dot(dp, bd), dp_ad = dot(dp, ad);
  if (dp_ad >= 0.0f && dp_bd >= 0.0f && dp_cd >= 0.0f) { *loc = Loc{LOC_VERTEX, 3, {1.f, 0.f, 0.f}}; return d; }
  V3 res;
  V3 nabc = cross(ab, ac), nabd = cross(ab, ad);
  float dabc, dabd, dacd, dacb, dadb, dadc, dbca, dbcd, dbdc, dbda, dcda, dcdb;
  if (tet_edge(0, a, nabc, nabd, ap, ab, ap_ab, bp_ab, &dabc, &dabd, &res, loc)) return res;
  V3 nacd = cross(ac, ad);
  if (tet_edge(1, a, nacd, -nabc, ap, ac, ap_ac, cp_ac, &dacd, &dacb, &res, loc)) return res;
  if (tet_edge(2, a, -nabd, -nacd, ap, ad, ap_ad, dp_ad, &dadb, &dadc, &res, loc)) return res;
  V3 nbcd = cross(bc, bd);
  if (tet_edge(3, b, nabc, nbcd, bp, bc, bp_bc, cp_bc, &dbca, &dbcd, &res, loc)) return res;
  if (tet_edge(4, b, -nbcd, nabd, bp, bd, bp_bd, dp_bd, &dbdc, &dbda, &res, loc)) return res;
  if (tet_edge(5, c, nacd, nbcd, cp, cd, cp_cd, dp_cd, &dcda, &dcdb, &res, loc)) return res;
  if (tet_face(0, a, b, c, ap, bp, cp, ab, ac, ad, dabc, dbca, dacb, &res, loc)) return res;
  if (tet_face(1, a, b, d, ap, bp, dp, ab, ad, ac, dadb, dabd, dbda, &res, loc)) return res;
  if (tet_face(2, a, c, d, ap, cp, dp, ac, ad, ab, dacd, dcda, dadc, &res, loc)) return res;
  if (tet_face(3, b, c, d, bp, cp, dp, bc, bd, -ab, dbcd, dcdb, dbdc, &res, loc)) return res;
  *loc = Loc{LOC_SOLID, 0, {0.f, 0.f, 0.f}};
  return pt;
}

static __device__ __noinline__ V3 project_tetrahedron(V3 a, V3 b, V3 c, V3 d, V3 pt, Loc* loc) {
  return project_tetrahedron_inl(a, b, c, d, pt, loc);
}

// ---------------- Voronoi simplex ----------------

struct Simplex {
  CSO v[4];
  float proj[3];
  float prev_proj[3];
  int8_t prev_v[4];
  int dim, prev_dim;
};

__device__ __forceinline__ void simplex_swap(Simplex& s, int i, int j) {
  CSO t = s.v[i]; s.v[i] = s.v[j]; s.v[j] = t;
  int8_t u = s.prev_v[i]; s.prev_v[i] = s.prev_v[j]; s.prev_v[j] = u;
}

__device__ __forceinline__ void simplex_reset(Simplex& s, const CSO& p) {
  s.dim = 0; s.prev_dim = 0; s.v[0] = p;
  s.prev_v[0] = 0; s.prev_v[1] = 1; s.prev_v[2] = 2; s.prev_v[3] = 3;
  s.proj[0] = s.proj[1] = s.proj[2] = 0.f;
  s.prev_proj[0] = s.prev_proj[1] = s.prev_proj[2] = 0.f;
}

__device__ __forceinline__ bool simplex_add(Simplex& s, const CSO& pt) {
  s.prev_dim = s.dim;
  s.prev_proj[0] = s.proj[0]; s.prev_proj[1] = s.proj[1]; s.prev_proj[2] = s.proj[2];
  s.prev_v[0] = 0; s.prev_v[1] = 1; s.prev_v[2] = 2; s.prev_v[3] = 3;
  if (s.dim == 0) {
    V3 d = s.v[0].p - pt.p;
    if (dot(d, d) < GJK_EPS_TOL) return false;
  } else if (s.dim == 1) {
    V3 ab = s.v[1].p - s.v[0].p, ac = pt.p - s.v[0].p;
    V3 c = cross(ab, ac);
    if (dot(c, c) < GJK_EPS_TOL) return false;
  } else if (s.dim == 2) {
    V3 ab = s.v[1].p - s.v[0].p, ac = s.v[2].p - s.v[0].p, ap = pt.p - s.v[0].p;
    V3 n = normalize(cross(ab, ac));
    if (fabsf(dot(n, ap)) < GJK_EPS_TOL) return false;
  }
  s.dim += 1;
  s.v[s.dim] = pt;
  return true;
}

static __device__ __noinline__ V3 simplex_project_origin_and_reduce(Simplex& s) {
  const V3 o = v3(0.f, 0.f, 0.f);
  Loc loc;
  if (s.dim == 0) {
    s.proj[0] = 1.0f;
    return s.v[0].p;
  } else if (s.dim == 1) {
    V3 p = project_segment(s.v[0].p, s.v[1].p, o, &loc);
    if (loc.kind == LOC_VERTEX && loc.id == 0) { s.proj[0] = 1.0f; s.dim = 0; }
    else if (loc.kind == LOC_VERTEX) { simplex_swap(s, 0, 1); s.proj[0] = 1.0f; s.dim = 0; }
    else { s.proj[0] = loc.bc[0]; s.proj[1] = loc.bc[1]; }
    return p;
  } else if (s.dim == 2) {
    V3 p = project_triangle(s.v[0].p, s.v[1].p, s.v[2].p, o, &loc);
    if (loc.kind == LOC_VERTEX) { simplex_swap(s, 0, loc.id); s.proj[0] = 1.0f; s.dim = 0; }
    else if (loc.kind == LOC_EDGE) {
      if (loc.id == 0) { s.proj[0] = loc.bc[0]; s.proj[1] = loc.bc[1]; }
      else if (loc.id == 1) { simplex_swap(s, 0, 2); s.proj[0] = loc.bc[1]; s.proj[1] = loc.bc[0]; }
      else { simplex_swap(s, 1, 2); s.proj[0] = loc.bc[0]; s.proj[1] = loc.bc[1]; }
      s.dim = 1;
    } else if (loc.kind == LOC_FACE) {
      s.proj[0] = loc.bc[0]; s.proj[1] = loc.bc[1]; s.proj[2] = loc.bc[2];
    }
    return p;
  } else {
    V3 p = project_tetrahedron(s.v[0].p, s.v[1].p, s.v[2].p, s.v[3].p, o, &loc);
    if (loc.kind == LOC_VERTEX) { simplex_swap(s, 0, loc.id); s.proj[0] = 1.0f; s.dim = 0; }
    else if (loc.kind == LOC_EDGE) {
      int i = loc.id;
      if (i == 1) simplex_swap(s, 1, 2);
      else if (i == 2) simplex_swap(s, 1, 3);
      else if (i == 3) simplex_swap(s, 0, 2);
      else if (i == 4) simplex_swap(s, 0, 3);
      else if (i == 5) { simplex_swap(s, 0, 2); simplex_swap(s, 1, 3); }
      if (i == 3 || i == 4) { s.proj[0] = loc.bc[1]; s.proj[1] = loc.bc[0]; }
      else { s.proj[0] = loc.bc[0]; s.proj[1] = loc.bc[1]; }
      s.dim = 1;
    } else if (loc.kind == LOC_FACE) {
      int i = loc.id;
      if (i == 0) { s.proj[0] = loc.bc[0]; s.proj[1] = loc.bc[1]; s.proj[2] = loc.bc[2]; }
      else if (i == 1) { s.v[2] = s.v[3]; s.proj[0] = loc.bc[0]; s.proj[1] = loc.bc[1]; s.proj[2] = loc.bc[2]; }
      else if (i == 2) { s.v[1] = s.v[3]; s.proj[0] = loc.bc[0]; s.proj[1] = loc.bc[2]; s.proj[2] = loc.bc[1]; }
      else { s.v[0] = s.v[3]; s.proj[0] = loc.bc[2]; s.proj[1] = loc.bc[0]; s.proj[2] = loc.bc[1]; }
      s.dim = 2;
    }
    return p;
  }
}

// ---------------- GJK ----------------

enum : int { GJK_INTERSECTION = 0, GJK_CLOSEST = 1, GJK_NO_INTERSECTION = 3 };
struct GjkOut {
  int kind;
  V3 p1, p2, dir;
};

__device__ __forceinline__ void gjk_result(const Simplex& s, bool prev, V3* p1, V3* p2) {
  V3 a = v3(0.f, 0.f, 0.f), b = v3(0.f, 0.f, 0.f);
  if (prev) {
    for (int i = 0; i < s.prev_dim + 1; ++i) {
      float c = s.prev_proj[i];
      const CSO& p = s.v[s.prev_v[i]];
      a = a + p.o1 * c;
      b = b + p.o2 * c;
    }
  } else {
    for (int i = 0; i < s.dim + 1; ++i) {
      float c = s.proj[i];
      a = a + s.v[i].o1 * c;
      b = b + s.v[i].o2 * c;
    }
  }
  *p1 = a;
  *p2 = b;
}

// gjk::closest_points with exact_dist = true (gjk.rs:353-453). `iters` counts support evaluations;
// `sup(dir)` is CSOPoint::from_shapes(pos12, g1, g2, dir).
template <class Sup>
__device__ __forceinline__ GjkOut gjk_closest_points_t(Sup sup, float max_dist, Simplex& s, uint32_t* iters) {
  const float eps_tol = GJK_EPS_TOL;
  const float eps_rel = sqrtf(eps_tol);
  GjkOut r;
  V3 proj = simplex_project_origin_and_reduce(s);
  V3 old_dir, u;
  if (try_normalize(proj, 0.0f, &u)) old_dir = -u;
  else { r.kind = GJK_INTERSECTION; return r; }
  float max_bound = FLT_MAX;
  V3 dir;
  int niter = 0;
  for (;;) {
    float old_max_bound = max_bound;
    float nb;
    if (try_normalize(-proj, eps_tol, &u, &nb)) { dir = u; max_bound = nb; }
    else { r.kind = GJK_INTERSECTION; return r; }
    if (max_bound >= old_max_bound) {
      r.kind = GJK_CLOSEST; r.dir = old_dir;
      gjk_result(s, true, &r.p1, &r.p2);
      return r;
    }
    (*iters)++;
    CSO cso = sup(dir);
    float min_bound = -dot(dir, cso.p);
    if (min_bound > max_dist) { r.kind = GJK_NO_INTERSECTION; r.dir = dir; return r; }
    if (max_bound - min_bound <= eps_rel * max_bound) {
      r.kind = GJK_CLOSEST; r.dir = dir;
      gjk_result(s, false, &r.p1, &r.p2);
      return r;
    }
    if (!simplex_add(s, cso)) {
      r.kind = GJK_CLOSEST; r.dir = dir;
      gjk_result(s, false, &r.p1, &r.p2);
      return r;
    }
    old_dir = dir;
    proj = simplex_project_origin_and_reduce(s);
    if (s.dim == 3) {
      if (min_bound >= eps_tol) {
        r.kind = GJK_CLOSEST; r.dir = old_dir;
        gjk_result(s, true, &r.p1, &r.p2);
        return r;
      }
      r.kind = GJK_INTERSECTION;
      return r;
    }
    niter += 1;
    if (niter == 100) { r.kind = GJK_NO_INTERSECTION; r.dir = v3(1.f, 0.f, 0.f); return r; }
  }
}

// The per-thread form.
static __device__ __noinline__ GjkOut gjk_closest_points(const Pose& pos12, const ShapeDev& g1, const ShapeDev& g2, float max_dist, Simplex& s,
                                                  uint32_t* iters) {
  return gjk_closest_points_t([&](V3 d) { return cso_from_shapes(pos12, g1, g2, d); }, max_dist, s, iters);
}

}  // namespace pg
