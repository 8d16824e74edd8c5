// Batched persistent contact manifolds (parry3d's ContactManifold) for convex pairs of balls,
// cuboids, capsules and ConvexPolyhedron hulls, updated in place from one frame to the next.
//
// Paths relative to the parry repository:
//   record update / matching  src/query/contact_manifolds/contact_manifold.rs:662-770
//   dispatch                  src/query/default_query_dispatcher.rs:749-831 (contact_manifold_convex_convex)
//   ball-ball                 src/query/contact_manifolds/contact_manifolds_ball_ball.rs:19-57
//   capsule-capsule (3-D)     src/query/contact_manifolds/contact_manifolds_capsule_capsule.rs:134-182
//   convex-ball               src/query/contact_manifolds/contact_manifolds_convex_ball.rs:20-145
//   cuboid-cuboid             src/query/contact_manifolds/contact_manifolds_cuboid_cuboid.rs:21-107,
//                             src/query/sat/sat_cuboid_cuboid.rs:59-279
//   polygonal features        src/query/contact_manifolds/contact_manifolds_pfm_pfm.rs:44-162,
//                             src/shape/polygonal_feature3d.rs:49-439, src/shape/cuboid.rs:267-352
//   segment-segment           src/query/closest_points/closest_points_segment_segment.rs:41-111
//   clipping                  src/query/clip/clip_segment_segment.rs
//
// Pipeline (one stream):
//   k_mf_classify     status of each pair and its generator kind (pairs binned by kind).
//   k_mf_kind<K>      one thread per pair of bin K. Analytic generators finish in place; the
//                     polygonal-feature path (cuboid/capsule/hull pairs) runs GJK and the hull-ball
//                     path a GJK point projection; when GJK ends inside, (pair, simplex, tag) goes to
//                     the EPA queue.
//   k_manifolds_epa   persistent loop over the queue (epa_device.cuh workspace slots), then the same
//                     feature clipping as the main kernel.
// Every step keeps the reference's evaluation order (compiled with --fmad=false) so the records match
// the f32 reference bit for bit.
#include "internal.hpp"
#include "epa_device.cuh"
#include "contact_device.cuh"
#include "pseudo_device.cuh"
#include "tri_ray_device.cuh"
#include <cstring>

using namespace pg;

namespace {

constexpr int MF_THREADS = 128;
constexpr int MF_EPA_THREADS = 64;
constexpr int MF_MAX = PARRYGPU_MANIFOLD_MAX_POINTS;
constexpr int MF_WORDS = 8 + 10 * MF_MAX;
static_assert(sizeof(parrygpu_manifold) == 4 * MF_WORDS, "record layout");

constexpr float COS_1_DEGREES = 0.99984769515f;
constexpr float COS_FRAC_PI_8 = 0.92387953251f;
constexpr uint32_t PF_UNKNOWN = 0;
__device__ __forceinline__ uint32_t pf_vertex(uint32_t c) { return (1u << 30) | c; }
__device__ __forceinline__ uint32_t pf_edge(uint32_t c) { return (2u << 30) | c; }
__device__ __forceinline__ uint32_t pf_face(uint32_t c) { return (3u << 30) | c; }

// One manifold record in global memory: n_points, status, local_n1, local_n2, then points of
// {local_p1, local_p2, dist, fid1, fid2, data}.
struct Rec {
  uint32_t* w;
  __device__ __forceinline__ float f(int i) const { return __uint_as_float(w[i]); }
  __device__ __forceinline__ void setf(int i, float v) const { w[i] = __float_as_uint(v); }
  __device__ __forceinline__ V3 v(int i) const { return v3(f(i), f(i + 1), f(i + 2)); }
  __device__ __forceinline__ void setv(int i, V3 a) const { setf(i, a.x); setf(i + 1, a.y); setf(i + 2, a.z); }
  __device__ __forceinline__ uint32_t n() const { uint32_t k = w[0]; return k > (uint32_t)MF_MAX ? (uint32_t)MF_MAX : k; }
  __device__ __forceinline__ static int pt(uint32_t i) { return 8 + 10 * (int)i; }
};

// The (fid1, fid2, data) of the previous points, for match_contacts.
struct OldPts {
  uint32_t n;
  uint32_t f1[MF_MAX], f2[MF_MAX];
  float d[MF_MAX];
};

__device__ __forceinline__ void save_old(const Rec& r, OldPts& o) {
  o.n = r.n();
  for (uint32_t i = 0; i < o.n; ++i) {
    int b = Rec::pt(i);
    o.f1[i] = r.w[b + 7];
    o.f2[i] = r.w[b + 8];
    o.d[i] = r.f(b + 9);
  }
}

// ContactManifold::match_contacts: the last old contact with the same feature pair wins.
__device__ __forceinline__ void match_contacts(const Rec& r, uint32_t n, const OldPts& o) {
  for (uint32_t i = 0; i < n; ++i) {
    int b = Rec::pt(i);
    uint32_t f1 = r.w[b + 7], f2 = r.w[b + 8];
    for (uint32_t j = 0; j < o.n; ++j)
      if (o.f1[j] == f1 && o.f2[j] == f2) r.setf(b + 9, o.d[j]);
  }
}

// manifold.points.push(TrackedContact::flipped(p1, p2, f1, f2, dist, flipped)); data = default.
struct Writer {
  Rec r;
  uint32_t n;
  bool overflow;
  __device__ __forceinline__ void push(V3 p1, V3 p2, uint32_t f1, uint32_t f2, float dist, bool flipped) {
    if (n >= (uint32_t)MF_MAX) { overflow = true; return; }
    int b = Rec::pt(n);
    if (!flipped) { r.setv(b, p1); r.setv(b + 3, p2); r.w[b + 7] = f1; r.w[b + 8] = f2; }
    else { r.setv(b, p2); r.setv(b + 3, p1); r.w[b + 7] = f2; r.w[b + 8] = f1; }
    r.setf(b + 6, dist);
    r.setf(b + 9, 0.0f);
    n++;
  }
};

// The reference's filter after a normal correction (contact_manifolds_pfm_pfm.rs:126-136,
// contact_manifolds_cuboid_triangle.rs:152-163): a point stays unless the unconstrained separation
// `dist` and the point's distance are both negative and the point is over five times deeper; kept
// points stay in order (Vec::retain).
__device__ __forceinline__ void retain_close_depths(const Rec& r, Writer* wr, float dist) {
  uint32_t k = 0;
  for (uint32_t i = 0; i < wr->n; ++i) {
    const int b = Rec::pt(i);
    const float pd = r.f(b + 6);
    if (dist >= 0.0f || pd >= 0.0f || pd >= dist * 5.0f) {
      if (k != i) {
        const int d = Rec::pt(k);
        for (int w = 0; w < 10; ++w) r.w[d + w] = r.w[b + w];
      }
      ++k;
    }
  }
  wr->n = k;
}

// TrackedContact::copy_geometry_from into point 0 (data kept).
__device__ __forceinline__ void copy_geometry0(const Rec& r, V3 p1, V3 p2, uint32_t f1, uint32_t f2, float dist, bool flipped) {
  int b = Rec::pt(0);
  if (!flipped) { r.setv(b, p1); r.setv(b + 3, p2); r.w[b + 7] = f1; r.w[b + 8] = f2; }
  else { r.setv(b, p2); r.setv(b + 3, p1); r.w[b + 7] = f2; r.w[b + 8] = f1; }
  r.setf(b + 6, dist);
}

// ContactManifold::try_update_contacts_eps (contact_manifold.rs:662-699).
__device__ __forceinline__ bool try_update_contacts(const Rec& r, const Pose& pos12, float angle_dot_threshold, float dist_sq_threshold) {
  uint32_t n = r.n();
  if (n == 0) return false;
  V3 ln1 = r.v(2);
  V3 ln2 = pose_rotate(pos12, r.v(5));
  if (-dot(ln1, ln2) < angle_dot_threshold) return false;
  for (uint32_t i = 0; i < n; ++i) {
    int b = Rec::pt(i);
    V3 p1 = r.v(b);
    V3 p2 = pose_point(pos12, r.v(b + 3));
    float dist = dot(p2 - p1, ln1);
    if (dist * r.f(b + 6) < 0.0f) return false;
    V3 np1 = p2 - ln1 * dist;
    V3 d = p1 - np1;
    if (dot(d, d) > dist_sq_threshold) return false;
    r.setf(b + 6, dist);
    r.setv(b, np1);
  }
  return true;
}

// approx::ulps_eq with epsilon = f32::EPSILON and max_ulps = 4.
__device__ __forceinline__ bool ulps_eq(float a, float b) {
  float d = a > b ? a - b : b - a;
  if (d <= EPS) return true;
  if (isnan(a) || isnan(b)) return false;
  if (signbit(a) != signbit(b)) return false;
  int ia = __float_as_int(a), ib = __float_as_int(b);
  int diff = ia <= ib ? ib - ia : ia - ib;
  return diff <= 4;
}

__device__ __forceinline__ float clamp01(float x) { return x > 1.0f ? 1.0f : (x < 0.0f ? 0.0f : x); }

// closest_points_segment_segment_with_locations_nD: the two segment parameters.
template <class Vec, class Dot>
__device__ __forceinline__ void seg_seg_params(Vec a0, Vec a1, Vec b0, Vec b1, Dot dotf, float* s_out, float* t_out) {
  Vec d1 = a1 - a0, d2 = b1 - b0, r = a0 - b0;
  float a = dotf(d1, d1), e = dotf(d2, d2), f = dotf(d2, r);
  float s, t;
  if (a <= EPS && e <= EPS) { s = 0.0f; t = 0.0f; }
  else if (a <= EPS) { s = 0.0f; t = clamp01(f / e); }
  else {
    float c = dotf(d1, r);
    if (e <= EPS) { t = 0.0f; s = clamp01(-c / a); }
    else {
      float b = dotf(d1, d2);
      float ae = a * e, bb = b * b;
      float denom = ae - bb;
      if (denom > EPS && !ulps_eq(ae, bb)) s = clamp01((b * f - c * e) / denom);
      else s = 0.0f;
      t = (b * s + f) / e;
      if (t < 0.0f) { t = 0.0f; s = clamp01(-c / a); }
      else if (t > 1.0f) { t = 1.0f; s = clamp01((b - c) / a); }
    }
  }
  *s_out = s;
  *t_out = t;
}
// SegmentPointLocation::barycentric_coordinates
__device__ __forceinline__ void seg_bc(float s, float* b0, float* b1) {
  if (s == 0.0f) { *b0 = 1.0f; *b1 = 0.0f; }
  else if (s == 1.0f) { *b0 = 0.0f; *b1 = 1.0f; }
  else { *b0 = 1.0f - s; *b1 = s; }
}

struct P2 {
  float x, y;
};
__device__ __forceinline__ P2 operator-(P2 a, P2 b) { return P2{a.x - b.x, a.y - b.y}; }
__device__ __forceinline__ float dot2(P2 a, P2 b) { return a.x * b.x + a.y * b.y; }
__device__ __forceinline__ float perp2(P2 a, P2 b) { return a.x * b.y - a.y * b.x; }

// WBasis::orthonormal_basis for a 3-D vector (wops.rs:96-109).
__device__ __forceinline__ void orthonormal_basis(V3 v, V3* b0, V3* b1) {
  float sign = copysignf(1.0f, v.z);
  float a = -1.0f / (sign + v.z);
  float b = v.x * v.y * a;
  *b0 = v3(1.0f + sign * v.x * v.x * a, sign * b, -sign * v.x);
  *b1 = v3(b, sign + v.y * v.y * a, -v.y);
}

struct PolyFeature {
  V3 v[4];
  uint32_t vids[4], eids[4], fid;
  int nv;
};

__constant__ uint32_t c_cuboid_vids[3][2][4] = {
    {{0b000, 0b010, 0b011, 0b001}, {0b100, 0b110, 0b111, 0b101}},
    {{0b000, 0b100, 0b101, 0b001}, {0b010, 0b110, 0b111, 0b011}},
    {{0b000, 0b010, 0b110, 0b100}, {0b001, 0b011, 0b111, 0b101}}};
__constant__ uint32_t c_cuboid_eids[3][2][4] = {
    {{0b11010000, 0b11011010, 0b11011001, 0b11001000}, {0b11110100, 0b11111110, 0b11111101, 0b11101100}},
    {{0b11100000, 0b11101100, 0b11101001, 0b11001000}, {0b11110010, 0b11111110, 0b11111011, 0b11011010}},
    {{0b11010000, 0b11110010, 0b11110100, 0b11100000}, {0b11011001, 0b11111011, 0b11111101, 0b11101001}}};

// Cuboid::support_face (cuboid.rs:267-352): the face whose normal is the largest |component| of dir.
__device__ __forceinline__ PolyFeature cuboid_support_face(V3 he, V3 dir) {
  float ax = fabsf(dir.x), ay = fabsf(dir.y), az = fabsf(dir.z);
  // Vector::iamax: first index of the maximum
  int ia = 0;
  float best = ax;
  if (ay > best) { ia = 1; best = ay; }
  if (az > best) { ia = 2; }
  float d = ia == 0 ? dir.x : (ia == 1 ? dir.y : dir.z);
  float sign = copysignf(1.0f, d);
  PolyFeature f;
  if (ia == 0) {
    f.v[0] = v3(he.x * sign, he.y, he.z); f.v[1] = v3(he.x * sign, -he.y, he.z);
    f.v[2] = v3(he.x * sign, -he.y, -he.z); f.v[3] = v3(he.x * sign, he.y, -he.z);
  } else if (ia == 1) {
    f.v[0] = v3(he.x, he.y * sign, he.z); f.v[1] = v3(-he.x, he.y * sign, he.z);
    f.v[2] = v3(-he.x, he.y * sign, -he.z); f.v[3] = v3(he.x, he.y * sign, -he.z);
  } else {
    f.v[0] = v3(he.x, he.y, he.z * sign); f.v[1] = v3(he.x, -he.y, he.z * sign);
    f.v[2] = v3(-he.x, -he.y, he.z * sign); f.v[3] = v3(-he.x, he.y, he.z * sign);
  }
  int si = ((int)sign + 1) / 2;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    f.vids[i] = pf_vertex(c_cuboid_vids[ia][si][i] * 2u);
    f.eids[i] = pf_edge(c_cuboid_eids[ia][si][i]);
  }
  f.fid = pf_face((uint32_t)(ia + si * 3 + 10));
  f.nv = 4;
  return f;
}

// PolygonalFeature::from(Segment) for a capsule axis (polygonal_feature3d.rs:49-59).
__device__ __forceinline__ PolyFeature segment_feature(float hh) {
  PolyFeature f;
  V3 a = v3(0.f, -hh, 0.f), b = v3(0.f, hh, 0.f);
  f.v[0] = a; f.v[1] = b; f.v[2] = b; f.v[3] = b;
  f.vids[0] = pf_vertex(0); f.vids[1] = pf_vertex(1); f.vids[2] = pf_vertex(1); f.vids[3] = pf_vertex(1);
#pragma unroll
  for (int i = 0; i < 4; ++i) f.eids[i] = pf_edge(0);
  f.fid = pf_face(0);
  f.nv = 2;
  return f;
}

// PolygonalFeature::from(Triangle) (polygonal_feature3d.rs:37-47): the whole triangle whatever the
// direction (Triangle::support_face, triangle.rs:280-282).
__device__ __forceinline__ PolyFeature triangle_feature(const ShapeDev& s) {
  PolyFeature f;
  f.v[0] = ldv(s.pts); f.v[1] = ldv(s.pts + 3); f.v[2] = ldv(s.pts + 6); f.v[3] = f.v[2];
  const uint32_t ids[4] = {0u, 1u, 2u, 2u};
#pragma unroll
  for (int i = 0; i < 4; ++i) { f.vids[i] = pf_vertex(ids[i]); f.eids[i] = pf_edge(ids[i]); }
  f.fid = pf_face(0);
  f.nv = 3;
  return f;
}

// approx::relative_eq (f32::EPSILON absolute and relative) on each component.
__device__ __forceinline__ bool relative_eq_f(float a, float b) {
  if (a == b) return true;
  if (isinf(a) || isinf(b)) return false;
  float d = fabsf(a - b);
  if (d <= EPS) return true;
  float largest = fabsf(b) > fabsf(a) ? fabsf(b) : fabsf(a);
  return d <= largest * EPS;
}

// Triangle::project_local_point_and_get_feature (point_triangle.rs:26-48, 3-D): the solid location,
// is_inside = relative_eq!(projection, point) (compute_result, :5-18), OnSolid inside.
__device__ __forceinline__ uint32_t triangle_projection_feature(const ShapeDev& s, V3 pt, V3* proj, bool* inside) {
  Loc loc;
  *proj = project_triangle(ldv(s.pts), ldv(s.pts + 3), ldv(s.pts + 6), pt, &loc);
  if (loc.kind == LOC_SOLID) { *inside = true; return pf_face(0); }
  *inside = relative_eq_f(proj->x, pt.x) && relative_eq_f(proj->y, pt.y) && relative_eq_f(proj->z, pt.z);
  if (loc.kind == LOC_VERTEX) return pf_vertex((uint32_t)loc.id);
  if (loc.kind == LOC_EDGE) return pf_edge((uint32_t)loc.id);
  return pf_face((uint32_t)loc.id);
}

// One ConvexPolyhedron's topology (hull-local ids); see parrygpu_polyhedra.
struct HullDev {
  const float* face_normals;    // this hull's faces x 3
  const uint32_t* face_ranges;  // this hull's faces x 2 (global first entry, count)
  const uint32_t* face_vertices;
  const uint32_t* face_edges;
  const uint32_t* vertex_ranges;  // this hull's vertices x 2 (global first entry, count)
  const uint32_t* vertex_faces;
  const uint32_t* vertex_edges;
  const float* edge_dirs;  // this hull's edges x 3
  uint32_t n_faces, n_edges;
  uint64_t n_face_entries, n_vertex_entries;
};

// The topology of convex shape i (params.z = hull index + 1), checked against the array sizes.
__device__ __forceinline__ bool load_hull(const ShapeArrays& sh, uint32_t i, HullDev* h) {
  const PolyArrays& P = sh.poly;
  if (!P.hulls || sh.types[i] != SH_CONVEX) return false;
  float4 prm = sh.params[i];
  uint32_t h1 = __float_as_uint(prm.z);
  if (h1 == 0 || h1 > P.n_hulls) return false;
  const uint32_t* r = P.hulls + 8 * (size_t)(h1 - 1);
  uint32_t first_vertex = __float_as_uint(prm.x), nv = __float_as_uint(prm.y);
  if (r[3] == 0 || r[0] != first_vertex || r[1] != nv) return false;
  if ((uint64_t)r[2] + r[3] > P.n_faces || (uint64_t)r[4] + r[5] > P.n_edges) return false;
  h->face_normals = P.face_normals + 3 * (size_t)r[2];
  h->face_ranges = P.face_ranges + 2 * (size_t)r[2];
  h->face_vertices = P.face_vertices;
  h->face_edges = P.face_edges;
  h->vertex_ranges = P.vertex_ranges + 2 * (size_t)first_vertex;
  h->vertex_faces = P.vertex_faces;
  h->vertex_edges = P.vertex_edges;
  h->edge_dirs = P.edge_dirs + 3 * (size_t)r[4];
  h->n_faces = r[3];
  h->n_edges = r[5];
  h->n_face_entries = P.n_face_entries;
  h->n_vertex_entries = P.n_vertex_entries;
  return true;
}

// ConvexPolyhedron::local_support_feature (convex_polyhedron.rs:959-991). Out-of-range topology
// indices set *bad and yield an empty feature.
static __device__ __noinline__ PolyFeature hull_support_feature(const ShapeDev& s, const HullDev& h, V3 dir, bool* bad) {
  uint32_t best = 0;
  float best_dot = dot(ldv(h.face_normals), dir);
  for (uint32_t f = 1; f < h.n_faces; ++f) {
    float d = dot(ldv(h.face_normals + 3 * f), dir);
    if (d > best_dot) { best = f; best_dot = d; }
  }
  PolyFeature out;
#pragma unroll
  for (int i = 0; i < 4; ++i) { out.v[i] = v3(0.f, 0.f, 0.f); out.vids[i] = 0; out.eids[i] = 0; }
  uint32_t first = h.face_ranges[2 * best], num = min(h.face_ranges[2 * best + 1], 4u);
  out.fid = pf_face(best);
  out.nv = 0;
  if ((uint64_t)first + num > h.n_face_entries) { *bad = true; return out; }
  for (uint32_t i = 0; i < num; ++i) {
    uint32_t vid = h.face_vertices[first + i], eid = h.face_edges[first + i];
    if (vid >= s.npts || eid >= h.n_edges) { *bad = true; out.nv = 0; return out; }
    out.v[i] = ldv(s.pts + 3 * vid);
    out.vids[i] = pf_vertex(vid);
    out.eids[i] = pf_edge(eid);
  }
  out.nv = (int)num;
  return out;
}

// sin / cos of (PI / 180 as f32), correctly rounded: ConvexPolyhedron::support_feature_id_toward's
// eps (convex_polyhedron.rs:919-922).
constexpr float HULL_SEPS = 0.017452406f;
constexpr float HULL_CEPS = 0.9998477f;

// ConvexPolyhedron::support_feature_id_toward_eps (convex_polyhedron.rs:885-917) as a PackedFeatureId.
static __device__ __noinline__ uint32_t hull_support_feature_id(const ShapeDev& s, const HullDev& h, V3 dir, bool* bad) {
  uint32_t vid = 0;
  float best = dot(ldv(s.pts), dir);
  for (uint32_t i = 1; i < s.npts; ++i) {
    float d = dot(ldv(s.pts + 3 * i), dir);
    if (d > best) { best = d; vid = i; }
  }
  uint32_t first = h.vertex_ranges[2 * vid], num = h.vertex_ranges[2 * vid + 1];
  if ((uint64_t)first + num > h.n_vertex_entries) { *bad = true; return PF_UNKNOWN; }
  for (uint32_t i = 0; i < num; ++i) {
    uint32_t f = h.vertex_faces[first + i];
    if (f >= h.n_faces) { *bad = true; return PF_UNKNOWN; }
    if (dot(ldv(h.face_normals + 3 * f), dir) >= HULL_CEPS) return pf_face(f);
  }
  for (uint32_t i = 0; i < num; ++i) {
    uint32_t e = h.vertex_edges[first + i];
    if (e >= h.n_edges) { *bad = true; return PF_UNKNOWN; }
    if (fabsf(dot(ldv(h.edge_dirs + 3 * e), dir)) <= HULL_SEPS) return pf_edge(e);
  }
  return pf_vertex(vid);
}

// clip_segment_segment (clip_segment_segment.rs): the two clipped points (p1, p2) and their
// feature codes (0 = first vertex, 1 = edge, 2 = second vertex).
struct ClipPt {
  V3 p1, p2;
  int f1, f2;
};
__device__ __forceinline__ bool clip_segment_segment(V3 s10, V3 s11, V3 s20, V3 s21, ClipPt* ca, ClipPt* cb) {
  V3 tangent1 = s11 - s10;
  float sq = dot(tangent1, tangent1);
  float r1a = 0.0f, r1b = sq;
  float r2a = dot(s20 - s10, tangent1), r2b = dot(s21 - s10, tangent1);
  int f1a = 0, f1b = 2, f2a = 0, f2b = 2;
  if (r1b < r1a) { float t = r1a; r1a = r1b; r1b = t; int u = f1a; f1a = f1b; f1b = u; V3 w = s10; s10 = s11; s11 = w; }
  if (r2b < r2a) { float t = r2a; r2a = r2b; r2b = t; int u = f2a; f2a = f2b; f2b = u; V3 w = s20; s20 = s21; s21 = w; }
  if (r2a > r1b || r1a > r2b) return false;
  float l1 = r1b - r1a, l2 = r2b - r2a;
  if (r2a > r1a) {
    float bc = (r2a - r1a) / l1;
    *ca = ClipPt{s10 + tangent1 * bc, s20, 1, f2a};
  } else {
    float bc = (r1a - r2a) / l2;
    *ca = ClipPt{s10, s20 + (s21 - s20) * bc, f1a, 1};
  }
  if (r2b < r1b) {
    float bc = (r2b - r1a) / l1;
    *cb = ClipPt{s10 + tangent1 * bc, s21, 1, f2b};
  } else {
    float bc = (r1b - r2a) / l2;
    *cb = ClipPt{s11, s20 + (s21 - s20) * bc, f1b, 1};
  }
  return true;
}

// polygonal_feature3d.rs closest_points_line2d: false when the lines are parallel.
__device__ __forceinline__ bool closest_points_line2d(P2 e10, P2 e11, P2 e20, P2 e21, float* s_out, float* t_out) {
  P2 d1 = e11 - e10, d2 = e21 - e20, r = e10 - e20;
  float a = dot2(d1, d1), e = dot2(d2, d2), f = dot2(d2, r);
  if (a <= EPS && e <= EPS) { *s_out = 0.0f; *t_out = 0.0f; return true; }
  if (a <= EPS) { *s_out = 0.0f; *t_out = f / e; return true; }
  float c = dot2(d1, r);
  if (e <= EPS) { *s_out = -c / a; *t_out = 0.0f; return true; }
  float b = dot2(d1, d2);
  float ae = a * e, bb = b * b;
  float denom = ae - bb;
  if (denom <= EPS || ulps_eq(ae, bb)) return false;
  float s = (b * f - c * e) / denom;
  *s_out = s;
  *t_out = (b * s + f) / e;
  return true;
}

__device__ __forceinline__ int feat_at(const PolyFeature& f, int id) { return id == 0 ? (int)f.vids[0] : (id == 1 ? (int)f.eids[0] : (int)f.vids[1]); }

// PolygonalFeature::contacts (polygonal_feature3d.rs:76-439), features in their own local frames,
// sep1 in shape 1's frame.
static __device__ __noinline__ void feature_contacts(const Pose& pos12, V3 sep1, const PolyFeature& f1, const PolyFeature& f2, Writer& wr,
                                                     bool flipped) {
  V3 b0, b1;
  orthonormal_basis(sep1, &b0, &b1);
  if (f1.nv == 2 && f2.nv == 2) {
    // contacts_edge_edge
    P2 pe1[2] = {P2{dot(f1.v[0], b0), dot(f1.v[0], b1)}, P2{dot(f1.v[1], b0), dot(f1.v[1], b1)}};
    V3 v21[2] = {pose_point(pos12, f2.v[0]), pose_point(pos12, f2.v[1])};
    P2 pe2[2] = {P2{dot(v21[0], b0), dot(v21[0], b1)}, P2{dot(v21[1], b0), dot(v21[1], b1)}};
    P2 t1 = pe1[1] - pe1[0], t2 = pe2[1] - pe2[0];
    float n1 = sqrtf(dot2(t1, t1)), n2 = sqrtf(dot2(t2, t2));
    if (n1 > EPS && n2 > EPS) {
      P2 u1{t1.x / n1, t1.y / n1}, u2{t2.x / n2, t2.y / n2};
      bool parallel = dot2(u1, u2) >= COS_FRAC_PI_8;
      if (!parallel) {
        float s, t;
        seg_seg_params(pe1[0], pe1[1], pe2[0], pe2[1], [](P2 x, P2 y) { return dot2(x, y); }, &s, &t);
        float a0, a1, c0, c1;
        seg_bc(s, &a0, &a1);
        seg_bc(t, &c0, &c1);
        V3 lp1 = f1.v[0] * a0 + f1.v[1] * a1;
        V3 lp21 = v21[0] * c0 + v21[1] * c1;
        float dist = dot(lp21 - lp1, sep1);
        wr.push(lp1, pose_inv_point(pos12, lp21), f1.eids[0], f2.eids[0], dist, flipped);
        return;
      }
    }
    ClipPt ca, cb;
    if (clip_segment_segment(f1.v[0], f1.v[1], v21[0], v21[1], &ca, &cb)) {
      wr.push(ca.p1, pose_inv_point(pos12, ca.p2), (uint32_t)feat_at(f1, ca.f1), (uint32_t)feat_at(f2, ca.f2), dot(ca.p2 - ca.p1, sep1),
              flipped);
      wr.push(cb.p1, pose_inv_point(pos12, cb.p2), (uint32_t)feat_at(f1, cb.f1), (uint32_t)feat_at(f2, cb.f2), dot(cb.p2 - cb.p1, sep1),
              flipped);
    }
    return;
  }
  // contacts_face_face
  P2 pf1[4], pf2[4];
  V3 v21[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    pf1[i] = P2{dot(f1.v[i], b0), dot(f1.v[i], b1)};
    v21[i] = pose_point(pos12, f2.v[i]);
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) pf2[i] = P2{dot(v21[i], b0), dot(v21[i], b1)};
  if (f2.nv > 2) {
    V3 normal2_1 = cross(v21[2] - v21[1], v21[0] - v21[1]);
    float denom = dot(normal2_1, sep1);
    if (!(fabsf(denom) <= EPS)) {
      int last2 = f2.nv - 1;
      for (int i = 0; i < f1.nv; ++i) {
        P2 p1 = pf1[i];
        float sign = perp2(pf2[0] - pf2[last2], p1 - pf2[last2]);
        bool outside = false;
        for (int j = 0; j < last2; ++j) {
          float ns = perp2(pf2[j + 1] - pf2[j], p1 - pf2[j]);
          if (sign == 0.0f) sign = ns;
          else if (sign * ns < 0.0f) { outside = true; break; }
        }
        if (outside) continue;
        float dist = dot(v21[0] - f1.v[i], normal2_1) / denom;
        V3 lp1 = f1.v[i];
        V3 lp21 = f1.v[i] + sep1 * dist;
        wr.push(lp1, pose_inv_point(pos12, lp21), f1.vids[i], f2.fid, dist, flipped);
      }
    }
  }
  if (f1.nv > 2) {
    V3 normal1 = cross(f1.v[2] - f1.v[1], f1.v[0] - f1.v[1]);
    float denom = -dot(normal1, sep1);
    if (!(fabsf(denom) <= EPS)) {
      int last1 = f1.nv - 1;
      for (int i = 0; i < f2.nv; ++i) {
        P2 p2 = pf2[i];
        float sign = perp2(pf1[0] - pf1[last1], p2 - pf1[last1]);
        bool outside = false;
        for (int j = 0; j < last1; ++j) {
          float ns = perp2(pf1[j + 1] - pf1[j], p2 - pf1[j]);
          if (sign == 0.0f) sign = ns;
          else if (sign * ns < 0.0f) { outside = true; break; }
        }
        if (outside) continue;
        float dist = dot(f1.v[0] - v21[i], normal1) / denom;
        V3 lp21 = v21[i];
        V3 lp1 = v21[i] - sep1 * dist;
        wr.push(lp1, pose_inv_point(pos12, lp21), f1.fid, f2.vids[i], dist, flipped);
      }
    }
  }
  for (int j = 0; j < f2.nv; ++j) {
    int j1 = (j + 1) % f2.nv;
    P2 e20 = pf2[j], e21 = pf2[j1];
    for (int i = 0; i < f1.nv; ++i) {
      int i1 = (i + 1) % f1.nv;
      P2 e10 = pf1[i], e11 = pf1[i1];
      float s, t;
      if (closest_points_line2d(e10, e11, e20, e21, &s, &t)) {
        if (s > 0.0f && s < 1.0f && t > 0.0f && t < 1.0f) {
          V3 lp1 = f1.v[i] * (1.0f - s) + f1.v[i1] * s;
          V3 lp21 = v21[j] * (1.0f - t) + v21[j1] * t;
          float dist = dot(lp21 - lp1, sep1);
          wr.push(lp1, pose_inv_point(pos12, lp21), f1.eids[i], f2.eids[j], dist, flipped);
        }
      }
    }
  }
}

// PackedFeatureId of a point projected on a cuboid (point_aabb.rs:70-132, 3-D branch).
__device__ __forceinline__ uint32_t cuboid_projection_feature(V3 he, const PointProj& p) {
  float sh[3] = {p.shift.x, p.shift.y, p.shift.z}, l[3] = {p.point.x, p.point.y, p.point.z};
  float mn[3] = {-he.x, -he.y, -he.z}, mx[3] = {he.x, he.y, he.z};
  int nz = 0, last_zero = 0, last_nz = 0;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    if (sh[i] == 0.0f) { nz++; last_zero = i; }
    else last_nz = i;
  }
  if (nz == 3) {
    for (int i = 0; i < 3; ++i) {
      if (l[i] > mx[i] - EPS) return pf_face((uint32_t)i);
      if (l[i] <= mn[i] + EPS) return pf_face((uint32_t)(i + 3));
    }
    return PF_UNKNOWN;
  }
  float c[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) c[i] = (mn[i] + mx[i]) * 0.5f;
  if (nz == 2) return l[last_nz] < c[last_nz] ? pf_face((uint32_t)(last_nz + 3)) : pf_face((uint32_t)last_nz);
  uint32_t id = 0;
#pragma unroll
  for (int i = 0; i < 3; ++i)
    if (l[i] < c[i]) id |= 1u << i;
  if (nz == 0) return pf_vertex(id);
  return pf_edge((id << 2) | (uint32_t)last_zero);
}

__device__ __forceinline__ void set_normals(const Rec& r, V3 n1, V3 n2) {
  r.setv(2, n1);
  r.setv(5, n2);
}

// contact_manifold_ball_ball (contact_manifolds_ball_ball.rs:19-57)
__device__ __forceinline__ void mf_ball_ball(const Rec& r, const Pose& pos12, float ra, float rb, float prediction) {
  V3 dc = pos12.t;
  float cd = norm(dc);
  float dist = (cd - ra) - rb;
  if (dist < prediction) {
    V3 n1 = cd != 0.0f ? dc / cd : v3(0.f, 1.f, 0.f);
    V3 n2 = pose_inv_rotate(pos12, -n1);
    if (r.n() > 0) {
      copy_geometry0(r, n1 * ra, n2 * rb, pf_face(0), pf_face(0), dist, false);
    } else {
      Writer wr{r, 0, false};
      wr.push(n1 * ra, n2 * rb, pf_face(0), pf_face(0), dist, false);
      r.w[0] = 1;
    }
    set_normals(r, n1, n2);
  } else {
    r.w[0] = 0;
  }
}

// contact_manifold_capsule_capsule, 3-D (contact_manifolds_capsule_capsule.rs:134-182)
__device__ __forceinline__ void mf_capsule_capsule(const Rec& r, const Pose& pos12, float hh1, float r1, float hh2, float r2,
                                                   float prediction) {
  V3 a1 = v3(0.f, -hh1, 0.f), b1 = v3(0.f, hh1, 0.f);
  V3 a2 = pose_point(pos12, v3(0.f, -hh2, 0.f)), b2 = pose_point(pos12, v3(0.f, hh2, 0.f));
  float s, t;
  seg_seg_params(a1, b1, a2, b2, [](V3 x, V3 y) { return dot(x, y); }, &s, &t);
  float s0, s1, t0, t1;
  seg_bc(s, &s0, &s1);
  seg_bc(t, &t0, &t1);
  V3 lp1 = a1 * s0 + b1 * s1;
  V3 lp21 = a2 * t0 + b2 * t1;
  V3 n1;
  if (!try_normalize(lp21 - lp1, EPS, &n1)) n1 = v3(0.f, 1.f, 0.f);
  float dist = (dot(lp21 - lp1, n1) - r1) - r2;
  if (dist <= prediction) {
    V3 n2 = pose_inv_rotate(pos12, -n1);
    V3 p1 = lp1 + n1 * r1, p2 = pose_inv_point(pos12, lp21) + n2 * r2;
    if (r.n() > 0) {
      copy_geometry0(r, p1, p2, pf_face(0), pf_face(0), dist, false);
    } else {
      Writer wr{r, 0, false};
      wr.push(p1, p2, pf_face(0), pf_face(0), dist, false);
      r.w[0] = 1;
    }
    set_normals(r, n1, n2);
  } else {
    r.w[0] = 0;
  }
}

// Row + 1 of shape i's normal constraints in sh.pseudo, 0 = none (only TriMesh triangles of a mesh
// with FIX_INTERNAL_EDGES have some).
__device__ __forceinline__ uint32_t constraint_row(const ShapeArrays& sh, uint32_t i) {
  if (!sh.pseudo || i < sh.pseudo_first || sh.types[i] != SH_TRIANGLE) return 0u;
  return __float_as_uint(sh.params[i].z);
}

// The end of contact_manifold_convex_ball (contact_manifolds_convex_ball.rs:61-145) from the
// projection of the ball centre (pos12.t) on shape 1. c1 / c2: normal constraints of shape 1 / the
// ball (null = None); a corrected normal moves the shape-1 point to where the ray from the ball
// centre along it meets shape 1, which only a triangle (the one shape with constraints) supports.
__device__ __forceinline__ void finish_convex_ball(const Rec& r, const Pose& pos12, V3 lp1, bool inside, uint32_t fid1, float radius2,
                                                   float prediction, bool flipped, const TriPN* c1 = nullptr, const TriPN* c2 = nullptr,
                                                   const ShapeDev* s1 = nullptr) {
  V3 lp21 = pos12.t;
  V3 n1;
  float dist;
  if (!try_normalize(lp21 - lp1, 0.0f, &n1, &dist)) {
    if (!try_normalize(pos12.t, 0.0f, &n1)) n1 = v3(1.f, 0.f, 0.f);
    dist = 0.0f;
  }
  if (inside) { n1 = -n1; dist = -dist; }
  if (dist <= radius2 + prediction) {
    V3 n2 = pose_inv_rotate(pos12, -n1);
    if (c1 || c2) {
      const V3 uncorrected_n2 = n2;
      if (!project_local_normals(c1, c2, pos12, &n1, &n2)) { r.w[0] = 0; return; }
      if (!v3_eq(uncorrected_n2, n2)) {
        // Shape::cast_local_ray_and_get_normal(ray from the ball centre, f32::MAX, solid = false)
        const V3 rd = inside ? n1 : -n1;
        TriHit h;
        if (!s1 || s1->type != SH_TRIANGLE || !ray_triangle_toi(ldv(s1->pts), ldv(s1->pts + 3), ldv(s1->pts + 6), lp21, rd, &h) ||
            !(h.toi <= FLT_MAX)) {
          r.w[0] = 0;
          return;
        }
        lp1 = lp21 + rd * h.toi;
        dist = inside ? -h.toi : h.toi;
        fid1 = pf_face(h.fid);
      }
    }
    V3 lp2 = n2 * radius2;
    if (r.n() != 1) {
      Writer wr{r, 0, false};
      wr.push(lp1, lp2, fid1, pf_face(0), dist - radius2, flipped);
      r.w[0] = 1;
    } else {
      copy_geometry0(r, lp1, lp2, fid1, pf_face(0), dist - radius2, flipped);
    }
    if (flipped) set_normals(r, n2, n1);
    else set_normals(r, n1, n2);
  } else {
    r.w[0] = 0;
  }
}

// contact_manifold_convex_ball for a cuboid, capsule or triangle shape 1: analytic projection.
__device__ __forceinline__ void mf_convex_ball(const Rec& r, const Pose& pos12, const ShapeDev& s1, float radius2, float prediction,
                                               bool flipped, const TriPN* c1 = nullptr) {
  V3 lp21 = pos12.t;
  PointProj p;
  uint32_t fid1;
  if (s1.type == SH_CUBOID) {
    V3 he = v3(s1.a, s1.b, s1.c);
    p = project_cuboid(he, lp21);
    fid1 = cuboid_projection_feature(he, p);
  } else if (s1.type == SH_TRIANGLE) {
    fid1 = triangle_projection_feature(s1, lp21, &p.point, &p.inside);
  } else {
    p = project_capsule(s1.a, s1.b, lp21);
    fid1 = pf_face(0);
  }
  finish_convex_ball(r, pos12, p.point, p.inside, fid1, radius2, prediction, flipped, c1, nullptr, &s1);
}

// ConvexPolyhedron::project_local_point_and_get_feature's feature (point_support_map.rs:62-76).
__device__ __forceinline__ uint32_t hull_projection_feature(const ShapeDev& s, const HullDev& h, V3 pt, V3 proj, bool inside, bool* bad) {
  V3 dpt = pt - proj;
  V3 dir;
  if (try_normalize(inside ? -dpt : dpt, EPS, &dir)) return hull_support_feature_id(s, h, dir, bad);
  return PF_UNKNOWN;
}

__device__ __forceinline__ V3 cuboid_support(V3 he, V3 d) { return v3(copysignf(he.x, d.x), copysignf(he.y, d.y), copysignf(he.z, d.z)); }

// sat::cuboid_cuboid_find_local_separating_normal_oneway (sat_cuboid_cuboid.rs:255-279)
__device__ __forceinline__ float sat_normal_oneway(V3 h1, V3 h2, const Pose& pos12, V3* best_dir) {
  float best = -FLT_MAX;
  V3 bd = v3(0.f, 0.f, 0.f);
  float h1c[3] = {h1.x, h1.y, h1.z}, tc[3] = {pos12.t.x, pos12.t.y, pos12.t.z};
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    float sign = copysignf(1.0f, tc[i]);
    V3 axis1 = v3(i == 0 ? sign : 0.0f, i == 1 ? sign : 0.0f, i == 2 ? sign : 0.0f);
    V3 axis2 = pose_inv_rotate(pos12, -axis1);
    V3 pt2 = pose_point(pos12, cuboid_support(h2, axis2));
    float sep = comp(pt2, i) * sign - h1c[i];
    if (sep > best) { best = sep; bd = axis1; }
  }
  *best_dir = bd;
  return best;
}

// sat::cuboid_cuboid_find_local_separating_edge_twoway (sat_cuboid_cuboid.rs:59-184)
static __device__ __noinline__ float sat_edge_twoway(V3 h1, V3 h2, const Pose& pos12, V3* best_dir) {
  float best = -FLT_MAX;
  V3 bd = v3(0.f, 0.f, 0.f);
  V3 x2 = pose_rotate(pos12, v3(1.f, 0.f, 0.f)), y2 = pose_rotate(pos12, v3(0.f, 1.f, 0.f)), z2 = pose_rotate(pos12, v3(0.f, 0.f, 1.f));
  V3 axes[9] = {v3(0.0f, -x2.z, x2.y), v3(x2.z, 0.0f, -x2.x), v3(-x2.y, x2.x, 0.0f),
                v3(0.0f, -y2.z, y2.y), v3(y2.z, 0.0f, -y2.x), v3(-y2.y, y2.x, 0.0f),
                v3(0.0f, -z2.z, z2.y), v3(z2.z, 0.0f, -z2.x), v3(-z2.y, z2.x, 0.0f)};
#pragma unroll 1
  for (int k = 0; k < 9; ++k) {
    float n = norm(axes[k]);
    if (n > EPS) {
      V3 a = axes[k] / n;
      float signum = copysignf(1.0f, dot(pos12.t, a));
      V3 a1 = a * signum;
      V3 a2 = pose_inv_rotate(pos12, -a1);
      V3 lp1 = cuboid_support(h1, a1);
      V3 p2 = pose_point(pos12, cuboid_support(h2, a2));
      float sep = dot(p2 - lp1, a1);
      if (sep > best) { best = sep; bd = a1; }
    }
  }
  *best_dir = bd;
  return best;
}

// contact_manifold_cuboid_cuboid (contact_manifolds_cuboid_cuboid.rs:21-107)
static __device__ __noinline__ void mf_cuboid_cuboid(const Rec& r, const Pose& pos12, V3 h1, V3 h2, float prediction, bool* overflow) {
  if (try_update_contacts(r, pos12, COS_1_DEGREES, 1.0e-6f)) return;
  Pose pos21 = pose_inverse(pos12);
  V3 d1, d2, d3;
  float sep1 = sat_normal_oneway(h1, h2, pos12, &d1);
  if (sep1 > prediction) { r.w[0] = 0; return; }
  float sep2 = sat_normal_oneway(h2, h1, pos21, &d2);
  if (sep2 > prediction) { r.w[0] = 0; return; }
  float sep3 = sat_edge_twoway(h1, h2, pos12, &d3);
  if (sep3 > prediction) { r.w[0] = 0; return; }
  V3 best = d1;
  if (sep2 > sep1 && sep2 > sep3) best = pose_rotate(pos12, -d2);
  else if (sep3 > sep1) best = d3;
  OldPts old;
  save_old(r, old);
  V3 n2 = pose_rotate(pos21, -best);
  PolyFeature f1 = cuboid_support_face(h1, best);
  PolyFeature f2 = cuboid_support_face(h2, n2);
  Writer wr{r, 0, false};
  feature_contacts(pos12, best, f1, f2, wr, false);
  r.w[0] = wr.n;
  set_normals(r, best, n2);
  match_contacts(r, wr.n, old);
  *overflow |= wr.overflow;
}

// sat::cuboid_support_map_find_local_separating_normal_oneway (sat_cuboid_support_map.rs:54-73)
// with triangle 2 as the support map (support_point_toward = pos12 * local support).
__device__ __forceinline__ float sat_cuboid_triangle_normal_oneway(V3 he1, const ShapeDev& tri2, const Pose& pos12, V3* best_dir) {
  float best = -FLT_MAX;
  V3 bd = v3(0.f, 0.f, 0.f);
  const float h[3] = {he1.x, he1.y, he1.z};
#pragma unroll
  for (int i = 0; i < 3; ++i) {
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      float sign = k == 0 ? -1.0f : 1.0f;
      V3 axis1 = v3(i == 0 ? sign : 0.0f, i == 1 ? sign : 0.0f, i == 2 ? sign : 0.0f);
      V3 pt2 = world_support(tri2, pos12, -axis1);
      float sep = comp(pt2, i) * sign - h[i];
      if (sep > best) { best = sep; bd = axis1; }
    }
  }
  *best_dir = bd;
  return best;
}

// sat::point_cuboid_find_local_separating_normal_oneway (sat_cuboid_point.rs) with the triangle's
// first vertex and normal (triangle_cuboid_find_local_separating_normal_oneway, 3-D).
__device__ __forceinline__ float sat_triangle_cuboid_normal_oneway(const ShapeDev& tri1, V3 he2, const Pose& pos12, V3* best_dir) {
  float best = -FLT_MAX;
  V3 bd = v3(0.f, 0.f, 0.f);
  V3 a = ldv(tri1.pts), b = ldv(tri1.pts + 3), c = ldv(tri1.pts + 6);
  V3 n;
  if (try_normalize(cross(b - a, c - a), EPS, &n)) {  // Triangle::normal
    V3 axis1 = dot(pos12.t - a, n) >= 0.0f ? n : -n;
    V3 pt2 = pose_point(pos12, cuboid_support(he2, pose_inv_rotate(pos12, -axis1)));
    float sep = dot(pt2 - a, axis1);
    if (sep > best) { best = sep; bd = axis1; }
  }
  *best_dir = bd;
  return best;
}

// sat::cuboid_triangle_find_local_separating_edge_twoway (sat_cuboid_triangle.rs, 3-D)
static __device__ __noinline__ float sat_cuboid_triangle_edge_twoway(V3 he1, const ShapeDev& tri2, const Pose& pos12, V3* best_dir) {
  V3 a = pose_point(pos12, ldv(tri2.pts)), b = pose_point(pos12, ldv(tri2.pts + 3)), c = pose_point(pos12, ldv(tri2.pts + 6));
  V3 ab = b - a, bc = c - b, ca = a - c;
  V3 axes[9] = {v3(0.0f, -ab.z, ab.y), v3(ab.z, 0.0f, -ab.x), v3(-ab.y, ab.x, 0.0f),
                v3(0.0f, -bc.z, bc.y), v3(bc.z, 0.0f, -bc.x), v3(-bc.y, bc.x, 0.0f),
                v3(0.0f, -ca.z, ca.y), v3(ca.z, 0.0f, -ca.x), v3(-ca.y, ca.x, 0.0f)};
  float best = -FLT_MAX;
  V3 bd = axes[0];
#pragma unroll 1
  for (int i = 0; i < 9; ++i) {
    V3 axis = axes[i];
    float d0 = dot(axis, a), d1 = i < 6 ? dot(axis, c) : dot(axis, b);
    float n2 = dot(axis, axis);
    if (n2 > EPS) {
      float n = sqrtf(n2);
      float dot1 = dot(cuboid_support(he1, axis), axis) / n;
      float mn = d0 > d1 ? d1 : d0, mx = d0 > d1 ? d0 : d1;  // utils::sort2
      float sep_a = mn / n - dot1;
      float sep_b = -mx / n - dot1;
      if (sep_a > best) { best = sep_a; bd = axis / n; }
      if (sep_b > best) { best = sep_b; bd = -axis / n; }
    }
  }
  *best_dir = bd;
  return best;
}

// contact_manifold_cuboid_triangle (contact_manifolds_cuboid_triangle.rs:57-174, no normal
// constraints): the cuboid is shape 1 of the SAT; `flipped` when the triangle is the record's first
// shape (pos12: cuboid frame to triangle frame).
static __device__ __noinline__ void mf_cuboid_triangle(const Rec& r, const Pose& pos12, const Pose& pos21, V3 he1, const ShapeDev& tri2,
                                                       float prediction, bool flipped, bool* overflow, const float* pseudo, uint32_t j2) {
  if (try_update_contacts(r, flipped ? pos21 : pos12, COS_1_DEGREES, 1.0e-6f)) return;
  V3 d1, d2, d3;
  float sep1 = sat_cuboid_triangle_normal_oneway(he1, tri2, pos12, &d1);
  if (sep1 > prediction) { r.w[0] = 0; return; }
  float sep2 = sat_triangle_cuboid_normal_oneway(tri2, he1, pos21, &d2);
  if (sep2 > prediction) { r.w[0] = 0; return; }
  float sep3 = sat_cuboid_triangle_edge_twoway(he1, tri2, pos12, &d3);
  if (sep3 > prediction) { r.w[0] = 0; return; }
  V3 normal1 = d1;
  float dist = sep1;
  if (sep2 > sep1 && sep2 > sep3) { normal1 = pose_rotate(pos12, -d2); dist = sep2; }
  else if (sep3 > sep1) { normal1 = d3; dist = sep3; }
  V3 normal2 = pose_rotate(pos21, -normal1);
  // the triangle's normal constraints (the cuboid has none)
  TriPN pn;
  const TriPN* c2 = nullptr;
  if (j2) { pn = load_tri_pn(pseudo, j2 - 1); c2 = &pn; }
  if (c2 && !project_local_normals(nullptr, c2, pos12, &normal1, &normal2)) { r.w[0] = 0; return; }
  PolyFeature f1 = cuboid_support_face(he1, normal1);
  PolyFeature f2 = triangle_feature(tri2);
  OldPts old;
  save_old(r, old);
  Writer wr{r, 0, false};
  feature_contacts(pos12, normal1, f1, f2, wr, flipped);
  if (c2) retain_close_depths(r, &wr, dist);
  r.w[0] = wr.n;
  if (flipped) set_normals(r, normal2, normal1);
  else set_normals(r, normal1, normal2);
  match_contacts(r, wr.n, old);
  *overflow |= wr.overflow;
}

// The shape contact_manifold_pfm_pfm works on (a capsule is its segment plus a border radius).
__device__ __forceinline__ ShapeDev pfm_of(const ShapeDev& s, float* border) {
  ShapeDev p = s;
  *border = 0.0f;
  if (s.type == SH_CAPSULE) { p.type = SH_SEGMENT; *border = s.b; }
  return p;
}

__device__ __forceinline__ PolyFeature support_feature(const ShapeDev& s, const HullDev& h, V3 dir, bool* bad) {
  if (s.type == SH_CUBOID) return cuboid_support_face(v3(s.a, s.b, s.c), dir);
  if (s.type == SH_CONVEX) return hull_support_feature(s, h, dir, bad);
  if (s.type == SH_TRIANGLE) return triangle_feature(s);
  return segment_feature(s.a);
}

// The part of contact_manifold_pfm_pfm after the GJK / EPA query (contact_manifolds_pfm_pfm.rs:77-162);
// c1 / c2 = normal constraints of shape 1 / 2 (null = None).
static __device__ __noinline__ void finish_pfm(const Rec& r, const Pose& pos12, const ShapeDev& s1, const HullDev& h1, const ShapeDev& s2,
                                               const HullDev& h2, int kind, V3 p1, V3 p2, V3 dir, bool* overflow, bool* bad,
                                               const float* pseudo, uint32_t j1, uint32_t j2) {
  float br1 = s1.type == SH_CAPSULE ? s1.b : 0.0f, br2 = s2.type == SH_CAPSULE ? s2.b : 0.0f;
  TriPN pn1, pn2;
  const TriPN* c1 = nullptr;
  const TriPN* c2 = nullptr;
  if (j1) { pn1 = load_tri_pn(pseudo, j1 - 1); c1 = &pn1; }
  if (j2) { pn2 = load_tri_pn(pseudo, j2 - 1); c2 = &pn2; }
  OldPts old;
  save_old(r, old);
  Writer wr{r, 0, false};
  if (kind == GJK_CLOSEST) {
    V3 n1 = dir;
    V3 n2 = pose_inv_rotate(pos12, -dir);
    const float dist = dot(p2 - p1, n1);
    if ((c1 || c2) && !project_local_normals(c1, c2, pos12, &n1, &n2)) {
      r.w[0] = 0;  // discarded: points cleared, cached normals and the old points' data left as they were
      return;
    }
    PolyFeature f1 = support_feature(s1, h1, n1, bad), f2 = support_feature(s2, h2, n2, bad);
    feature_contacts(pos12, n1, f1, f2, wr, false);
    // the GJK point only while the normal is GJK's own direction
    if (v3_eq(n1, dir)) wr.push(p1, pose_inv_point(pos12, p2), PF_UNKNOWN, PF_UNKNOWN, dot(p2 - p1, n1), false);
    if (c1 || c2) retain_close_depths(r, &wr, dist);
    if (br1 != 0.0f || br2 != 0.0f) {
      for (uint32_t i = 0; i < wr.n; ++i) {
        int b = Rec::pt(i);
        r.setv(b, r.v(b) + n1 * br1);
        r.setv(b + 3, r.v(b + 3) + n2 * br2);
        r.setf(b + 6, r.f(b + 6) - (br1 + br2));
      }
    }
    set_normals(r, n1, n2);
  } else if (kind == GJK_NO_INTERSECTION) {
    r.setv(2, dir);
  } else {
    r.setv(2, v3(0.f, 0.f, 0.f));
  }
  r.w[0] = wr.n;
  match_contacts(r, wr.n, old);
  *overflow |= wr.overflow;
}

// Pair kinds with a manifold generator here: balls, cuboids, capsules, triangles, and convex shapes
// that carry ConvexPolyhedron topology.
__device__ __forceinline__ bool has_generator(const ShapeArrays& sh, uint32_t i, HullDev* h) {
  uint32_t t = sh.types[i];
  if (t == SH_BALL || t == SH_CUBOID || t == SH_CAPSULE || t == SH_TRIANGLE) return true;
  return t == SH_CONVEX && load_hull(sh, i, h);
}

// EPA queue tags of the manifold kernels.
enum : uint32_t { TAG_PFM = 0, TAG_BALL_SECOND = 1, TAG_BALL_FIRST = 2 };

// GJK projection of the ball centre `center` (in the hull's frame) onto the hull
// (point_support_map.rs:17-57 up to the EPA fallback): true with *proj when GJK ends outside,
// false with the simplex `s` for EPA.
__device__ __forceinline__ bool hull_project_gjk(const ShapeDev& cs, V3 center, V3* proj, Simplex& s, uint32_t* iters) {
  Pose m{0.f, 0.f, 0.f, 1.f, -center};
  Pose minv = pose_inverse(m);
  Pose m_inv{0.f, 0.f, 0.f, 1.f, center};
  ShapeDev origin;
  origin.type = SH_ORIGIN;
  V3 dir;
  if (!try_normalize(-m.t, EPS, &dir)) dir = v3(1.f, 0.f, 0.f);
  simplex_reset(s, cso_from_shapes(m_inv, cs, origin, dir));
  GjkOut g = gjk_closest_points(minv, cs, origin, FLT_MAX, s, iters);
  if (g.kind == GJK_CLOSEST) { *proj = g.p1; return true; }
  return false;
}

// `d_n` (may be null) holds a device-side pair count; the kernel then handles min(n, *d_n) pairs.
// The pairs are binned by generator kind first (k_mf_classify), then each kind runs its own small
// kernel over its bin: warps see one code path, the simple kinds keep few registers, and the
// instruction cache holds one generator at a time.
// The polyhedral pairs (contact_manifold_pfm_pfm) are split by shape kinds - cuboid-capsule,
// cuboid-hull, capsule-hull, hull-hull, any with a triangle - so that a warp runs one support and
// feature path; one kernel (k_mf_kind<MK_PFM>) runs the five bins. Cuboid-triangle pairs have their
// own generator (SAT, contact_manifolds_cuboid_triangle.rs).
enum : uint32_t {
  MK_BALL_BALL = 0, MK_CUBOID_CUBOID, MK_CAPSULE_CAPSULE, MK_CONVEX_BALL, MK_HULL_BALL,
  MK_PFM, MK_PFM_CUBOID_HULL, MK_PFM_CAPSULE_HULL, MK_PFM_HULL_HULL, MK_PFM_TRIANGLE, MK_CUBOID_TRIANGLE, MK_KINDS
};
// counters: [0] EPA queue length, [1..3] GJK / EPA stats, [4 + kind] bin lengths, [15] learned-seed
// list length
constexpr int MF_CTR_BINS = 4;
constexpr int MF_CTR_SEED = 15;
constexpr size_t MF_CTR_BYTES = 128;
static_assert(MF_CTR_BINS + MK_KINDS <= MF_CTR_SEED, "the 128-byte counter block holds every bin length and the seed count");

__device__ __forceinline__ uint32_t manifold_kind(uint32_t t1, uint32_t t2) {
  if (t1 == SH_BALL && t2 == SH_BALL) return MK_BALL_BALL;
  if (t1 == SH_CUBOID && t2 == SH_CUBOID) return MK_CUBOID_CUBOID;
  if (t1 == SH_CAPSULE && t2 == SH_CAPSULE) return MK_CAPSULE_CAPSULE;
  if (t1 == SH_BALL || t2 == SH_BALL) return (t1 == SH_CONVEX || t2 == SH_CONVEX) ? MK_HULL_BALL : MK_CONVEX_BALL;
  if ((t1 == SH_CUBOID && t2 == SH_TRIANGLE) || (t1 == SH_TRIANGLE && t2 == SH_CUBOID)) return MK_CUBOID_TRIANGLE;
  if (t1 == SH_TRIANGLE || t2 == SH_TRIANGLE) return MK_PFM_TRIANGLE;
  const bool h1 = t1 == SH_CONVEX, h2 = t2 == SH_CONVEX;
  if (h1 && h2) return MK_PFM_HULL_HULL;
  if (h1 || h2) return (h1 ? t2 : t1) == SH_CUBOID ? MK_PFM_CUBOID_HULL : MK_PFM_CAPSULE_HULL;
  return MK_PFM;  // cuboid-capsule
}

// Status of each pair (invalid / unsupported records keep their content) and its bin, appended with
// warp-aggregated atomics. A pair (PARRYGPU_PAIR_NONE, PARRYGPU_PAIR_NONE) is an empty slot: skipped. `d_n` (may be null) holds a device-side pair count: min(n, *d_n) pairs.
// With `seed_list`, the polyhedral pairs whose record holds no cached normal (the pairs that take a
// learned GJK start direction) are listed too, their count in ctr[MF_CTR_SEED].
__global__ void __launch_bounds__(MF_THREADS) k_mf_classify(ShapeArrays sh, const uint32_t* __restrict__ pairs, uint64_t n,
                                                            uint32_t* __restrict__ recs, uint32_t* __restrict__ bins, uint64_t stride,
                                                            unsigned long long* __restrict__ ctr, uint32_t* __restrict__ err,
                                                            const unsigned long long* __restrict__ d_n, uint32_t* __restrict__ seed_list) {
  uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (d_n && *d_n < n) n = *d_n;
  uint32_t kind = MK_KINDS;
  bool seed = false;
  if (k < n) {
    Rec r{recs + (size_t)k * MF_WORDS};
    uint32_t a = pairs[2 * k], b = pairs[2 * k + 1];
    HullDev h1, h2;
    if (a == PARRYGPU_PAIR_NONE && b == PARRYGPU_PAIR_NONE) {
      // an empty slot of a fixed-capacity pair list: no query, the record is left untouched
    } else if (!valid_pair(sh, a, b)) {
      atomicOr(err, ERR_BAD_INDEX);
      r.w[1] = PARRYGPU_INVALID_ARG;
    } else if (!has_generator(sh, a, &h1) || !has_generator(sh, b, &h2)) {
      r.w[1] = PARRYGPU_UNSUPPORTED_PAIR;  // Err(Unsupported): the manifold is left as it was
    } else {
      r.w[1] = PARRYGPU_OK;
      kind = manifold_kind(sh.types[a], sh.types[b]);
      V3 n1;
      seed = seed_list && kind >= MK_PFM && kind <= MK_PFM_TRIANGLE && !try_normalize(r.v(2), EPS, &n1);
    }
  }
  const uint32_t lane = threadIdx.x & 31;
  if (seed_list) {
    const uint32_t sm = __ballot_sync(0xffffffffu, seed);
    unsigned long long sbase = 0;
    if (sm && lane == 0) sbase = atomicAdd(&ctr[MF_CTR_SEED], (unsigned long long)__popc(sm));
    sbase = __shfl_sync(0xffffffffu, sbase, 0);
    if (seed) seed_list[sbase + __popc(sm & ((1u << lane) - 1))] = (uint32_t)k;
  }
  uint32_t mask = __match_any_sync(0xffffffffu, kind);
  uint32_t leader = (uint32_t)__ffs(mask) - 1;
  unsigned long long base = 0;
  if (kind < MK_KINDS && lane == leader) base = atomicAdd(&ctr[MF_CTR_BINS + kind], (unsigned long long)__popc(mask));
  base = __shfl_sync(mask, base, leader);
  if (kind < MK_KINDS) bins[(size_t)kind * stride + base + __popc(mask & ((1u << lane) - 1))] = (uint32_t)k;
}

template <uint32_t KIND>
__global__ void __launch_bounds__(MF_THREADS) k_mf_kind(ShapeArrays sh, const uint32_t* __restrict__ pairs, float prediction,
                                                        uint32_t* __restrict__ recs, const uint32_t* __restrict__ bins, uint64_t stride,
                                                        unsigned long long* __restrict__ ctr, uint32_t* __restrict__ queue,
                                                        uint32_t* __restrict__ err, const float* __restrict__ init_dirs) {
  // The polyhedral kernel walks its five sub-bins as one index space: warps see one pair kind (but
  // at the bin boundaries), and one launch keeps the sub-bins' slowest pairs overlapped.
  constexpr uint32_t LAST = KIND == MK_PFM ? MK_PFM_TRIANGLE : KIND;
  unsigned long long cnt = 0;
#pragma unroll
  for (uint32_t b = KIND; b <= LAST; ++b) cnt += ctr[MF_CTR_BINS + b];
  uint32_t iters = 0;
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < cnt;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    uint32_t bin = KIND;
    unsigned long long j = i;
    while (bin < LAST && j >= ctr[MF_CTR_BINS + bin]) { j -= ctr[MF_CTR_BINS + bin]; ++bin; }
    uint64_t k = bins[(size_t)bin * stride + j];
    Rec r{recs + (size_t)k * MF_WORDS};
    uint32_t a = pairs[2 * k], b = pairs[2 * k + 1];
    ShapeDev s1 = load_shape(sh.types, sh.params, sh.pool, a);
    ShapeDev s2 = load_shape(sh.types, sh.params, sh.pool, b);
    Pose pos12 = pose_inv_mul(load_pose(sh.poses, a), load_pose(sh.poses, b));
    bool overflow = false, bad = false;
    if constexpr (KIND == MK_BALL_BALL) {
      mf_ball_ball(r, pos12, s1.a, s2.a, prediction);
    } else if constexpr (KIND == MK_CUBOID_CUBOID) {
      mf_cuboid_cuboid(r, pos12, v3(s1.a, s1.b, s1.c), v3(s2.a, s2.b, s2.c), prediction, &overflow);
    } else if constexpr (KIND == MK_CAPSULE_CAPSULE) {
      mf_capsule_capsule(r, pos12, s1.a, s1.b, s2.a, s2.b, prediction);
    } else if constexpr (KIND == MK_CUBOID_TRIANGLE) {
      if (s1.type == SH_CUBOID)
        mf_cuboid_triangle(r, pos12, pose_inverse(pos12), v3(s1.a, s1.b, s1.c), s2, prediction, false, &overflow, sh.pseudo,
                           constraint_row(sh, b));
      else
        mf_cuboid_triangle(r, pose_inverse(pos12), pos12, v3(s2.a, s2.b, s2.c), s1, prediction, true, &overflow, sh.pseudo,
                           constraint_row(sh, a));
    } else if constexpr (KIND == MK_CONVEX_BALL) {
      bool ball_first = s1.type == SH_BALL;
      const uint32_t j = constraint_row(sh, ball_first ? b : a);
      TriPN pn;
      if (j) pn = load_tri_pn(sh.pseudo, j - 1);
      mf_convex_ball(r, ball_first ? pose_inverse(pos12) : pos12, ball_first ? s2 : s1, ball_first ? s1.a : s2.a, prediction, ball_first,
                     j ? &pn : nullptr);
    } else if constexpr (KIND == MK_HULL_BALL) {
      bool ball_first = s1.type == SH_BALL;
      Pose cpos = ball_first ? pose_inverse(pos12) : pos12;
      const ShapeDev& cs = ball_first ? s2 : s1;
      HullDev ch{};
      load_hull(sh, ball_first ? b : a, &ch);
      float radius = ball_first ? s1.a : s2.a;
      V3 proj;
      Simplex s;
      if (hull_project_gjk(cs, cpos.t, &proj, s, &iters)) {
        uint32_t fid = hull_projection_feature(cs, ch, cpos.t, proj, false, &bad);
        finish_convex_ball(r, cpos, proj, false, fid, radius, prediction, ball_first);
      } else {
        enqueue(queue, ctr, k, s, ball_first ? TAG_BALL_FIRST : TAG_BALL_SECOND);
      }
    } else {
      if (!try_update_contacts(r, pos12, COS_1_DEGREES, 1.0e-6f)) {
        // contact_manifold_pfm_pfm: GJK warm-started from the cached normal, else from the caller's
        // (learned) direction, else the relative translation, else +x
        HullDev h1{}, h2{};
        load_hull(sh, a, &h1);
        load_hull(sh, b, &h2);
        float br1, br2;
        ShapeDev p1 = pfm_of(s1, &br1), p2 = pfm_of(s2, &br2);
        V3 dir;
        if (!try_normalize(r.v(2), EPS, &dir) &&
            !(init_dirs && try_normalize(v3(init_dirs[3 * k], init_dirs[3 * k + 1], init_dirs[3 * k + 2]), EPS, &dir)) &&
            !try_normalize(pos12.t, EPS, &dir))
          dir = v3(1.f, 0.f, 0.f);
        float total_prediction = (prediction + br1) + br2;
        Simplex s;
        simplex_reset(s, cso_from_shapes(pos12, p1, p2, dir));
        GjkOut g = gjk_closest_points(pos12, p1, p2, total_prediction, s, &iters);
        if (g.kind == GJK_INTERSECTION) enqueue(queue, ctr, k, s, TAG_PFM);
        else finish_pfm(r, pos12, s1, h1, s2, h2, g.kind, g.p1, g.p2, g.dir, &overflow, &bad, sh.pseudo, constraint_row(sh, a),
                        constraint_row(sh, b));
      }
    }
    if (overflow) atomicOr(err, ERR_CAPACITY);
    if (bad) atomicOr(err, ERR_BAD_INDEX);
  }
  if (KIND >= MK_HULL_BALL && KIND != MK_CUBOID_TRIANGLE) {
    uint32_t w = __reduce_add_sync(0xffffffffu, iters);
    if ((threadIdx.x & 31) == 0 && w) atomicAdd(&ctr[1], (unsigned long long)w);
  }
}

// One queued EPA (the ball projections or the polyhedral pair's contact) and its feature clipping,
// on workspace `ws`.
template <class WS>
__device__ __forceinline__ void manifold_epa_entry(const WS& ws, ShapeArrays& sh, const uint32_t* __restrict__ pairs,
                                                   float prediction, uint32_t* __restrict__ recs, const uint32_t* __restrict__ q,
                                                   uint32_t* __restrict__ err, uint32_t* iters) {
  uint64_t k;
  Simplex s;
  dequeue(q, &k, &s);
  uint32_t tag = q[QUEUE_WORDS - 1];
  uint32_t a = pairs[2 * k], b = pairs[2 * k + 1];
  ShapeDev s1 = load_shape(sh.types, sh.params, sh.pool, a);
  ShapeDev s2 = load_shape(sh.types, sh.params, sh.pool, b);
  HullDev h1, h2;
  load_hull(sh, a, &h1);
  load_hull(sh, b, &h2);
  Pose pos12 = pose_inv_mul(load_pose(sh.poses, a), load_pose(sh.poses, b));
  V3 q1, q2, nn;
  bool overflow = false, bad = false;
  Rec r{recs + (size_t)k * MF_WORDS};
  if (tag == TAG_PFM) {
    float br1, br2;
    ShapeDev p1 = pfm_of(s1, &br1), p2 = pfm_of(s2, &br2);
    int res = epa_closest_points(ws, pos12, p1, p2, s, &q1, &q2, &nn, iters);
    if (res == EPA_OVERFLOW) atomicOr(err, ERR_POLYTOPE_FULL);
    // EPA failure: contact_support_map_support_map_with_params returns NoIntersection(x axis)
    const uint32_t j1 = constraint_row(sh, a), j2 = constraint_row(sh, b);
    if (res == EPA_OK) finish_pfm(r, pos12, s1, h1, s2, h2, GJK_CLOSEST, q1, q2, nn, &overflow, &bad, sh.pseudo, j1, j2);
    else finish_pfm(r, pos12, s1, h1, s2, h2, GJK_NO_INTERSECTION, q1, q2, v3(1.f, 0.f, 0.f), &overflow, &bad, sh.pseudo, j1, j2);
  } else {
    // the ball centre is inside the hull: EPA projection (point_support_map.rs:42-55)
    bool ball_first = tag == TAG_BALL_FIRST;
    Pose cpos = ball_first ? pose_inverse(pos12) : pos12;
    const ShapeDev& cs = ball_first ? s2 : s1;
    const HullDev& ch = ball_first ? h2 : h1;
    float radius = ball_first ? s1.a : s2.a;
    V3 center = cpos.t;
    Pose m{0.f, 0.f, 0.f, 1.f, -center};
    Pose minv = pose_inverse(m);
    ShapeDev origin;
    origin.type = SH_ORIGIN;
    int res = epa_closest_points(ws, minv, cs, origin, s, &q1, &q2, &nn, iters);
    if (res == EPA_OVERFLOW) atomicOr(err, ERR_POLYTOPE_FULL);
    V3 proj = res == EPA_OK ? q1 : center;
    uint32_t fid = hull_projection_feature(cs, ch, center, proj, true, &bad);
    finish_convex_ball(r, cpos, proj, true, fid, radius, prediction, ball_first);
  }
  if (overflow) atomicOr(err, ERR_CAPACITY);
  if (bad) atomicOr(err, ERR_BAD_INDEX);
}

// The queued EPAs, one per thread of a persistent grid, each thread on its own global workspace slot.
__global__ void __launch_bounds__(MF_EPA_THREADS) k_manifolds_epa(ShapeArrays sh, const uint32_t* __restrict__ pairs, float prediction,
                                                                  uint32_t* __restrict__ recs, const uint32_t* __restrict__ queue,
                                                                  const unsigned long long* __restrict__ qcount, uint32_t* __restrict__ ws_pool,
                                                                  unsigned long long* __restrict__ stats, uint32_t* __restrict__ err) {
  const uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x;
  EpaWs ws = epa_slot(ws_pool, slot);
  const unsigned long long total = *qcount;
  uint32_t iters = 0, calls = 0;
  for (unsigned long long e = slot; e < total; e += (unsigned long long)gridDim.x * blockDim.x) {
    manifold_epa_entry(ws, sh, pairs, prediction, recs, queue + (size_t)e * QUEUE_WORDS, err, &iters);
    calls++;
  }
  if (stats) {
    uint32_t w = __reduce_add_sync(0xffffffffu, iters);
    uint32_t cw = __reduce_add_sync(0xffffffffu, calls);
    if ((threadIdx.x & 31) == 0) {
      if (w) atomicAdd(&stats[1], (unsigned long long)w);
      if (cw) atomicAdd(&stats[2], (unsigned long long)cw);
    }
  }
}

}  // namespace

// Manifold update of the first min(cap, *d_count) pairs on device buffers, without host
// synchronisation or allocation once the scratch is reserved: the frame pipeline's narrow phase,
// capturable in a CUDA graph. The scratch is the caller's, so a captured graph never points at
// context scratch that a later call may reallocate.
parrygpu_status pg::manifolds_reserve(parrygpu_ctx* ctx, uint64_t cap, MfScratch& sc) {
  PG_CUDA(ctx, sc.queue.reserve((size_t)cap * QUEUE_WORDS * 4));
  PG_CUDA(ctx, sc.counters.reserve(MF_CTR_BYTES));
  PG_CUDA(ctx, sc.bins.reserve((size_t)cap * MK_KINDS * 4));
  uint32_t epa_blocks = (uint32_t)(ctx->sm_count > 0 ? ctx->sm_count : 152) * 8;
  PG_CUDA(ctx, sc.epa_ws.reserve((size_t)epa_blocks * MF_EPA_THREADS * EPA_SLOT_BYTES));
  if (cap > sc.cap) sc.cap = cap;
  return PARRYGPU_OK;
}

template <uint32_t KIND>
static parrygpu_status launch_kind(parrygpu_ctx* ctx, const ShapeArrays& sh, const uint32_t* d_pairs, float prediction, uint32_t* d_recs,
                                   MfScratch& sc, uint64_t stride, uint32_t grid, const float* init_dirs = nullptr) {
  k_mf_kind<KIND><<<grid, MF_THREADS, 0, ctx->stream>>>(sh, d_pairs, prediction, d_recs, sc.bins.as<uint32_t>(), stride,
                                                        sc.counters.as<unsigned long long>(), sc.queue.as<uint32_t>(), ctx->d_err,
                                                        init_dirs);
  PG_LAUNCHED(ctx);
  return PARRYGPU_OK;
}

parrygpu_status pg::launch_manifolds(parrygpu_ctx* ctx, const ShapeArrays& sh, const uint32_t* d_pairs, uint64_t cap,
                                     const unsigned long long* d_count, float prediction, uint32_t* d_recs, MfScratch& sc,
                                     const float* init_dirs, const LearnedSeed* seed) {
  if (cap == 0) return PARRYGPU_OK;
  if (cap > sc.cap) return set_error(ctx, PARRYGPU_INVALID_ARG, "manifold scratch reserved for fewer pairs");
  const uint64_t stride = cap;
  uint32_t sms = (uint32_t)(ctx->sm_count > 0 ? ctx->sm_count : 152);
  uint32_t epa_blocks = sms * 8;
  uint32_t grid = div_up(cap, MF_THREADS);
  if (grid > sms * 16) grid = sms * 16;
  unsigned long long* ctr = sc.counters.as<unsigned long long>();
  PG_CUDA(ctx, cudaMemsetAsync(ctr, 0, MF_CTR_BYTES, ctx->stream));
  k_mf_classify<<<div_up(cap, MF_THREADS), MF_THREADS, 0, ctx->stream>>>(sh, d_pairs, cap, d_recs, sc.bins.as<uint32_t>(), stride, ctr,
                                                                        ctx->d_err, d_count, seed ? seed->list : nullptr);
  PG_LAUNCHED(ctx);
  parrygpu_status s;
  if (seed) {  // the network's directions for the listed pairs, ahead of the polyhedral kernel
    if ((s = launch_seed_dirs(ctx, sh, d_pairs, *seed, ctr + MF_CTR_SEED, cap)) != PARRYGPU_OK) return s;
    init_dirs = seed->dirs;
  }
  if ((s = launch_kind<MK_BALL_BALL>(ctx, sh, d_pairs, prediction, d_recs, sc, stride, grid)) != PARRYGPU_OK) return s;
  if ((s = launch_kind<MK_CUBOID_CUBOID>(ctx, sh, d_pairs, prediction, d_recs, sc, stride, grid)) != PARRYGPU_OK) return s;
  if ((s = launch_kind<MK_CAPSULE_CAPSULE>(ctx, sh, d_pairs, prediction, d_recs, sc, stride, grid)) != PARRYGPU_OK) return s;
  if ((s = launch_kind<MK_CONVEX_BALL>(ctx, sh, d_pairs, prediction, d_recs, sc, stride, grid)) != PARRYGPU_OK) return s;
  if ((s = launch_kind<MK_HULL_BALL>(ctx, sh, d_pairs, prediction, d_recs, sc, stride, grid)) != PARRYGPU_OK) return s;
  if ((s = launch_kind<MK_PFM>(ctx, sh, d_pairs, prediction, d_recs, sc, stride, grid, init_dirs)) != PARRYGPU_OK) return s;
  if ((s = launch_kind<MK_CUBOID_TRIANGLE>(ctx, sh, d_pairs, prediction, d_recs, sc, stride, grid)) != PARRYGPU_OK) return s;
  k_manifolds_epa<<<epa_blocks, MF_EPA_THREADS, 0, ctx->stream>>>(sh, d_pairs, prediction, d_recs, sc.queue.as<uint32_t>(), ctr,
                                                                 sc.epa_ws.as<uint32_t>(), ctr + 1, ctx->d_err);
  PG_LAUNCHED(ctx);
  return PARRYGPU_OK;
}

// Host records on a large batch: the records go up, get updated and come down in chunks, uploads on
// one copy stream, the manifold kernels on the context stream and downloads on another, so that the
// copies of one chunk overlap the kernels of the next (the records are most of the bytes; shapes,
// pairs and directions are already staged). Each chunk is an independent batch of pairs, so the
// records are those of the single-shot call.
constexpr uint64_t MF_PIPE_CHUNKS = 8;
constexpr uint64_t MF_PIPE_MIN = 262144;  // pairs per chunk at least

static parrygpu_status manifolds_pipelined(parrygpu_ctx* ctx, const ShapeArrays& sh, const uint32_t* dp, const float* di, uint64_t n_pairs,
                                           float prediction, parrygpu_manifold* host, uint32_t* d_rec) {
  if (!ctx->up_stream) {
    PG_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->up_stream, cudaStreamNonBlocking));
    PG_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->down_stream, cudaStreamNonBlocking));
    for (cudaEvent_t& e : ctx->pipe_ev) PG_CUDA(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    if (!ctx->ev_fork) {
      PG_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming));
      PG_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming));
    }
  }
  uint64_t chunks = MF_PIPE_CHUNKS;
  while (chunks > 2 && n_pairs / chunks < MF_PIPE_MIN) --chunks;
  const uint64_t chunk = (n_pairs + chunks - 1) / chunks;
  parrygpu_status s;
  if ((s = manifolds_reserve(ctx, chunk, ctx->mf)) != PARRYGPU_OK) return s;
  cudaStream_t main = ctx->stream;
  // the copy streams start after the staging already queued on the context stream
  PG_CUDA(ctx, cudaEventRecord(ctx->ev_fork, main));
  PG_CUDA(ctx, cudaStreamWaitEvent(ctx->up_stream, ctx->ev_fork, 0));
  PG_CUDA(ctx, cudaStreamWaitEvent(ctx->down_stream, ctx->ev_fork, 0));
  const size_t rb = sizeof(parrygpu_manifold);
  uint64_t c = 0;
  for (uint64_t off = 0; off < n_pairs; off += chunk, ++c) {
    const uint64_t m = n_pairs - off < chunk ? n_pairs - off : chunk;
    cudaEvent_t up_done = ctx->pipe_ev[(2 * c) % parrygpu_ctx::PIPE_EVENTS];
    cudaEvent_t comp_done = ctx->pipe_ev[(2 * c + 1) % parrygpu_ctx::PIPE_EVENTS];
    PG_CUDA(ctx, cudaMemcpyAsync(d_rec + off * MF_WORDS, host + off, m * rb, cudaMemcpyHostToDevice, ctx->up_stream));
    PG_CUDA(ctx, cudaEventRecord(up_done, ctx->up_stream));
    PG_CUDA(ctx, cudaStreamWaitEvent(main, up_done, 0));
    if ((s = launch_manifolds(ctx, sh, dp + 2 * off, m, nullptr, prediction, d_rec + off * MF_WORDS, ctx->mf, di ? di + 3 * off : nullptr)) !=
        PARRYGPU_OK)
      return s;
    PG_CUDA(ctx, cudaEventRecord(comp_done, main));
    PG_CUDA(ctx, cudaStreamWaitEvent(ctx->down_stream, comp_done, 0));
    PG_CUDA(ctx, cudaMemcpyAsync(host + off, d_rec + off * MF_WORDS, m * rb, cudaMemcpyDeviceToHost, ctx->down_stream));
  }
  PG_CUDA(ctx, cudaEventRecord(ctx->ev_join, ctx->down_stream));
  PG_CUDA(ctx, cudaStreamWaitEvent(main, ctx->ev_join, 0));
  return parrygpu_sync(ctx);
}

extern "C" {

parrygpu_status parrygpu_contact_manifolds(parrygpu_ctx* ctx, const parrygpu_shapes* shapes, const uint32_t* pairs, uint64_t n_pairs,
                                           float prediction, parrygpu_manifold* manifolds, parrygpu_gjk_stats* stats) {
  return parrygpu_contact_manifolds_with_dirs(ctx, shapes, pairs, n_pairs, prediction, nullptr, manifolds, stats);
}

parrygpu_status parrygpu_contact_manifolds_with_dirs(parrygpu_ctx* ctx, const parrygpu_shapes* shapes, const uint32_t* pairs, uint64_t n_pairs,
                                                     float prediction, const float* init_dirs, parrygpu_manifold* manifolds,
                                                     parrygpu_gjk_stats* stats) {
  if (!ctx || !shapes) return PARRYGPU_INVALID_ARG;
  if (stats) std::memset(stats, 0, sizeof(*stats));
  if (n_pairs == 0) return PARRYGPU_OK;
  if (!pairs || !manifolds) return set_error(ctx, PARRYGPU_INVALID_ARG, "pairs and manifolds are required");
  PG_CUDA(ctx, cudaSetDevice(ctx->device));
  ShapeArrays sh;
  parrygpu_status s = stage_shapes(ctx, shapes, &sh);
  if (s != PARRYGPU_OK) return s;
  const void* dp;
  if ((s = stage_input(ctx, ctx->stage_in[4], pairs, (size_t)n_pairs * 8, &dp)) != PARRYGPU_OK) return s;
  const void* di = nullptr;
  if (init_dirs && (s = stage_input(ctx, ctx->stage_in[5], init_dirs, (size_t)n_pairs * 12, &di)) != PARRYGPU_OK) return s;
  const size_t rec_bytes = (size_t)n_pairs * sizeof(parrygpu_manifold);
  // The records are read and written: host records go through a device copy and back.
  void* d_rec;
  bool c_rec;
  if ((s = stage_output(ctx, ctx->stage_out[0], manifolds, rec_bytes, &d_rec, &c_rec)) != PARRYGPU_OK) return s;
  if (c_rec && !stats && !ctx->timing && n_pairs >= 2 * MF_PIPE_MIN)
    return manifolds_pipelined(ctx, sh, (const uint32_t*)dp, (const float*)di, n_pairs, prediction, manifolds, (uint32_t*)d_rec);
  if (c_rec) PG_CUDA(ctx, cudaMemcpyAsync(d_rec, manifolds, rec_bytes, cudaMemcpyHostToDevice, ctx->stream));
  if ((s = manifolds_reserve(ctx, n_pairs, ctx->mf)) != PARRYGPU_OK) return s;
  unsigned long long* ctr = ctx->mf.counters.as<unsigned long long>();  // [0] queue count, [1..3] stats
  {
    KernelTimer kt(ctx, "manifolds");
    if ((s = launch_manifolds(ctx, sh, (const uint32_t*)dp, n_pairs, nullptr, prediction, (uint32_t*)d_rec, ctx->mf, (const float*)di)) !=
        PARRYGPU_OK)
      return s;
    kt.stop();
  }
  if (c_rec) PG_CUDA(ctx, cudaMemcpyAsync(manifolds, d_rec, rec_bytes, cudaMemcpyDeviceToHost, ctx->stream));
  if (stats) {
    unsigned long long h[4];
    PG_CUDA(ctx, cudaMemcpyAsync(h, ctr, 32, cudaMemcpyDeviceToHost, ctx->stream));
    PG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    stats->gjk_iterations = h[1];
    stats->epa_iterations = h[2];
    stats->epa_calls = h[3];
  }
  bool staged_in = sh.types != shapes->types || sh.params != (const float4*)shapes->params || sh.poses != shapes->poses ||
                   dp != pairs || (init_dirs && di != init_dirs) || (shapes->n_vertices && sh.pool != shapes->vertices);
  if (c_rec || stats || staged_in) return parrygpu_sync(ctx);
  return PARRYGPU_OK;
}

}  // extern "C"
