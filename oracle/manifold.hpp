// Oracle (test infrastructure only): CPU restatement of parry3d's persistent contact manifolds for
// convex pairs of balls, cuboids and capsules. Paths relative to the parry repository:
//   src/query/contact_manifolds/contact_manifold.rs:108-226, 662-770   TrackedContact, ContactManifold
//   src/query/default_query_dispatcher.rs:749-831                      contact_manifold_convex_convex
//   src/query/contact_manifolds/contact_manifolds_ball_ball.rs:19-57
//   src/query/contact_manifolds/contact_manifolds_capsule_capsule.rs:134-182 (3-D)
//   src/query/contact_manifolds/contact_manifolds_convex_ball.rs:20-145
//   src/query/contact_manifolds/contact_manifolds_cuboid_cuboid.rs:21-107, src/query/sat/sat_cuboid_cuboid.rs
//   src/query/contact_manifolds/contact_manifolds_pfm_pfm.rs:44-162
//   src/shape/polygonal_feature3d.rs:60-439, src/shape/cuboid.rs:267-352 (support_face),
//   src/shape/polygonal_feature_map.rs:30-46, src/shape/shape.rs:855-857 (capsule = segment + radius)
//   src/query/clip/clip_segment_segment.rs, src/query/closest_points/closest_points_segment_segment.rs
//   src/query/contact_manifolds/contact_manifolds_cuboid_triangle.rs:10-174 (with normal constraints)
// Normal constraints (TrianglePseudoNormals of a TriMesh with FIX_INTERNAL_EDGES) enter the
// convex-ball, cuboid-triangle and pfm-pfm generators as in the reference; nullptr = None.
#pragma once
#include "contact.hpp"
#include "pseudo_normals.hpp"
#include "ray.hpp"
#include <cstring>

namespace oracle {

constexpr uint32_t PFID_UNKNOWN = 0;
inline uint32_t pfid_vertex(uint32_t c) { return (1u << 30) | c; }
inline uint32_t pfid_edge(uint32_t c) { return (2u << 30) | c; }
inline uint32_t pfid_face(uint32_t c) { return (3u << 30) | c; }

template <class R> inline R cos_1_degrees() { return R(0.99984769515); }
template <class R> inline R cos_frac_pi_8() { return R(0.92387953251); }

// approx::ulps_eq with the default epsilon and max_ulps = 4
inline bool ulps_eq(float a, float b) {
  if (std::fabs(a - b) <= std::numeric_limits<float>::epsilon()) return true;
  if (std::isnan(a) || std::isnan(b)) return false;  // NaN.signum() never equals another signum
  if (std::signbit(a) != std::signbit(b)) return false;
  int32_t ia, ib;
  std::memcpy(&ia, &a, 4);
  std::memcpy(&ib, &b, 4);
  int64_t d = (int64_t)ia - (int64_t)ib;
  return (d < 0 ? -d : d) <= 4;
}
inline bool ulps_eq(double a, double b) {
  if (std::fabs(a - b) <= std::numeric_limits<double>::epsilon()) return true;
  if (std::isnan(a) || std::isnan(b)) return false;
  if (std::signbit(a) != std::signbit(b)) return false;
  int64_t ia, ib;
  std::memcpy(&ia, &a, 8);
  std::memcpy(&ib, &b, 8);
  __int128 d = (__int128)ia - (__int128)ib;
  return (d < 0 ? -d : d) <= 4;
}

template <class R> inline R clamp01(R x) { return x > R(1) ? R(1) : (x < R(0) ? R(0) : x); }

template <class R> struct TrackedContact {
  Vec3<R> local_p1, local_p2;
  R dist;
  uint32_t fid1, fid2;
  float data = 0.0f;
  static TrackedContact make(const Vec3<R>& p1, const Vec3<R>& p2, uint32_t f1, uint32_t f2, R d, bool flipped) {
    TrackedContact c;
    if (!flipped) { c.local_p1 = p1; c.local_p2 = p2; c.fid1 = f1; c.fid2 = f2; }
    else { c.local_p1 = p2; c.local_p2 = p1; c.fid1 = f2; c.fid2 = f1; }
    c.dist = d;
    return c;
  }
  void copy_geometry_from(const TrackedContact& o) { local_p1 = o.local_p1; local_p2 = o.local_p2; fid1 = o.fid1; fid2 = o.fid2; dist = o.dist; }
};

template <class R> struct Manifold {
  std::vector<TrackedContact<R>> points;
  Vec3<R> local_n1, local_n2;

  bool try_update_contacts_eps(const Iso<R>& pos12, R angle_dot_threshold, R dist_sq_threshold) {
    if (points.empty()) return false;
    Vec3<R> n2 = pos12.transform_vector(local_n2);
    if (-dot(local_n1, n2) < angle_dot_threshold) return false;
    for (auto& pt : points) {
      Vec3<R> p2 = pos12.transform_point(pt.local_p2);
      Vec3<R> dpt = p2 - pt.local_p1;
      R dist = dot(dpt, local_n1);
      if (dist * pt.dist < R(0)) return false;
      Vec3<R> np1 = p2 - local_n1 * dist;
      if (norm_squared(pt.local_p1 - np1) > dist_sq_threshold) return false;
      pt.dist = dist;
      pt.local_p1 = np1;
    }
    return true;
  }
  bool try_update_contacts(const Iso<R>& pos12) { return try_update_contacts_eps(pos12, cos_1_degrees<R>(), R(1.0e-6)); }
  void match_contacts(const std::vector<TrackedContact<R>>& old) {
    for (auto& c : points)
      for (const auto& o : old)
        if (c.fid1 == o.fid1 && c.fid2 == o.fid2) c.data = o.data;
  }
};

// Pixar orthonormal basis (src/utils/wops.rs WBasis)
template <class R> inline void orthonormal_basis(const Vec3<R>& v, Vec3<R>* b0, Vec3<R>* b1) {
  R sign = std::copysign(R(1), v.z);
  R a = R(-1) / (sign + v.z);
  R b = v.x * v.y * a;
  *b0 = Vec3<R>(R(1) + sign * v.x * v.x * a, sign * b, -sign * v.x);
  *b1 = Vec3<R>(b, sign + v.y * v.y * a, -v.y);
}

template <class R> struct P2 {
  R x, y;
};
template <class R> inline P2<R> p2sub(P2<R> a, P2<R> b) { return {a.x - b.x, a.y - b.y}; }
template <class R> inline R p2dot(P2<R> a, P2<R> b) { return a.x * b.x + a.y * b.y; }
template <class R> inline R p2perp(P2<R> a, P2<R> b) { return a.x * b.y - a.y * b.x; }

// closest_points_segment_segment_with_locations_nD: returns s, t (0 / 1 = vertex)
template <class R, class V, class DotF>
inline void seg_seg_params(const V& a0, const V& a1, const V& b0, const V& b1, DotF dotf, R* s_out, R* t_out) {
  V d1 = a1 - a0, d2 = b1 - b0, r = a0 - b0;
  R a = dotf(d1, d1), e = dotf(d2, d2), f = dotf(d2, r);
  R s, t;
  const R eps = eps_default<R>();
  if (a <= eps && e <= eps) { s = R(0); t = R(0); }
  else if (a <= eps) { s = R(0); t = clamp01(f / e); }
  else {
    R c = dotf(d1, r);
    if (e <= eps) { t = R(0); s = clamp01(-c / a); }
    else {
      R b = dotf(d1, d2);
      R ae = a * e, bb = b * b;
      R denom = ae - bb;
      if (denom > eps && !ulps_eq(ae, bb)) s = clamp01((b * f - c * e) / denom);
      else s = R(0);
      t = (b * s + f) / e;
      if (t < R(0)) { t = R(0); s = clamp01(-c / a); }
      else if (t > R(1)) { t = R(1); s = clamp01((b - c) / a); }
    }
  }
  *s_out = s;
  *t_out = t;
}
// SegmentPointLocation::barycentric_coordinates from the parameter
template <class R> inline void seg_bc(R s, R* b0, R* b1) {
  if (s == R(0)) { *b0 = R(1); *b1 = R(0); }
  else if (s == R(1)) { *b0 = R(0); *b1 = R(1); }
  else { *b0 = R(1) - s; *b1 = s; }
}

template <class R> struct PolyFeature {
  Vec3<R> vertices[4];
  uint32_t vids[4], eids[4], fid;
  int num_vertices;
};

// Cuboid::support_face (cuboid.rs:267-352)
template <class R> inline PolyFeature<R> cuboid_support_face(const Vec3<R>& he, const Vec3<R>& dir) {
  int ia = iamax(dir);
  R sign = std::copysign(R(1), dir[ia]);
  PolyFeature<R> f;
  if (ia == 0) {
    f.vertices[0] = Vec3<R>(he.x * sign, he.y, he.z); f.vertices[1] = Vec3<R>(he.x * sign, -he.y, he.z);
    f.vertices[2] = Vec3<R>(he.x * sign, -he.y, -he.z); f.vertices[3] = Vec3<R>(he.x * sign, he.y, -he.z);
  } else if (ia == 1) {
    f.vertices[0] = Vec3<R>(he.x, he.y * sign, he.z); f.vertices[1] = Vec3<R>(-he.x, he.y * sign, he.z);
    f.vertices[2] = Vec3<R>(-he.x, he.y * sign, -he.z); f.vertices[3] = Vec3<R>(he.x, he.y * sign, -he.z);
  } else {
    f.vertices[0] = Vec3<R>(he.x, he.y, he.z * sign); f.vertices[1] = Vec3<R>(he.x, -he.y, he.z * sign);
    f.vertices[2] = Vec3<R>(-he.x, -he.y, he.z * sign); f.vertices[3] = Vec3<R>(-he.x, he.y, he.z * sign);
  }
  int si = ((int)sign + 1) / 2;
  static const uint32_t VIDS[3][2][4] = {
      {{0b000, 0b010, 0b011, 0b001}, {0b100, 0b110, 0b111, 0b101}},
      {{0b000, 0b100, 0b101, 0b001}, {0b010, 0b110, 0b111, 0b011}},
      {{0b000, 0b010, 0b110, 0b100}, {0b001, 0b011, 0b111, 0b101}}};
  static const uint32_t EIDS[3][2][4] = {
      {{0b11010000, 0b11011010, 0b11011001, 0b11001000}, {0b11110100, 0b11111110, 0b11111101, 0b11101100}},
      {{0b11100000, 0b11101100, 0b11101001, 0b11001000}, {0b11110010, 0b11111110, 0b11111011, 0b11011010}},
      {{0b11010000, 0b11110010, 0b11110100, 0b11100000}, {0b11011001, 0b11111011, 0b11111101, 0b11101001}}};
  for (int i = 0; i < 4; ++i) { f.vids[i] = pfid_vertex(VIDS[ia][si][i] * 2); f.eids[i] = pfid_edge(EIDS[ia][si][i]); }
  f.fid = pfid_face((uint32_t)(ia + si * 3 + 10));
  f.num_vertices = 4;
  return f;
}

// PolygonalFeature::from(Segment): capsule axis (0,-h,0)-(0,h,0)
template <class R> inline PolyFeature<R> segment_feature(R hh) {
  PolyFeature<R> f;
  Vec3<R> a(0, -hh, 0), b(0, hh, 0);
  f.vertices[0] = a; f.vertices[1] = b; f.vertices[2] = b; f.vertices[3] = b;
  f.vids[0] = pfid_vertex(0); f.vids[1] = pfid_vertex(1); f.vids[2] = pfid_vertex(1); f.vids[3] = pfid_vertex(1);
  for (int i = 0; i < 4; ++i) f.eids[i] = pfid_edge(0);
  f.fid = pfid_face(0);
  f.num_vertices = 2;
  return f;
}

// PolygonalFeature::from(Triangle) (polygonal_feature3d.rs:37-47): the whole triangle, whatever the
// direction (Triangle::support_face, triangle.rs:280-282; polygonal_feature_map.rs:36-40).
template <class R> inline PolyFeature<R> triangle_feature(const Shape<R>& s) {
  PolyFeature<R> f;
  f.vertices[0] = s.pts[0]; f.vertices[1] = s.pts[1]; f.vertices[2] = s.pts[2]; f.vertices[3] = s.pts[2];
  const uint32_t ids[4] = {0, 1, 2, 2};
  for (int i = 0; i < 4; ++i) { f.vids[i] = pfid_vertex(ids[i]); f.eids[i] = pfid_edge(ids[i]); }
  f.fid = pfid_face(0);
  f.num_vertices = 3;
  return f;
}

// approx::relative_eq with f32::EPSILON (or f64) as both the absolute and relative epsilon.
template <class R> inline bool relative_eq_scalar(R a, R b) {
  if (a == b) return true;
  if (std::isinf(a) || std::isinf(b)) return false;
  R d = std::fabs(a - b);
  if (d <= eps_default<R>()) return true;
  R largest = std::fabs(b) > std::fabs(a) ? std::fabs(b) : std::fabs(a);
  return d <= largest * eps_default<R>();
}
template <class R> inline bool relative_eq_v3(const Vec3<R>& a, const Vec3<R>& b) {
  return relative_eq_scalar(a.x, b.x) && relative_eq_scalar(a.y, b.y) && relative_eq_scalar(a.z, b.z);
}

// Triangle::project_local_point_and_get_feature (point_triangle.rs:26-48, 3-D: solid location,
// is_inside = relative_eq!(projection, point) by compute_result :5-18, OnSolid inside).
template <class R> inline uint32_t triangle_projection_feature(const Shape<R>& s, const Vec3<R>& pt, Vec3<R>* proj, bool* inside) {
  Loc<R> loc;
  *proj = project_triangle(s.pts[0], s.pts[1], s.pts[2], pt, &loc);
  if (loc.kind == LOC_SOLID) { *inside = true; return pfid_face(0); }
  *inside = relative_eq_v3(*proj, pt);
  if (loc.kind == LOC_VERTEX) return pfid_vertex((uint32_t)loc.id);
  if (loc.kind == LOC_EDGE) return pfid_edge((uint32_t)loc.id);
  return pfid_face((uint32_t)loc.id);
}

// ConvexPolyhedron::local_support_feature (convex_polyhedron.rs:959-991): the face whose normal has
// the largest dot product with dir (first on ties), at most its first 4 vertices.
template <class R> inline PolyFeature<R> hull_support_feature(const Shape<R>& s, const Vec3<R>& dir) {
  const HullTopo& t = *s.topo;
  auto normal = [&](uint32_t f) { return Vec3<R>(R(t.face_normals[3 * f]), R(t.face_normals[3 * f + 1]), R(t.face_normals[3 * f + 2])); };
  uint32_t best = 0;
  R best_dot = dot(normal(0), dir);
  for (uint32_t f = 1; f < t.n_faces; ++f) {
    R d = dot(normal(f), dir);
    if (d > best_dot) { best = f; best_dot = d; }
  }
  PolyFeature<R> out{};
  uint32_t first = t.face_ranges[2 * best], num = std::min(t.face_ranges[2 * best + 1], 4u);
  for (uint32_t i = 0; i < num; ++i) {
    uint32_t vid = t.face_vertices[first + i], eid = t.face_edges[first + i];
    out.vertices[i] = s.pts[vid];
    out.vids[i] = pfid_vertex(vid);
    out.eids[i] = pfid_edge(eid);
  }
  out.fid = pfid_face(best);
  out.num_vertices = (int)num;
  return out;
}

// f32 sin / cos of (PI / 180 as f32), the eps of ConvexPolyhedron::support_feature_id_toward
// (convex_polyhedron.rs:919-922), correctly rounded.
template <class R> inline R hull_feature_seps() { return R(0.017452406f); }
template <class R> inline R hull_feature_ceps() { return R(0.9998477f); }

// ConvexPolyhedron::support_feature_id_toward_eps (convex_polyhedron.rs:885-917) as a PackedFeatureId.
template <class R> inline uint32_t hull_support_feature_id(const Shape<R>& s, const Vec3<R>& local_dir) {
  const HullTopo& t = *s.topo;
  R seps = hull_feature_seps<R>(), ceps = hull_feature_ceps<R>();
  uint32_t vid = 0;
  R best = dot(s.pts[0], local_dir);
  for (uint32_t i = 1; i < s.npts; ++i) {
    R d = dot(s.pts[i], local_dir);
    if (d > best) { best = d; vid = i; }
  }
  uint32_t first = t.vertex_ranges[2 * vid], num = t.vertex_ranges[2 * vid + 1];
  for (uint32_t i = 0; i < num; ++i) {
    uint32_t f = t.vertex_faces[first + i];
    Vec3<R> n(R(t.face_normals[3 * f]), R(t.face_normals[3 * f + 1]), R(t.face_normals[3 * f + 2]));
    if (dot(n, local_dir) >= ceps) return pfid_face(f);
  }
  for (uint32_t i = 0; i < num; ++i) {
    uint32_t e = t.vertex_edges[first + i];
    Vec3<R> d(R(t.edge_dirs[3 * e]), R(t.edge_dirs[3 * e + 1]), R(t.edge_dirs[3 * e + 2]));
    if (std::fabs(dot(d, local_dir)) <= seps) return pfid_edge(e);
  }
  return pfid_vertex(vid);
}

// ConvexPolyhedron::project_local_point_and_get_feature (point_support_map.rs:55-77).
template <class R> inline uint32_t hull_projection_feature(const Shape<R>& s, const Vec3<R>& pt, const PointProj<R>& proj) {
  Vec3<R> dpt = pt - proj.point;
  Vec3<R> local_dir = proj.is_inside ? -dpt : dpt;
  Vec3<R> u;
  if (try_normalize(local_dir, eps_default<R>(), &u)) return hull_support_feature_id(s, u);
  return PFID_UNKNOWN;
}

// clip_segment_segment (clip/clip_segment_segment.rs): two clipping points (p1, p2, feat1, feat2)
template <class R> struct ClipPt {
  Vec3<R> p1, p2;
  int f1, f2;
};
template <class R> inline bool clip_segment_segment(Vec3<R> s10, Vec3<R> s11, Vec3<R> s20, Vec3<R> s21, ClipPt<R>* ca, ClipPt<R>* cb) {
  Vec3<R> tangent1 = s11 - s10;
  R sq = norm_squared(tangent1);
  R r1[2] = {R(0), sq};
  R r2[2] = {dot(s20 - s10, tangent1), dot(s21 - s10, tangent1)};
  int f1[2] = {0, 2}, f2[2] = {0, 2};
  if (r1[1] < r1[0]) { std::swap(r1[0], r1[1]); std::swap(f1[0], f1[1]); std::swap(s10, s11); }
  if (r2[1] < r2[0]) { std::swap(r2[0], r2[1]); std::swap(f2[0], f2[1]); std::swap(s20, s21); }
  if (r2[0] > r1[1] || r1[0] > r2[1]) return false;
  R l1 = r1[1] - r1[0], l2 = r2[1] - r2[0];
  if (r2[0] > r1[0]) {
    R bc = (r2[0] - r1[0]) / l1;
    *ca = {s10 + tangent1 * bc, s20, 1, f2[0]};
  } else {
    R bc = (r1[0] - r2[0]) / l2;
    *ca = {s10, s20 + (s21 - s20) * bc, f1[0], 1};
  }
  if (r2[1] < r1[1]) {
    R bc = (r2[1] - r1[0]) / l1;
    *cb = {s10 + tangent1 * bc, s21, 1, f2[1]};
  } else {
    R bc = (r1[1] - r2[0]) / l2;
    *cb = {s11, s20 + (s21 - s20) * bc, f1[1], 1};
  }
  return true;
}

// polygonal_feature3d.rs closest_points_line2d
template <class R> inline bool closest_points_line2d(P2<R> e10, P2<R> e11, P2<R> e20, P2<R> e21, R* s_out, R* t_out) {
  P2<R> d1 = p2sub(e11, e10), d2 = p2sub(e21, e20), r = p2sub(e10, e20);
  R a = p2dot(d1, d1), e = p2dot(d2, d2), f = p2dot(d2, r);
  R eps = eps_default<R>();
  if (a <= eps && e <= eps) { *s_out = R(0); *t_out = R(0); return true; }
  if (a <= eps) { *s_out = R(0); *t_out = f / e; return true; }
  R c = p2dot(d1, r);
  if (e <= eps) { *s_out = -c / a; *t_out = R(0); return true; }
  R b = p2dot(d1, d2);
  R ae = a * e, bb = b * b;
  R denom = ae - bb;
  bool parallel = denom <= eps || ulps_eq(ae, bb);
  if (parallel) return false;
  R s = (b * f - c * e) / denom;
  *s_out = s;
  *t_out = (b * s + f) / e;
  return true;
}

template <class R>
inline void feature_contacts(const Iso<R>& pos12, const Vec3<R>& sep1, const PolyFeature<R>& f1, const PolyFeature<R>& f2, Manifold<R>& m,
                             bool flipped) {
  Vec3<R> b0, b1;
  orthonormal_basis(sep1, &b0, &b1);
  if (f1.num_vertices == 2 && f2.num_vertices == 2) {
    // contacts_edge_edge
    P2<R> pe1[2] = {{dot(f1.vertices[0], b0), dot(f1.vertices[0], b1)}, {dot(f1.vertices[1], b0), dot(f1.vertices[1], b1)}};
    Vec3<R> v21[2] = {pos12.transform_point(f2.vertices[0]), pos12.transform_point(f2.vertices[1])};
    P2<R> pe2[2] = {{dot(v21[0], b0), dot(v21[0], b1)}, {dot(v21[1], b0), dot(v21[1], b1)}};
    P2<R> t1 = p2sub(pe1[1], pe1[0]), t2 = p2sub(pe2[1], pe2[0]);
    R n1 = std::sqrt(p2dot(t1, t1)), n2 = std::sqrt(p2dot(t2, t2));
    if (n1 > eps_default<R>() && n2 > eps_default<R>()) {
      P2<R> u1 = {t1.x / n1, t1.y / n1}, u2 = {t2.x / n2, t2.y / n2};
      bool parallel = p2dot(u1, u2) >= cos_frac_pi_8<R>();
      if (!parallel) {
        R s, t;
        auto d2f = [](const P2<R>& x, const P2<R>& y) { return p2dot(x, y); };
        struct PV { P2<R> p; PV operator-(const PV& o) const { return {p2sub(p, o.p)}; } };
        seg_seg_params<R>(PV{pe1[0]}, PV{pe1[1]}, PV{pe2[0]}, PV{pe2[1]},
                          [&](const PV& x, const PV& y) { return d2f(x.p, y.p); }, &s, &t);
        R a0, a1, c0, c1;
        seg_bc(s, &a0, &a1);
        seg_bc(t, &c0, &c1);
        Vec3<R> lp1 = f1.vertices[0] * a0 + f1.vertices[1] * a1;
        Vec3<R> lp21 = v21[0] * c0 + v21[1] * c1;
        R dist = dot(lp21 - lp1, sep1);
        m.points.push_back(TrackedContact<R>::make(lp1, pos12.inverse_transform_point(lp21), f1.eids[0], f2.eids[0], dist, flipped));
        return;
      }
    }
    ClipPt<R> ca, cb;
    if (clip_segment_segment(f1.vertices[0], f1.vertices[1], v21[0], v21[1], &ca, &cb)) {
      auto feat = [](const PolyFeature<R>& f, int id) { return id == 0 ? f.vids[0] : (id == 1 ? f.eids[0] : f.vids[1]); };
      m.points.push_back(TrackedContact<R>::make(ca.p1, pos12.inverse_transform_point(ca.p2), feat(f1, ca.f1), feat(f2, ca.f2),
                                                 dot(ca.p2 - ca.p1, sep1), flipped));
      m.points.push_back(TrackedContact<R>::make(cb.p1, pos12.inverse_transform_point(cb.p2), feat(f1, cb.f1), feat(f2, cb.f2),
                                                 dot(cb.p2 - cb.p1, sep1), flipped));
    }
    return;
  }
  // contacts_face_face
  P2<R> pf1[4], pf2[4];
  Vec3<R> v21[4];
  for (int i = 0; i < 4; ++i) {
    pf1[i] = {dot(f1.vertices[i], b0), dot(f1.vertices[i], b1)};
    v21[i] = pos12.transform_point(f2.vertices[i]);
  }
  for (int i = 0; i < 4; ++i) pf2[i] = {dot(v21[i], b0), dot(v21[i], b1)};
  if (f2.num_vertices > 2) {
    Vec3<R> normal2_1 = cross(v21[2] - v21[1], v21[0] - v21[1]);
    R denom = dot(normal2_1, sep1);
    if (!(std::fabs(denom) <= eps_default<R>())) {
      int last2 = f2.num_vertices - 1;
      for (int i = 0; i < f1.num_vertices; ++i) {
        P2<R> p1 = pf1[i];
        R sign = p2perp(p2sub(pf2[0], pf2[last2]), p2sub(p1, pf2[last2]));
        bool outside = false;
        for (int j = 0; j < last2; ++j) {
          R ns = p2perp(p2sub(pf2[j + 1], pf2[j]), p2sub(p1, pf2[j]));
          if (sign == R(0)) sign = ns;
          else if (sign * ns < R(0)) { outside = true; break; }
        }
        if (outside) continue;
        R dist = dot(v21[0] - f1.vertices[i], normal2_1) / denom;
        Vec3<R> lp1 = f1.vertices[i];
        Vec3<R> lp21 = f1.vertices[i] + sep1 * dist;
        m.points.push_back(TrackedContact<R>::make(lp1, pos12.inverse_transform_point(lp21), f1.vids[i], f2.fid, dist, flipped));
      }
    }
  }
  if (f1.num_vertices > 2) {
    Vec3<R> normal1 = cross(f1.vertices[2] - f1.vertices[1], f1.vertices[0] - f1.vertices[1]);
    R denom = -dot(normal1, sep1);
    if (!(std::fabs(denom) <= eps_default<R>())) {
      int last1 = f1.num_vertices - 1;
      for (int i = 0; i < f2.num_vertices; ++i) {
        P2<R> p2 = pf2[i];
        R sign = p2perp(p2sub(pf1[0], pf1[last1]), p2sub(p2, pf1[last1]));
        bool outside = false;
        for (int j = 0; j < last1; ++j) {
          R ns = p2perp(p2sub(pf1[j + 1], pf1[j]), p2sub(p2, pf1[j]));
          if (sign == R(0)) sign = ns;
          else if (sign * ns < R(0)) { outside = true; break; }
        }
        if (outside) continue;
        R dist = dot(f1.vertices[0] - v21[i], normal1) / denom;
        Vec3<R> lp21 = v21[i];
        Vec3<R> lp1 = v21[i] - sep1 * dist;
        m.points.push_back(TrackedContact<R>::make(lp1, pos12.inverse_transform_point(lp21), f1.fid, f2.vids[i], dist, flipped));
      }
    }
  }
  for (int j = 0; j < f2.num_vertices; ++j) {
    P2<R> e20 = pf2[j], e21 = pf2[(j + 1) % f2.num_vertices];
    for (int i = 0; i < f1.num_vertices; ++i) {
      P2<R> e10 = pf1[i], e11 = pf1[(i + 1) % f1.num_vertices];
      R s, t;
      if (closest_points_line2d(e10, e11, e20, e21, &s, &t)) {
        if (s > R(0) && s < R(1) && t > R(0) && t < R(1)) {
          Vec3<R> lp1 = f1.vertices[i] * (R(1) - s) + f1.vertices[(i + 1) % f1.num_vertices] * s;
          Vec3<R> lp21 = v21[j] * (R(1) - t) + v21[(j + 1) % f2.num_vertices] * t;
          R dist = dot(lp21 - lp1, sep1);
          m.points.push_back(TrackedContact<R>::make(lp1, pos12.inverse_transform_point(lp21), f1.eids[i], f2.eids[j], dist, flipped));
        }
      }
    }
  }
}

}  // namespace oracle

namespace oracle {

// contact_manifolds_ball_ball.rs:19-57
template <class R> inline void manifold_ball_ball(const Iso<R>& pos12, R ra, R rb, R prediction, Manifold<R>& m) {
  Vec3<R> dc = pos12.tra;
  R cd = norm(dc);
  R dist = (cd - ra) - rb;
  if (dist < prediction) {
    Vec3<R> n1 = cd != R(0) ? dc / cd : Vec3<R>(0, 1, 0);
    Vec3<R> n2 = pos12.inverse_transform_vector(-n1);
    TrackedContact<R> c = TrackedContact<R>::make(n1 * ra, n2 * rb, pfid_face(0), pfid_face(0), dist, false);
    if (!m.points.empty()) m.points[0].copy_geometry_from(c);
    else m.points.push_back(c);
    m.local_n1 = n1;
    m.local_n2 = n2;
  } else {
    m.points.clear();
  }
}

// contact_manifolds_capsule_capsule.rs:134-182 (3-D)
template <class R> inline void manifold_capsule_capsule(const Iso<R>& pos12, R hh1, R r1, R hh2, R r2, R prediction, Manifold<R>& m) {
  Vec3<R> a1(0, -hh1, 0), b1(0, hh1, 0);
  Vec3<R> a2 = pos12.transform_point(Vec3<R>(0, -hh2, 0)), b2 = pos12.transform_point(Vec3<R>(0, hh2, 0));
  R s, t;
  seg_seg_params<R>(a1, b1, a2, b2, [](const Vec3<R>& x, const Vec3<R>& y) { return dot(x, y); }, &s, &t);
  R s0, s1, t0, t1;
  seg_bc(s, &s0, &s1);
  seg_bc(t, &t0, &t1);
  Vec3<R> lp1 = a1 * s0 + b1 * s1;
  Vec3<R> lp21 = a2 * t0 + b2 * t1;
  Vec3<R> n1;
  if (!try_normalize(lp21 - lp1, eps_default<R>(), &n1)) n1 = Vec3<R>(0, 1, 0);
  R dist = (dot(lp21 - lp1, n1) - r1) - r2;
  if (dist <= prediction) {
    Vec3<R> n2 = pos12.inverse_transform_vector(-n1);
    TrackedContact<R> c = TrackedContact<R>::make(lp1 + n1 * r1, pos12.inverse_transform_point(lp21) + n2 * r2, pfid_face(0),
                                                  pfid_face(0), dist, false);
    if (!m.points.empty()) m.points[0].copy_geometry_from(c);
    else m.points.push_back(c);
    m.local_n1 = n1;
    m.local_n2 = n2;
  } else {
    m.points.clear();
  }
}

// point_aabb.rs:70-132 feature of the projection on a cuboid (PackedFeatureId)
template <class R> inline uint32_t cuboid_projection_feature(const Vec3<R>& he, const Vec3<R>& pt, Vec3<R>* proj, bool* inside) {
  Vec3<R> mins = -he, maxs = he;
  PointProj<R> p = project_cuboid(he, pt);
  *proj = p.point;
  *inside = p.is_inside;
  Vec3<R> ls = p.point;
  Vec3<R> shift = p.shift;
  int nz = 0, last_zero = 0, last_nz = 0;
  for (int i = 0; i < 3; ++i) { if (shift[i] == R(0)) { nz++; last_zero = i; } else last_nz = i; }
  if (nz == 3) {
    for (int i = 0; i < 3; ++i) {
      if (ls[i] > maxs[i] - eps_default<R>()) return pfid_face(i);
      if (ls[i] <= mins[i] + eps_default<R>()) return pfid_face(i + 3);
    }
    return PFID_UNKNOWN;
  }
  Vec3<R> center = (mins + maxs) * R(0.5);
  if (nz == 2) return ls[last_nz] < center[last_nz] ? pfid_face(last_nz + 3) : pfid_face(last_nz);
  uint32_t id = 0;
  for (int i = 0; i < 3; ++i) if (ls[i] < center[i]) id |= 1u << i;
  if (nz == 0) return pfid_vertex(id);
  return pfid_edge((id << 2) | (uint32_t)last_zero);
}

// contact_manifolds_convex_ball.rs:45-145 for a cuboid, capsule, triangle or hull shape1; c1 / c2 are
// the normal constraints of shape1 / the ball.
template <class R>
inline void manifold_convex_ball(const Iso<R>& pos12, const Shape<R>& s1, R radius2, R prediction, Manifold<R>& m, bool flipped,
                                 GjkStats* st, const TriPseudoNormals<R>* c1 = nullptr, const TriPseudoNormals<R>* c2 = nullptr) {
  Vec3<R> lp21 = pos12.tra;
  Vec3<R> proj;
  bool inside;
  uint32_t fid1;
  if (s1.type == SHAPE_CUBOID) fid1 = cuboid_projection_feature(s1.half, lp21, &proj, &inside);
  else if (s1.type == SHAPE_TRIANGLE) fid1 = triangle_projection_feature(s1, lp21, &proj, &inside);
  else if (s1.type == SHAPE_CAPSULE) {
    PointProj<R> p = project_capsule(s1.half_height, s1.radius, lp21);
    proj = p.point; inside = p.is_inside; fid1 = pfid_face(0);
  } else {
    PointProj<R> p = project_support_map(s1, lp21, st);
    proj = p.point; inside = p.is_inside; fid1 = hull_projection_feature(s1, lp21, p);
  }
  Vec3<R> lp1 = proj;
  Vec3<R> dpos = lp21 - lp1;
  Vec3<R> n1;
  R dist;
  if (!try_normalize(dpos, R(0), &n1, &dist)) {
    if (!try_normalize(pos12.tra, R(0), &n1)) n1 = Vec3<R>(1, 0, 0);
    dist = R(0);
  }
  if (inside) { n1 = -n1; dist = -dist; }
  if (dist <= radius2 + prediction) {
    Vec3<R> n2 = pos12.inverse_transform_vector(-n1);
    const Vec3<R> uncorrected_n2 = n2;
    if (!project_local_normals(c1, c2, pos12, &n1, &n2)) {
      m.points.clear();  // the contact got discarded by the normal correction
      return;
    }
    Vec3<R> lp2 = n2 * radius2;
    if (!(uncorrected_n2 == n2)) {
      // corrected normal: the contact point on shape1 is where the ray from the ball centre along
      // the corrected normal meets it (Shape::cast_local_ray_and_get_normal, solid = false)
      Ray<R> ray1{pos12.tra, inside ? n1 : -n1};
      RayHit<R> hit;
      if (s1.type != SHAPE_TRIANGLE || !ray_triangle(s1.pts[0], s1.pts[1], s1.pts[2], ray1, &hit) ||
          !(hit.toi <= std::numeric_limits<R>::max())) {
        m.points.clear();
        return;
      }
      lp1 = ray1.origin + ray1.dir * hit.toi;
      dist = inside ? -hit.toi : hit.toi;
      fid1 = pfid_face(hit.fid);
    }
    TrackedContact<R> c = TrackedContact<R>::make(lp1, lp2, fid1, pfid_face(0), dist - radius2, flipped);
    if (m.points.size() != 1) { m.points.clear(); m.points.push_back(c); }
    else m.points[0].copy_geometry_from(c);
    if (flipped) { m.local_n1 = n2; m.local_n2 = n1; }
    else { m.local_n1 = n1; m.local_n2 = n2; }
  } else {
    m.points.clear();
  }
}

// sat_cuboid_cuboid.rs
template <class R> inline std::pair<R, Vec3<R>> sat_normal_oneway(const Vec3<R>& h1, const Vec3<R>& h2, const Iso<R>& pos12) {
  R best = -std::numeric_limits<R>::max();
  Vec3<R> best_dir;
  Shape<R> c2; c2.type = SHAPE_CUBOID; c2.half = h2;
  for (int i = 0; i < 3; ++i) {
    R sign = std::copysign(R(1), pos12.tra[i]);
    Vec3<R> axis1; axis1[i] = sign;
    Vec3<R> axis2 = pos12.inverse_transform_vector(-axis1);
    Vec3<R> pt2 = pos12.transform_point(c2.local_support(axis2));
    R sep = pt2[i] * sign - h1[i];
    if (sep > best) { best = sep; best_dir = axis1; }
  }
  return {best, best_dir};
}
template <class R> inline std::pair<R, Vec3<R>> sat_edge_twoway(const Vec3<R>& h1, const Vec3<R>& h2, const Iso<R>& pos12) {
  R best = -std::numeric_limits<R>::max();
  Vec3<R> best_dir;
  Shape<R> c1; c1.type = SHAPE_CUBOID; c1.half = h1;
  Shape<R> c2; c2.type = SHAPE_CUBOID; c2.half = h2;
  Vec3<R> x2 = pos12.transform_vector(Vec3<R>(1, 0, 0)), y2 = pos12.transform_vector(Vec3<R>(0, 1, 0)), z2 = pos12.transform_vector(Vec3<R>(0, 0, 1));
  Vec3<R> axes[9] = {Vec3<R>(0, -x2.z, x2.y), Vec3<R>(x2.z, 0, -x2.x), Vec3<R>(-x2.y, x2.x, 0),
                     Vec3<R>(0, -y2.z, y2.y), Vec3<R>(y2.z, 0, -y2.x), Vec3<R>(-y2.y, y2.x, 0),
                     Vec3<R>(0, -z2.z, z2.y), Vec3<R>(z2.z, 0, -z2.x), Vec3<R>(-z2.y, z2.x, 0)};
  for (auto& ax : axes) {
    R n = norm(ax);
    if (n > eps_default<R>()) {
      Vec3<R> a = ax / n;
      R signum = std::copysign(R(1), dot(pos12.tra, a));
      Vec3<R> a1 = a * signum;
      Vec3<R> a2 = pos12.inverse_transform_vector(-a1);
      Vec3<R> lp1 = c1.local_support(a1);
      Vec3<R> lp2 = c2.local_support(a2);
      Vec3<R> p2 = pos12.transform_point(lp2);
      R sep = dot(p2 - lp1, a1);
      if (sep > best) { best = sep; best_dir = a1; }
    }
  }
  return {best, best_dir};
}

// contact_manifolds_cuboid_cuboid.rs:21-107
template <class R> inline void manifold_cuboid_cuboid(const Iso<R>& pos12, const Vec3<R>& h1, const Vec3<R>& h2, R prediction, Manifold<R>& m) {
  if (m.try_update_contacts(pos12)) return;
  Iso<R> pos21 = pos12.inverse();
  auto sep1 = sat_normal_oneway(h1, h2, pos12);
  if (sep1.first > prediction) { m.points.clear(); return; }
  auto sep2 = sat_normal_oneway(h2, h1, pos21);
  if (sep2.first > prediction) { m.points.clear(); return; }
  auto sep3 = sat_edge_twoway(h1, h2, pos12);
  if (sep3.first > prediction) { m.points.clear(); return; }
  std::pair<R, Vec3<R>> best = sep1;
  if (sep2.first > sep1.first && sep2.first > sep3.first) best = {sep2.first, pos12.transform_vector(-sep2.second)};
  else if (sep3.first > sep1.first) best = sep3;
  auto old = m.points;
  m.points.clear();
  Vec3<R> n2 = pos21.transform_vector(-best.second);
  PolyFeature<R> f1 = cuboid_support_face(h1, best.second);
  PolyFeature<R> f2 = cuboid_support_face(h2, n2);
  feature_contacts(pos12, best.second, f1, f2, m, false);
  m.local_n1 = best.second;
  m.local_n2 = n2;
  m.match_contacts(old);
}

// sat_cuboid_support_map.rs:54-73 with a triangle as the support map.
template <class R>
inline std::pair<R, Vec3<R>> sat_cuboid_triangle_normal_oneway(const Vec3<R>& he1, const Shape<R>& tri2, const Iso<R>& pos12) {
  R best = -std::numeric_limits<R>::max();
  Vec3<R> best_dir;
  for (int i = 0; i < 3; ++i) {
    for (R sign : {R(-1), R(1)}) {
      Vec3<R> axis1;
      axis1[i] = sign;
      Vec3<R> pt2 = tri2.support(pos12, -axis1);  // support_point_toward(pos12, -axis1)
      R sep = pt2[i] * sign - he1[i];
      if (sep > best) { best = sep; best_dir = axis1; }
    }
  }
  return {best, best_dir};
}

// sat_cuboid_point.rs point_cuboid_find_local_separating_normal_oneway (the triangle's first vertex
// and normal against the cuboid, in the triangle's frame).
template <class R>
inline std::pair<R, Vec3<R>> sat_point_cuboid_normal_oneway(const Vec3<R>& point1, bool has_normal, const Vec3<R>& normal1, const Vec3<R>& he2,
                                                            const Iso<R>& pos12) {
  R best = -std::numeric_limits<R>::max();
  Vec3<R> best_dir;
  if (has_normal) {
    Vec3<R> axis1 = dot(pos12.tra - point1, normal1) >= R(0) ? normal1 : -normal1;
    Shape<R> cub;
    cub.type = SHAPE_CUBOID;
    cub.half = he2;
    Vec3<R> pt2 = cub.support(pos12, -axis1);
    R sep = dot(pt2 - point1, axis1);
    if (sep > best) { best = sep; best_dir = axis1; }
  }
  return {best, best_dir};
}

// sat_cuboid_triangle.rs cuboid_triangle_find_local_separating_edge_twoway (3-D)
template <class R>
inline std::pair<R, Vec3<R>> sat_cuboid_triangle_edge_twoway(const Vec3<R>& he1, const Shape<R>& tri2, const Iso<R>& pos12) {
  Vec3<R> a = pos12.transform_point(tri2.pts[0]), b = pos12.transform_point(tri2.pts[1]), c = pos12.transform_point(tri2.pts[2]);
  Vec3<R> ab = b - a, bc = c - b, ca = a - c;
  const Vec3<R> axes[9] = {Vec3<R>(0, -ab.z, ab.y), Vec3<R>(ab.z, 0, -ab.x), Vec3<R>(-ab.y, ab.x, 0),
                           Vec3<R>(0, -bc.z, bc.y), Vec3<R>(bc.z, 0, -bc.x), Vec3<R>(-bc.y, bc.x, 0),
                           Vec3<R>(0, -ca.z, ca.y), Vec3<R>(ca.z, 0, -ca.x), Vec3<R>(-ca.y, ca.x, 0)};
  R best = -std::numeric_limits<R>::max();
  Vec3<R> best_axis = axes[0];
  Shape<R> cub;
  cub.type = SHAPE_CUBOID;
  cub.half = he1;
  for (int i = 0; i < 9; ++i) {
    const Vec3<R>& axis = axes[i];
    R d0 = dot(axis, a), d1 = i < 6 ? dot(axis, c) : dot(axis, b);
    R n2 = norm_squared(axis);
    if (n2 > eps_default<R>()) {
      R n = std::sqrt(n2);
      Vec3<R> pt1 = cub.local_support(axis);
      R dot1 = dot(pt1, axis) / n;
      R mn = d0 > d1 ? d1 : d0, mx = d0 > d1 ? d0 : d1;  // utils::sort2
      R sep_a = mn / n - dot1;
      R sep_b = -mx / n - dot1;
      if (sep_a > best) { best = sep_a; best_axis = axis / n; }
      if (sep_b > best) { best = sep_b; best_axis = -axis / n; }
    }
  }
  return {best, best_axis};
}

// contact_manifolds_cuboid_triangle.rs:57-174: the cuboid is shape 1 of the SAT; `flipped` when the
// triangle is the manifold's first shape; c1 / c2 = normal constraints of the cuboid / triangle.
template <class R>
inline void manifold_cuboid_triangle(const Iso<R>& pos12, const Iso<R>& pos21, const Vec3<R>& he1, const Shape<R>& tri2, R prediction,
                                     Manifold<R>& m, bool flipped, const TriPseudoNormals<R>* c1 = nullptr,
                                     const TriPseudoNormals<R>* c2 = nullptr) {
  if ((!flipped && m.try_update_contacts(pos12)) || (flipped && m.try_update_contacts(pos21))) return;
  auto sep1 = sat_cuboid_triangle_normal_oneway(he1, tri2, pos12);
  if (sep1.first > prediction) { m.points.clear(); return; }
  Vec3<R> tn;
  bool has_n = try_normalize(cross(tri2.pts[1] - tri2.pts[0], tri2.pts[2] - tri2.pts[0]), eps_default<R>(), &tn);
  auto sep2 = sat_point_cuboid_normal_oneway(tri2.pts[0], has_n, tn, he1, pos21);
  if (sep2.first > prediction) { m.points.clear(); return; }
  auto sep3 = sat_cuboid_triangle_edge_twoway(he1, tri2, pos12);
  if (sep3.first > prediction) { m.points.clear(); return; }
  Vec3<R> normal1 = sep1.second;
  R dist = sep1.first;
  if (sep2.first > sep1.first && sep2.first > sep3.first) { normal1 = pos12.transform_vector(-sep2.second); dist = sep2.first; }
  else if (sep3.first > sep1.first) { normal1 = sep3.second; dist = sep3.first; }
  Vec3<R> normal2 = pos21.transform_vector(-normal1);
  if (!project_local_normals(c1, c2, pos12, &normal1, &normal2)) {
    m.points.clear();  // the contact got discarded by the normal correction
    return;
  }
  PolyFeature<R> f1 = cuboid_support_face(he1, normal1);
  PolyFeature<R> f2 = triangle_feature(tri2);
  auto old = m.points;
  m.points.clear();
  feature_contacts(pos12, normal1, f1, f2, m, flipped);
  if (c1 || c2) {
    // drop points whose depth diverges from the unconstrained one (the reference's retain filter)
    std::vector<TrackedContact<R>> kept;
    for (const auto& c : m.points)
      if (dist >= R(0) || c.dist >= R(0) || c.dist >= dist * R(5)) kept.push_back(c);
    m.points.swap(kept);
  }
  if (flipped) { m.local_n1 = normal2; m.local_n2 = normal1; }
  else { m.local_n1 = normal1; m.local_n2 = normal2; }
  m.match_contacts(old);
}

// contact_manifolds_pfm_pfm.rs:44-162 for cuboids, capsules (segment + border radius), triangles and
// hulls; c1 / c2 = normal constraints of shape 1 / 2. `learned` (may be null) is a caller-supplied
// GJK start direction, used when the manifold holds no cached normal (contact_manifolds_pfm_pfm.rs:67-76
// then falls back to the relative translation, else +x; a learned direction that does not normalise
// keeps that fallback).
template <class R> inline void manifold_pfm_pfm(const Iso<R>& pos12, const Shape<R>& s1, const Shape<R>& s2, R prediction, Manifold<R>& m,
                                                GjkStats* st, const TriPseudoNormals<R>* c1 = nullptr,
                                                const TriPseudoNormals<R>* c2 = nullptr, const Vec3<R>* learned = nullptr) {
  if (m.try_update_contacts_eps(pos12, cos_1_degrees<R>(), R(1.0e-6))) return;
  auto pfm = [](const Shape<R>& s, R* border) {
    Shape<R> p = s;
    *border = R(0);
    if (s.type == SHAPE_CAPSULE) { p.type = SHAPE_SEGMENT_PFM; *border = s.radius; }
    return p;
  };
  R br1, br2;
  Shape<R> p1 = pfm(s1, &br1), p2 = pfm(s2, &br2);
  Vec3<R> init;
  bool has_init = try_normalize(m.local_n1, eps_default<R>(), &init);
  if (!has_init && learned) has_init = try_normalize(*learned, eps_default<R>(), &init);
  R total_prediction = (prediction + br1) + br2;
  VoronoiSimplex<R> simplex;
  GjkResult<R> r = contact_support_map_support_map_with_params(pos12, p1, p2, total_prediction, simplex, has_init ? &init : nullptr, st);
  auto old = m.points;
  m.points.clear();
  if (r.kind == GJK_CLOSEST_POINTS) {
    Vec3<R> n1 = r.dir;
    Vec3<R> n2 = pos12.inverse_transform_vector(-r.dir);
    const R dist = dot(r.p2 - r.p1, n1);
    if (!project_local_normals(c1, c2, pos12, &n1, &n2)) return;  // discarded: points cleared, no matching
    auto feature_of = [](const Shape<R>& s, const Vec3<R>& d) {
      if (s.type == SHAPE_CUBOID) return cuboid_support_face(s.half, d);
      if (s.type == SHAPE_CONVEX) return hull_support_feature(s, d);
      if (s.type == SHAPE_TRIANGLE) return triangle_feature(s);
      return segment_feature(s.half_height);
    };
    PolyFeature<R> f1 = feature_of(s1, n1), f2 = feature_of(s2, n2);
    feature_contacts(pos12, n1, f1, f2, m, false);
    // the GJK point only while the normal is GJK's own direction
    if (n1 == r.dir)
      m.points.push_back(TrackedContact<R>::make(r.p1, pos12.inverse_transform_point(r.p2), PFID_UNKNOWN, PFID_UNKNOWN, dot(r.p2 - r.p1, n1), false));
    if (c1 || c2) {
      std::vector<TrackedContact<R>> kept;
      for (const auto& c : m.points)
        if (dist >= R(0) || c.dist >= R(0) || c.dist >= dist * R(5)) kept.push_back(c);
      m.points.swap(kept);
    }
    if (br1 != R(0) || br2 != R(0)) {
      for (auto& c : m.points) {
        c.local_p1 += n1 * br1;
        c.local_p2 += n2 * br2;
        c.dist -= br1 + br2;
      }
    }
    m.local_n1 = n1;
    m.local_n2 = n2;
  } else if (r.kind == GJK_NO_INTERSECTION) {
    m.local_n1 = r.dir;
  } else {
    m.local_n1 = Vec3<R>();
  }
  m.match_contacts(old);
}

// DefaultQueryDispatcher::contact_manifold_convex_convex (default_query_dispatcher.rs:749-831) for
// balls, cuboids, capsules, triangles and convex polyhedra, with the optional normal constraints of
// each shape. Returns false (Unsupported) for other shapes.
template <class R>
inline bool contact_manifold_convex_convex(const Iso<R>& pos12, const Shape<R>& s1, const Shape<R>& s2, R prediction, Manifold<R>& m,
                                           GjkStats* st = nullptr, const TriPseudoNormals<R>* c1 = nullptr,
                                           const TriPseudoNormals<R>* c2 = nullptr, const Vec3<R>* learned = nullptr) {
  auto ok = [](const Shape<R>& s) {
    return s.type == SHAPE_BALL || s.type == SHAPE_CUBOID || s.type == SHAPE_CAPSULE || s.type == SHAPE_TRIANGLE ||
           (s.type == SHAPE_CONVEX && s.topo && s.topo->n_faces);
  };
  if (!ok(s1) || !ok(s2)) return false;
  if (s1.type == SHAPE_BALL && s2.type == SHAPE_BALL) manifold_ball_ball(pos12, s1.radius, s2.radius, prediction, m);
  else if (s1.type == SHAPE_CUBOID && s2.type == SHAPE_CUBOID) manifold_cuboid_cuboid(pos12, s1.half, s2.half, prediction, m);
  else if (s1.type == SHAPE_CUBOID && s2.type == SHAPE_TRIANGLE)
    manifold_cuboid_triangle(pos12, pos12.inverse(), s1.half, s2, prediction, m, false, c1, c2);
  else if (s1.type == SHAPE_TRIANGLE && s2.type == SHAPE_CUBOID)
    manifold_cuboid_triangle(pos12.inverse(), pos12, s2.half, s1, prediction, m, true, c2, c1);
  else if (s1.type == SHAPE_CAPSULE && s2.type == SHAPE_CAPSULE)
    manifold_capsule_capsule(pos12, s1.half_height, s1.radius, s2.half_height, s2.radius, prediction, m);
  else if (s1.type == SHAPE_BALL) manifold_convex_ball(pos12.inverse(), s2, s1.radius, prediction, m, true, st, c2, c1);
  else if (s2.type == SHAPE_BALL) manifold_convex_ball(pos12, s1, s2.radius, prediction, m, false, st, c1, c2);
  else manifold_pfm_pfm(pos12, s1, s2, prediction, m, st, c1, c2, learned);
  return true;
}

}  // namespace oracle
