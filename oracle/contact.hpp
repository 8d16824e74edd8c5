// Oracle (test infrastructure only): CPU restatement of parry3d's query::contact for convex shapes
// (ball, cuboid, capsule, convex polyhedron) and of the shape AABB formulas. Paths relative to the
// parry repository:
//   src/query/contact/contact_shape_shape.rs:123-138          query::contact (world transform)
//   src/query/default_query_dispatcher.rs:302-356             dispatch order
//   src/query/contact/contact_ball_ball.rs:9-42
//   src/query/contact/contact_ball_convex_polyhedron.rs:12-63
//   src/query/contact/contact_support_map_support_map.rs:10-77 (init_dir warm start)
//   src/query/point/point_aabb.rs:9-132, point_cuboid.rs, point_capsule.rs:7-51,
//   src/query/point/point_support_map.rs:17-77
//   src/bounding_volume/aabb_ball.rs:7-33, aabb_cuboid.rs:9-14, aabb_capsule.rs:8-20,
//   src/bounding_volume/aabb_convex_polyhedron.rs:8-10 + aabb_utils.rs:58-86, aabb.rs:303-305, :982
#pragma once
#include "epa.hpp"

namespace oracle {

template <class R> struct Contact {
  Vec3<R> point1, point2, normal1, normal2;
  R dist;
  void flip() { std::swap(point1, point2); std::swap(normal1, normal2); }
};

// contact_ball_ball.rs:9-42
template <class R> inline bool contact_ball_ball(const Iso<R>& pos12, R r1, R r2, R prediction, Contact<R>* c) {
  Vec3<R> center2_1 = pos12.tra;
  R d2 = norm_squared(center2_1);
  R sum = r1 + r2;
  R sum_err = sum + prediction;
  if (!(d2 < sum_err * sum_err)) return false;
  Vec3<R> n1 = d2 != R(0) ? normalize(center2_1) : Vec3<R>(1, 0, 0);
  Vec3<R> n2 = -pos12.inverse_transform_vector(n1);
  c->point1 = n1 * r1;
  c->point2 = n2 * r2;
  c->normal1 = n1;
  c->normal2 = n2;
  c->dist = std::sqrt(d2) - sum;
  return true;
}

template <class R> struct PointProj {
  bool is_inside;
  Vec3<R> point;
  int face = -1;  // cuboid: FeatureId::Face(i) when the projection is on a face, -1 otherwise
  Vec3<R> shift;  // cuboid: the shift do_project_local_point returns (ls = pt + shift)
};

// point_aabb.rs:9-132 on the cuboid [-h, h] with solid = false (project_local_point_and_get_feature).
template <class R> inline PointProj<R> project_cuboid(const Vec3<R>& h, const Vec3<R>& pt) {
  Vec3<R> mins = -h, maxs = h;
  Vec3<R> mins_pt = mins - pt;
  Vec3<R> pt_maxs = pt - maxs;
  Vec3<R> shift = vsup(mins_pt, Vec3<R>()) - vsup(pt_maxs, Vec3<R>());
  bool inside = shift.x == R(0) && shift.y == R(0) && shift.z == R(0);
  PointProj<R> out;
  Vec3<R> ls;
  if (!inside) {
    ls = pt + shift;
    out.is_inside = false;
  } else {
    R best = -std::numeric_limits<R>::max();
    bool is_mins = false;
    int best_id = 0;
    for (int i = 0; i < 3; ++i) {
      R a = mins_pt[i], b = pt_maxs[i];
      if (a < b) {
        if (pt_maxs[i] > best) { best_id = i; is_mins = false; best = b; }
      } else if (a > best) { best_id = i; is_mins = true; best = a; }
    }
    Vec3<R> s;
    s[best_id] = is_mins ? best : -best;
    shift = s;
    ls = pt + s;
    out.is_inside = true;
  }
  out.point = ls;
  out.shift = shift;
  // feature: only the face case is needed (feature_normal_at_point fallback)
  int nz = 0, last_nz = 0;
  for (int i = 0; i < 3; ++i) { if (shift[i] == R(0)) nz++; else last_nz = i; }
  Vec3<R> center = (mins + maxs) * R(0.5);
  if (nz == 3) {
    for (int i = 0; i < 3; ++i) {
      if (ls[i] > maxs[i] - eps_default<R>()) { out.face = i; break; }
      if (ls[i] <= mins[i] + eps_default<R>()) { out.face = i + 3; break; }
    }
  } else if (nz == 2) {
    out.face = ls[last_nz] < center[last_nz] ? last_nz + 3 : last_nz;
  }
  return out;
}

// point_capsule.rs:7-51 with solid = false.
template <class R> inline PointProj<R> project_capsule(R hh, R radius, const Vec3<R>& pt) {
  Loc<R> loc;
  Vec3<R> a(0, -hh, 0), b(0, hh, 0);
  Vec3<R> proj = project_segment(a, b, pt, &loc);
  Vec3<R> dproj = pt - proj;
  Vec3<R> dir;
  R dist;
  PointProj<R> out;
  if (try_normalize(dproj, eps_default<R>(), &dir, &dist)) {
    out.is_inside = dist <= radius;
    out.point = proj + dir * radius;
    return out;
  }
  // degenerate: the point lies on the segment; Segment::direction -> orthonormal_basis()[0]
  Vec3<R> sd;
  if (try_normalize(b - a, eps_default<R>(), &sd)) {
    // utils WBasis::orthonormal_basis (Pixar "Building an Orthonormal Basis, Revisited")
    R sign = std::copysign(R(1), sd.z);
    R aa = R(-1) / (sign + sd.z);
    R bb = sd.x * sd.y * aa;
    Vec3<R> t(R(1) + sign * sd.x * sd.x * aa, sign * bb, -sign * sd.x);
    out.is_inside = true;
    out.point = proj + t * radius;
  } else {
    out.is_inside = true;
    out.point = proj + Vec3<R>(0, radius, 0);
  }
  return out;
}

// point_support_map.rs:17-57 with solid = false.
template <class R> inline PointProj<R> project_support_map(const Shape<R>& s, const Vec3<R>& point, GjkStats* st) {
  Iso<R> m(Quat<R>(), -point);
  Iso<R> m_inv(Quat<R>(), point);
  Vec3<R> dir;
  if (!try_normalize(-m.tra, eps_default<R>(), &dir)) dir = Vec3<R>(1, 0, 0);
  Support<R> g1{&s}, g2{nullptr};
  CSOPoint<R> sp = cso_from_shapes(m_inv, g1, g2, dir);
  VoronoiSimplex<R> simplex;
  simplex.reset(sp);
  Iso<R> minv = m.inverse();
  GjkResult<R> r = gjk_closest_points(minv, g1, g2, std::numeric_limits<R>::max(), simplex, st);
  PointProj<R> out;
  if (r.kind == GJK_CLOSEST_POINTS) { out.is_inside = false; out.point = r.p1; return out; }
  Epa<R> epa;
  Vec3<R> p1, p2, n;
  if (epa.closest_points(minv, g1, g2, simplex, &p1, &p2, &n, st)) { out.is_inside = true; out.point = p1; return out; }
  out.is_inside = true;
  out.point = point;
  return out;
}

template <class R> inline PointProj<R> project_local_point_and_get_feature(const Shape<R>& s, const Vec3<R>& pt, GjkStats* st) {
  switch (s.type) {
    case SHAPE_CUBOID: return project_cuboid(s.half, pt);
    case SHAPE_CAPSULE: return project_capsule(s.half_height, s.radius, pt);
    default: return project_support_map(s, pt, st);
  }
}

// contact_ball_convex_polyhedron.rs:26-63
template <class R>
inline bool contact_convex_ball(const Iso<R>& pos12, const Shape<R>& s1, R r2, R prediction, Contact<R>* c, GjkStats* st) {
  Vec3<R> center2_1 = pos12.tra;
  PointProj<R> proj = project_local_point_and_get_feature(s1, center2_1, st);
  R dist;
  Vec3<R> n1;
  Vec3<R> dir1;
  R len;
  if (try_normalize(proj.point - center2_1, eps_default<R>(), &dir1, &len)) {
    if (proj.is_inside) { dist = -len - r2; n1 = dir1; }
    else { dist = len - r2; n1 = -dir1; }
  } else {
    dist = -r2;
    if (s1.type == SHAPE_CUBOID && proj.face >= 0) {
      Vec3<R> d;
      if (proj.face < 3) d[proj.face] = R(1); else d[proj.face - 3] = R(-1);
      n1 = d;
    } else if (!try_normalize(proj.point, eps_default<R>(), &n1)) {
      n1 = Vec3<R>(0, 1, 0);
    }
  }
  if (!(dist <= prediction)) return false;
  Vec3<R> n2 = pos12.inverse_transform_vector(-n1);
  c->point1 = proj.point;
  c->point2 = n2 * r2;
  c->normal1 = n1;
  c->normal2 = n2;
  c->dist = dist;
  return true;
}

// contact_support_map_support_map.rs:40-77. init_dir = nullptr for the default direction.
template <class R>
inline GjkResult<R> contact_support_map_support_map_with_params(const Iso<R>& pos12, const Shape<R>& s1, const Shape<R>& s2, R prediction,
                                                               VoronoiSimplex<R>& simplex, const Vec3<R>* init_dir, GjkStats* st) {
  Vec3<R> dir;
  if (init_dir) dir = *init_dir;
  else if (!try_normalize(pos12.tra, eps_default<R>(), &dir)) dir = Vec3<R>(1, 0, 0);
  Support<R> g1{&s1}, g2{&s2};
  simplex.reset(cso_from_shapes(pos12, g1, g2, dir));
  GjkResult<R> r = gjk_closest_points(pos12, g1, g2, prediction, simplex, st);
  if (r.kind != GJK_INTERSECTION) return r;
  Epa<R> epa;
  Vec3<R> p1, p2, n;
  if (epa.closest_points(pos12, g1, g2, simplex, &p1, &p2, &n, st)) return {GJK_CLOSEST_POINTS, p1, p2, n};
  return {GJK_NO_INTERSECTION, {}, {}, Vec3<R>(1, 0, 0)};
}

template <class R>
inline bool contact_support_map_support_map(const Iso<R>& pos12, const Shape<R>& s1, const Shape<R>& s2, R prediction,
                                            const Vec3<R>* init_dir, Contact<R>* c, GjkStats* st) {
  VoronoiSimplex<R> simplex;
  GjkResult<R> r = contact_support_map_support_map_with_params(pos12, s1, s2, prediction, simplex, init_dir, st);
  if (r.kind != GJK_CLOSEST_POINTS) return false;
  c->dist = dot(r.p2 - r.p1, r.dir);
  c->point1 = r.p1;
  c->point2 = pos12.inverse_transform_point(r.p2);
  c->normal1 = r.dir;
  c->normal2 = pos12.inverse_transform_vector(-r.dir);
  return true;
}

// DefaultQueryDispatcher::contact (default_query_dispatcher.rs:302-356), all shapes convex.
template <class R>
inline bool contact_local(const Iso<R>& pos12, const Shape<R>& s1, const Shape<R>& s2, R prediction, const Vec3<R>* init_dir,
                          Contact<R>* c, GjkStats* st) {
  if (s1.is_ball() && s2.is_ball()) return contact_ball_ball(pos12, s1.radius, s2.radius, prediction, c);
  if (s1.is_ball()) {
    if (!contact_convex_ball(pos12.inverse(), s2, s1.radius, prediction, c, st)) return false;
    c->flip();
    return true;
  }
  if (s2.is_ball()) return contact_convex_ball(pos12, s1, s2.radius, prediction, c, st);
  return contact_support_map_support_map(pos12, s1, s2, prediction, init_dir, c, st);
}

// query::contact(pos1, g1, pos2, g2, prediction) (contact_shape_shape.rs:123-138)
template <class R>
inline bool contact_world(const Iso<R>& pos1, const Shape<R>& s1, const Iso<R>& pos2, const Shape<R>& s2, R prediction, Contact<R>* c,
                          GjkStats* st = nullptr, const Vec3<R>* init_dir = nullptr) {
  Iso<R> pos12 = pos1.inv_mul(pos2);
  if (!contact_local(pos12, s1, s2, prediction, init_dir, c, st)) return false;
  c->point1 = pos1.transform_point(c->point1);
  c->point2 = pos2.transform_point(c->point2);
  c->normal1 = pos1.transform_vector(c->normal1);
  c->normal2 = pos2.transform_vector(c->normal2);
  return true;
}

// Shape::compute_aabb(pos) for the supported shapes.
template <class R> inline Aabb<R> shape_aabb(const Shape<R>& s, const Iso<R>& pos) {
  switch (s.type) {
    case SHAPE_BALL: return Aabb<R>(pos.tra + Vec3<R>::repeat(-s.radius), pos.tra + Vec3<R>::repeat(s.radius));
    case SHAPE_CUBOID: {
      Vec3<R> he = absolute_transform_vector(pos, s.half);
      return Aabb<R>(pos.tra - he, pos.tra + he);
    }
    case SHAPE_CAPSULE: {
      Vec3<R> a = pos.transform_point(Vec3<R>(0, -s.half_height, 0));
      Vec3<R> b = pos.transform_point(Vec3<R>(0, s.half_height, 0));
      return Aabb<R>(vinf(a, b) - Vec3<R>::repeat(s.radius), vsup(a, b) + Vec3<R>::repeat(s.radius));
    }
    default: {
      Vec3<R> p0 = pos.transform_point(s.pts[0]);
      Aabb<R> r(p0, p0);
      for (uint32_t i = 1; i < s.npts; ++i) {
        Vec3<R> p = pos.transform_point(s.pts[i]);
        r.mins = vinf(r.mins, p);
        r.maxs = vsup(r.maxs, p);
      }
      return r;
    }
  }
}

}  // namespace oracle
