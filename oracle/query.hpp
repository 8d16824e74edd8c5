// Oracle (test infrastructure only): CPU restatement of parry3d's convex contact queries
// (support maps, Voronoi simplex, GJK, EPA, query::contact). Used by tests/, the smoke check and the
// bench's CPU-baseline leg as the checker; the product path never calls it.
//
// Follows (paths relative to the parry repository):
//   src/shape/ball.rs:242-249, cuboid.rs:454-456, capsule.rs:407-418, convex_polyhedron.rs:952-957,
//   src/utils/point_cloud_support_point.rs:5-19, src/utils/wops.rs:30-36 (copy_sign_to),
//   src/shape/triangle.rs:697-715,
//   src/shape/support_map.rs:380-383                      support maps
//   src/query/gjk/cso_point.rs:13-98                      CSOPoint
//   src/query/point/point_segment.rs:49-84, point_triangle.rs:58-291, point_tetrahedron.rs:32-340
//   src/query/gjk/voronoi_simplex3.rs:14-351              VoronoiSimplex
//   src/query/gjk/gjk.rs:141-144, 196-213, 353-453, 797-818  GJK
//   src/query/epa/epa3.rs:17-675                          EPA (with Rust's BinaryHeap order)
//   src/query/contact/contact_support_map_support_map.rs:10-77
//   src/query/contact/contact_ball_ball.rs:9-42, contact_ball_convex_polyhedron.rs:12-63
//   src/query/point/point_aabb.rs:9-132, point_cuboid.rs, point_capsule.rs:7-51,
//   src/query/point/point_support_map.rs:17-77
//   src/query/default_query_dispatcher.rs:302-356, src/query/contact/contact_shape_shape.rs:123-138
#pragma once
#include "bvh.hpp"
#include <atomic>
#include <vector>
#include <cstring>

namespace oracle {

template <class R> inline R eps_default() { return std::numeric_limits<R>::epsilon(); }
template <class R> inline R gjk_eps_tol() { return eps_default<R>() * R(10); }

enum ShapeType : uint32_t { SHAPE_BALL = 0, SHAPE_CUBOID = 1, SHAPE_CAPSULE = 2, SHAPE_CONVEX = 3, SHAPE_TRIANGLE = 4,
                            SHAPE_SEGMENT_PFM = 5 /* a capsule's axis segment, as its polygonal feature map */ };

// ConvexPolyhedron topology of one hull (convex_polyhedron.rs:172-185, built by from_convex_mesh),
// ids hull-local. face_normals / face_ranges / vertex_ranges / edge_dirs point at this hull's rows;
// the ranges index the shared face_vertices / face_edges / vertex_faces / vertex_edges arrays.
struct HullTopo {
  uint32_t n_faces = 0, n_edges = 0;
  const float* face_normals = nullptr;
  const uint32_t* face_ranges = nullptr;
  const uint32_t* face_vertices = nullptr;
  const uint32_t* face_edges = nullptr;
  const uint32_t* vertex_ranges = nullptr;
  const uint32_t* vertex_faces = nullptr;
  const uint32_t* vertex_edges = nullptr;
  const float* edge_dirs = nullptr;
};

// One convex shape. Capsule = Capsule::new_y(half_height, radius): segment (0,-h,0)-(0,h,0).
template <class R> struct Shape {
  uint32_t type = SHAPE_BALL;
  R radius = 0;                 // ball, capsule
  Vec3<R> half;                 // cuboid half extents
  R half_height = 0;            // capsule
  const Vec3<R>* pts = nullptr; // convex hull vertices (triangle: its 3 vertices)
  uint32_t npts = 0;
  const HullTopo* topo = nullptr;  // convex: face topology when built as a ConvexPolyhedron

  // SupportMap::local_support_point
  Vec3<R> local_support(const Vec3<R>& dir) const {
    switch (type) {
      case SHAPE_BALL: return normalize(dir) * radius;
      case SHAPE_CUBOID: {
        Vec3<R> r;
        for (int i = 0; i < 3; ++i) r[i] = std::copysign(half[i], dir[i]);
        return r;
      }
      case SHAPE_CAPSULE: {
        Vec3<R> d;
        if (!try_normalize(dir, R(0), &d)) d = Vec3<R>(0, 1, 0);
        Vec3<R> a(0, -half_height, 0), b(0, half_height, 0);
        if (dot(d, a) > dot(d, b)) return a + d * radius;
        return b + d * radius;
      }
      case SHAPE_SEGMENT_PFM: {
        // segment.rs:461-467: a if a.dir > b.dir else b
        Vec3<R> a(0, -half_height, 0), b(0, half_height, 0);
        return dot(a, dir) > dot(b, dir) ? a : b;
      }
      case SHAPE_TRIANGLE: {
        // triangle.rs:697-715: ties resolve towards the later vertex
        R d1 = dot(pts[0], dir), d2 = dot(pts[1], dir), d3 = dot(pts[2], dir);
        if (d1 > d2) return d1 > d3 ? pts[0] : pts[2];
        return d2 > d3 ? pts[1] : pts[2];
      }
      default: {
        uint32_t best = 0;
        R bd = dot(pts[0], dir);
        for (uint32_t i = 1; i < npts; ++i) {
          R d = dot(pts[i], dir);
          if (d > bd) { bd = d; best = i; }
        }
        return pts[best];
      }
    }
  }
  // SupportMap::local_support_point_toward for a unit direction: the ball and the capsule use it
  // without renormalising (ball.rs:247-249, capsule.rs:412-418); the others forward to
  // local_support_point (support_map.rs:302).
  Vec3<R> local_support_toward(const Vec3<R>& u) const {
    if (type == SHAPE_BALL) return u * radius;
    if (type == SHAPE_CAPSULE) {
      Vec3<R> a(0, -half_height, 0), b(0, half_height, 0);
      if (dot(u, a) > dot(u, b)) return a + u * radius;
      return b + u * radius;
    }
    return local_support(u);
  }
  // SupportMap::support_point(transform, dir)
  Vec3<R> support(const Iso<R>& m, const Vec3<R>& dir) const {
    Vec3<R> ld = m.inverse_transform_vector(dir);
    return m.transform_point(local_support(ld));
  }
  bool is_ball() const { return type == SHAPE_BALL; }
};

// Support of the constant origin (special_support_maps.rs ConstantOrigin) under pos12.
template <class R> struct OriginShape {};

template <class R> struct CSOPoint {
  Vec3<R> point, orig1, orig2;
  static CSOPoint make(const Vec3<R>& o1, const Vec3<R>& o2) { return {o1 - o2, o1, o2}; }
  static CSOPoint single_point(const Vec3<R>& p) { return {p, p, Vec3<R>()}; }
  CSOPoint translate(const Vec3<R>& d) const { return {point + d, orig1, orig2}; }
};

// Support provider: either a shape or the constant origin (for point projections).
// Counts the vertices scanned by support calls (the dominant FP32 work: 5 flops per vertex dot).
inline thread_local uint64_t g_support_vertices = 0;

template <class R> struct Support {
  const Shape<R>* shape;  // nullptr = ConstantOrigin
  // RoundShapeRef (round_shape.rs:330-349): support toward the normalised direction plus the
  // direction times the border radius.
  bool round = false;
  R border = R(0);
  static void count(const Shape<R>* s) {
    if (s && (s->type == SHAPE_CONVEX || s->type == SHAPE_TRIANGLE)) g_support_vertices += s->npts;
  }
  Vec3<R> local(const Vec3<R>& d) const {
    count(shape);
    if (!shape) return Vec3<R>();
    if (round) {
      Vec3<R> u = normalize(d);  // Unit::new_normalize
      return shape->local_support_toward(u) + u * border;
    }
    return shape->local_support(d);
  }
  Vec3<R> world(const Iso<R>& m, const Vec3<R>& d) const {
    if (!shape) { count(shape); return m.tra; }
    if (round) return m.transform_point(local(m.inverse_transform_vector(d)));
    count(shape);
    return shape->support(m, d);
  }
};

template <class R>
inline CSOPoint<R> cso_from_shapes(const Iso<R>& pos12, const Support<R>& g1, const Support<R>& g2, const Vec3<R>& dir) {
  Vec3<R> sp1 = g1.local(dir);
  Vec3<R> sp2 = g2.world(pos12, -dir);
  return CSOPoint<R>::make(sp1, sp2);
}

// ---------------- point projections with location (solid = true) ----------------

enum LocKind { LOC_VERTEX, LOC_EDGE, LOC_FACE, LOC_SOLID };
template <class R> struct Loc {
  LocKind kind;
  int id;      // vertex / edge / face index (face side for triangles)
  R bc[3];     // barycentric coordinates (2 for edges, 3 for faces)
};

// point_segment.rs:49-84
template <class R> inline Vec3<R> project_segment(const Vec3<R>& a, const Vec3<R>& b, const Vec3<R>& pt, Loc<R>* loc) {
  Vec3<R> ab = b - a;
  Vec3<R> ap = pt - a;
  R ab_ap = dot(ab, ap);
  R sqnab = norm_squared(ab);
  if (ab_ap <= R(0)) { *loc = {LOC_VERTEX, 0, {1, 0, 0}}; return a; }
  if (ab_ap >= sqnab) { *loc = {LOC_VERTEX, 1, {0, 1, 0}}; return b; }
  R u = ab_ap / sqnab;
  *loc = {LOC_EDGE, 0, {R(1) - u, u, 0}};
  return a + ab * u;
}

// point_triangle.rs:58-291 (3-D, solid)
template <class R>
inline Vec3<R> project_triangle(const Vec3<R>& a, const Vec3<R>& b, const Vec3<R>& c, const Vec3<R>& pt, Loc<R>* loc) {
  Vec3<R> ab = b - a, ac = c - a, ap = pt - a;
  R ab_ap = dot(ab, ap), ac_ap = dot(ac, ap);
  if (ab_ap <= R(0) && ac_ap <= R(0)) { *loc = {LOC_VERTEX, 0, {1, 0, 0}}; return a; }
  Vec3<R> bp = pt - b;
  R ab_bp = dot(ab, bp), ac_bp = dot(ac, bp);
  if (ab_bp >= R(0) && ac_bp <= ab_bp) { *loc = {LOC_VERTEX, 1, {0, 1, 0}}; return b; }
  Vec3<R> cp = pt - c;
  R ab_cp = dot(ab, cp), ac_cp = dot(ac, cp);
  if (ac_cp >= R(0) && ab_cp <= ac_cp) { *loc = {LOC_VERTEX, 2, {0, 0, 1}}; return c; }
  Vec3<R> bc = c - b;
  // stable_check_edges_voronoi (dim3, no improved_fixed_point_support)
  Vec3<R> n = cross(ab, ac);
  R vc = dot(n, cross(ab, ap));
  if (vc < R(0) && ab_ap >= R(0) && ab_bp <= R(0)) {
    R v = ab_ap / norm_squared(ab);
    *loc = {LOC_EDGE, 0, {R(1) - v, v, 0}};
    return a + ab * v;
  }
  R vb = -dot(n, cross(ac, cp));
  if (vb < R(0) && ac_ap >= R(0) && ac_cp <= R(0)) {
    R w = ac_ap / norm_squared(ac);
    *loc = {LOC_EDGE, 2, {R(1) - w, w, 0}};
    return a + ac * w;
  }
  R va = dot(n, cross(bc, bp));
  if (va < R(0) && ac_bp - ab_bp >= R(0) && ab_cp - ac_cp >= R(0)) {
    R w = dot(bc, bp) / norm_squared(bc);
    *loc = {LOC_EDGE, 1, {R(1) - w, w, 0}};
    return b + bc * w;
  }
  int side = dot(n, ap) >= R(0) ? 0 : 1;
  if (va + vb + vc != R(0)) {
    R denom = R(1) / (va + vb + vc);
    R v = vb * denom;
    R w = vc * denom;
    *loc = {LOC_FACE, side, {(R(1) - v) - w, v, w}};
    return (a + ab * v) + ac * w;
  }
  *loc = {LOC_SOLID, 0, {0, 0, 0}};
  return pt;
}

// point_tetrahedron.rs:32-340 (solid)
template <class R>
inline bool tetra_check_edge(int i, const Vec3<R>& a, const Vec3<R>& nabc, const Vec3<R>& nabd, const Vec3<R>& ap, const Vec3<R>& ab,
                             R ap_ab, R bp_ab, R* dabc, R* dabd, Vec3<R>* res, Loc<R>* loc) {
  R ab_ab = ap_ab - bp_ab;
  Vec3<R> ap_x_ab = cross(ap, ab);
  *dabc = dot(ap_x_ab, nabc);
  *dabd = dot(ap_x_ab, nabd);
  if (ab_ab != R(0) && *dabc >= R(0) && *dabd >= R(0) && ap_ab >= R(0) && ap_ab <= ab_ab) {
    R u = ap_ab / ab_ab;
    *loc = {LOC_EDGE, i, {R(1) - u, u, 0}};
    *res = a + ab * u;
    return true;
  }
  return false;
}

template <class R>
inline bool tetra_check_face(int i, const Vec3<R>& a, const Vec3<R>& b, const Vec3<R>& c, const Vec3<R>& ap, const Vec3<R>& bp,
                             const Vec3<R>& cp, const Vec3<R>& ab, const Vec3<R>& ac, const Vec3<R>& ad, R dabc, R dbca, R dacb,
                             Vec3<R>* res, Loc<R>* loc) {
  if (dabc < R(0) && dbca < R(0) && dacb < R(0)) {
    Vec3<R> n = cross(ab, ac);
    if (dot(n, ad) * dot(n, ap) < R(0)) {
      // n.try_normalize(DEFAULT_EPSILON): None when |n| <= eps
      R nn = norm(n);
      if (nn <= eps_default<R>()) return false;
      Vec3<R> normal = n / nn;
      R vc = dot(normal, cross(ap, bp));
      R va = dot(normal, cross(bp, cp));
      R vb = dot(normal, cross(cp, ap));
      R denom = va + vb + vc;
      R inv = R(1) / denom;
      R b0 = va * inv, b1 = vb * inv, b2 = vc * inv;
      *loc = {LOC_FACE, i, {b0, b1, b2}};
      *res = (a * b0 + b * b1) + c * b2;
      return true;
    }
  }
  return false;
}

template <class R>
inline Vec3<R> project_tetrahedron(const Vec3<R>& a, const Vec3<R>& b, const Vec3<R>& c, const Vec3<R>& d, const Vec3<R>& pt,
                                   Loc<R>* loc) {
  Vec3<R> ab = b - a, ac = c - a, ad = d - a, ap = pt - a;
  R ap_ab = dot(ap, ab), ap_ac = dot(ap, ac), ap_ad = dot(ap, ad);
  if (ap_ab <= R(0) && ap_ac <= R(0) && ap_ad <= R(0)) { *loc = {LOC_VERTEX, 0, {1, 0, 0}}; return a; }
  Vec3<R> bc = c - b, bd = d - b, bp = pt - b;
  R bp_bc = dot(bp, bc), bp_bd = dot(bp, bd), bp_ab = dot(bp, ab);
  if (bp_bc <= R(0) && bp_bd <= R(0) && bp_ab >= R(0)) { *loc = {LOC_VERTEX, 1, {1, 0, 0}}; return b; }
  Vec3<R> cd = d - c, cp = pt - c;
  R cp_ac = dot(cp, ac), cp_bc = dot(cp, bc), cp_cd = dot(cp, cd);
  if (cp_cd <= R(0) && cp_bc >= R(0) && cp_ac >= R(0)) { *loc = {LOC_VERTEX, 2, {1, 0, 0}}; return c; }
  Vec3<R> dp = pt - d;
  R dp_cd = dot(dp, cd), dp_bd = dot(dp, bd), dp_ad = dot(dp, ad);
  if (dp_ad >= R(0) && dp_bd >= R(0) && dp_cd >= R(0)) { *loc = {LOC_VERTEX, 3, {1, 0, 0}}; return d; }
  Vec3<R> res;
  Vec3<R> nabc = cross(ab, ac);
  Vec3<R> nabd = cross(ab, ad);
  R dabc, dabd, dacd, dacb, dadb, dadc, dbca, dbcd, dbdc, dbda, dcda, dcdb;
  if (tetra_check_edge(0, a, nabc, nabd, ap, ab, ap_ab, bp_ab, &dabc, &dabd, &res, loc)) return res;
  Vec3<R> nacd = cross(ac, ad);
  if (tetra_check_edge(1, a, nacd, -nabc, ap, ac, ap_ac, cp_ac, &dacd, &dacb, &res, loc)) return res;
  if (tetra_check_edge(2, a, -nabd, -nacd, ap, ad, ap_ad, dp_ad, &dadb, &dadc, &res, loc)) return res;
  Vec3<R> nbcd = cross(bc, bd);
  if (tetra_check_edge(3, b, nabc, nbcd, bp, bc, bp_bc, cp_bc, &dbca, &dbcd, &res, loc)) return res;
  if (tetra_check_edge(4, b, -nbcd, nabd, bp, bd, bp_bd, dp_bd, &dbdc, &dbda, &res, loc)) return res;
  if (tetra_check_edge(5, c, nacd, nbcd, cp, cd, cp_cd, dp_cd, &dcda, &dcdb, &res, loc)) return res;
  if (tetra_check_face(0, a, b, c, ap, bp, cp, ab, ac, ad, dabc, dbca, dacb, &res, loc)) return res;
  if (tetra_check_face(1, a, b, d, ap, bp, dp, ab, ad, ac, dadb, dabd, dbda, &res, loc)) return res;
  if (tetra_check_face(2, a, c, d, ap, cp, dp, ac, ad, ab, dacd, dcda, dadc, &res, loc)) return res;
  if (tetra_check_face(3, b, c, d, bp, cp, dp, bc, bd, -ab, dbcd, dcdb, dbdc, &res, loc)) return res;
  *loc = {LOC_SOLID, 0, {0, 0, 0}};
  return pt;
}

}  // namespace oracle
