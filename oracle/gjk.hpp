// Oracle (test infrastructure only): CPU restatement of parry3d's VoronoiSimplex and GJK.
// Follows src/query/gjk/voronoi_simplex3.rs:14-351 and src/query/gjk/gjk.rs:141-144, 196-213,
// 353-453, 797-818 (paths relative to the parry repository).
#pragma once
#include "query.hpp"

namespace oracle {

template <class R> struct VoronoiSimplex {
  int prev_vertices[4] = {0, 1, 2, 3};
  R prev_proj[3] = {0, 0, 0};
  int prev_dim = 0;
  CSOPoint<R> vertices[4];
  R proj[3] = {0, 0, 0};
  int dim = 0;

  void swap(int i1, int i2) {
    std::swap(vertices[i1], vertices[i2]);
    std::swap(prev_vertices[i1], prev_vertices[i2]);
  }
  void reset(const CSOPoint<R>& pt) { dim = 0; prev_dim = 0; vertices[0] = pt; }

  // voronoi_simplex3.rs:57-92
  bool add_point(const CSOPoint<R>& pt) {
    prev_dim = dim;
    for (int i = 0; i < 3; ++i) prev_proj[i] = proj[i];
    for (int i = 0; i < 4; ++i) prev_vertices[i] = i;
    if (dim == 0) {
      if (norm_squared(vertices[0].point - pt.point) < gjk_eps_tol<R>()) return false;
    } else if (dim == 1) {
      Vec3<R> ab = vertices[1].point - vertices[0].point;
      Vec3<R> ac = pt.point - vertices[0].point;
      if (norm_squared(cross(ab, ac)) < gjk_eps_tol<R>()) return false;
    } else if (dim == 2) {
      Vec3<R> ab = vertices[1].point - vertices[0].point;
      Vec3<R> ac = vertices[2].point - vertices[0].point;
      Vec3<R> ap = pt.point - vertices[0].point;
      Vec3<R> n = normalize(cross(ab, ac));
      if (std::fabs(dot(n, ap)) < gjk_eps_tol<R>()) return false;
    }
    dim += 1;
    vertices[dim] = pt;
    return true;
  }

  // voronoi_simplex3.rs:123-279
  Vec3<R> project_origin_and_reduce() {
    const Vec3<R> o;
    if (dim == 0) {
      proj[0] = R(1);
      return vertices[0].point;
    } else if (dim == 1) {
      Loc<R> loc;
      Vec3<R> p = project_segment(vertices[0].point, vertices[1].point, o, &loc);
      if (loc.kind == LOC_VERTEX && loc.id == 0) { proj[0] = R(1); dim = 0; }
      else if (loc.kind == LOC_VERTEX) { swap(0, 1); proj[0] = R(1); dim = 0; }
      else { proj[0] = loc.bc[0]; proj[1] = loc.bc[1]; }
      return p;
    } else if (dim == 2) {
      Loc<R> loc;
      Vec3<R> p = project_triangle(vertices[0].point, vertices[1].point, vertices[2].point, o, &loc);
      switch (loc.kind) {
        case LOC_VERTEX: swap(0, loc.id); proj[0] = R(1); dim = 0; break;
        case LOC_EDGE:
          if (loc.id == 0) { proj[0] = loc.bc[0]; proj[1] = loc.bc[1]; dim = 1; }
          else if (loc.id == 1) { swap(0, 2); proj[0] = loc.bc[1]; proj[1] = loc.bc[0]; dim = 1; }
          else { swap(1, 2); proj[0] = loc.bc[0]; proj[1] = loc.bc[1]; dim = 1; }
          break;
        case LOC_FACE: proj[0] = loc.bc[0]; proj[1] = loc.bc[1]; proj[2] = loc.bc[2]; break;
        default: break;
      }
      return p;
    } else {
      Loc<R> loc;
      Vec3<R> p = project_tetrahedron(vertices[0].point, vertices[1].point, vertices[2].point, vertices[3].point, o, &loc);
      switch (loc.kind) {
        case LOC_VERTEX: swap(0, loc.id); proj[0] = R(1); dim = 0; break;
        case LOC_EDGE: {
          int i = loc.id;
          if (i == 1) swap(1, 2);
          else if (i == 2) swap(1, 3);
          else if (i == 3) swap(0, 2);
          else if (i == 4) swap(0, 3);
          else if (i == 5) { swap(0, 2); swap(1, 3); }
          if (i == 3 || i == 4) { proj[0] = loc.bc[1]; proj[1] = loc.bc[0]; }
          else { proj[0] = loc.bc[0]; proj[1] = loc.bc[1]; }
          dim = 1;
          break;
        }
        case LOC_FACE: {
          int i = loc.id;
          if (i == 0) { proj[0] = loc.bc[0]; proj[1] = loc.bc[1]; proj[2] = loc.bc[2]; }
          else if (i == 1) { vertices[2] = vertices[3]; proj[0] = loc.bc[0]; proj[1] = loc.bc[1]; proj[2] = loc.bc[2]; }
          else if (i == 2) { vertices[1] = vertices[3]; proj[0] = loc.bc[0]; proj[1] = loc.bc[2]; proj[2] = loc.bc[1]; }
          else { vertices[0] = vertices[3]; proj[0] = loc.bc[2]; proj[1] = loc.bc[0]; proj[2] = loc.bc[1]; }
          dim = 2;
          break;
        }
        default: break;
      }
      return p;
    }
  }

  const CSOPoint<R>& prev_point(int i) const { return vertices[prev_vertices[i]]; }
};

enum GjkKind { GJK_INTERSECTION, GJK_CLOSEST_POINTS, GJK_PROXIMITY, GJK_NO_INTERSECTION };
template <class R> struct GjkResult {
  GjkKind kind;
  Vec3<R> p1, p2, dir;
};

// gjk.rs:797-818
template <class R> inline void gjk_result(const VoronoiSimplex<R>& s, bool prev, Vec3<R>* p1, Vec3<R>* p2) {
  Vec3<R> a, b;
  if (prev) {
    for (int i = 0; i < s.prev_dim + 1; ++i) {
      R c = s.prev_proj[i];
      const CSOPoint<R>& p = s.prev_point(i);
      a += p.orig1 * c;
      b += p.orig2 * c;
    }
  } else {
    for (int i = 0; i < s.dim + 1; ++i) {
      R c = s.proj[i];
      a += s.vertices[i].orig1 * c;
      b += s.vertices[i].orig2 * c;
    }
  }
  *p1 = a;
  *p2 = b;
}

struct GjkStats {
  uint64_t gjk_iters = 0;  // support evaluations in the GJK loop
  uint64_t epa_iters = 0;  // support evaluations in the EPA loop
  uint64_t epa_calls = 0;
  uint64_t epa_max_faces = 0;   // largest polytope face array in one EPA call
  uint64_t epa_max_verts = 0;
  uint64_t epa_max_sil = 0;     // largest silhouette
};

// gjk.rs:353-453 with exact_dist = true.
template <class R>
inline GjkResult<R> gjk_closest_points(const Iso<R>& pos12, const Support<R>& g1, const Support<R>& g2, R max_dist,
                                       VoronoiSimplex<R>& simplex, GjkStats* st = nullptr) {
  const R eps_tol = gjk_eps_tol<R>();
  const R eps_rel = std::sqrt(eps_tol);
  Vec3<R> proj = simplex.project_origin_and_reduce();
  Vec3<R> old_dir;
  {
    Vec3<R> u;
    if (try_normalize(proj, R(0), &u)) old_dir = -u;
    else return {GJK_INTERSECTION, {}, {}, {}};
  }
  R max_bound = std::numeric_limits<R>::max();
  Vec3<R> dir;
  int niter = 0;
  for (;;) {
    R old_max_bound = max_bound;
    {
      Vec3<R> u;
      R n;
      if (try_normalize(-proj, eps_tol, &u, &n)) { dir = u; max_bound = n; }
      else return {GJK_INTERSECTION, {}, {}, {}};
    }
    if (max_bound >= old_max_bound) {
      GjkResult<R> r{GJK_CLOSEST_POINTS, {}, {}, old_dir};
      gjk_result(simplex, true, &r.p1, &r.p2);
      return r;
    }
    if (st) st->gjk_iters++;
    CSOPoint<R> cso = cso_from_shapes(pos12, g1, g2, dir);
    R min_bound = -dot(dir, cso.point);
    if (min_bound > max_dist) return {GJK_NO_INTERSECTION, {}, {}, dir};
    if (max_bound - min_bound <= eps_rel * max_bound) {
      GjkResult<R> r{GJK_CLOSEST_POINTS, {}, {}, dir};
      gjk_result(simplex, false, &r.p1, &r.p2);
      return r;
    }
    if (!simplex.add_point(cso)) {
      GjkResult<R> r{GJK_CLOSEST_POINTS, {}, {}, dir};
      gjk_result(simplex, false, &r.p1, &r.p2);
      return r;
    }
    old_dir = dir;
    proj = simplex.project_origin_and_reduce();
    if (simplex.dim == 3) {
      if (min_bound >= eps_tol) {
        GjkResult<R> r{GJK_CLOSEST_POINTS, {}, {}, old_dir};
        gjk_result(simplex, true, &r.p1, &r.p2);
        return r;
      }
      return {GJK_INTERSECTION, {}, {}, {}};
    }
    niter += 1;
    if (niter == 100) return {GJK_NO_INTERSECTION, {}, {}, Vec3<R>(1, 0, 0)};
  }
}

}  // namespace oracle
