// Oracle (test infrastructure only): CPU restatement of parry3d's ray casts against convex shapes
// and against a Compound (shape set). Paths relative to the parry repository:
//   src/query/ray/ray_ball.rs:33-98          ray_toi_with_ball / ray_toi_and_normal_with_ball
//   src/query/ray/ray_cuboid.rs:6-25, ray_aabb.rs:51-92, src/query/clip/clip_aabb_line.rs:79-185
//   src/query/ray/ray_support_map.rs:19-71   support-map ray cast (capsule, convex polyhedron)
//   src/query/gjk/gjk.rs:519-534, 660-795    gjk::cast_local_ray / minkowski_ray_cast
//   src/query/ray/ray_halfspace.rs           ray_toi_with_halfspace
//   src/query/ray/ray_triangle.rs:49-62      Triangle::cast_local_ray_and_get_normal
//   src/query/ray/ray_composite_shape.rs:86-105, src/shape/compound.rs:113-144  Compound
#pragma once
#include "contact.hpp"
#include "ray.hpp"
#include <memory>

namespace oracle {

// ray_ball.rs:33-77; returns (inside, toi)
template <class R> inline bool ray_toi_with_ball(R radius, const Ray<R>& ray, bool solid, bool* inside, R* toi) {
  Vec3<R> dcenter = ray.origin;  // origin - center(0)
  R a = norm_squared(ray.dir);
  R b = dot(dcenter, ray.dir);
  R c = norm_squared(dcenter) - radius * radius;
  if (a == R(0)) {
    if (c > R(0)) { *inside = false; return false; }
    *inside = true; *toi = R(0); return true;
  }
  if (c > R(0) && b > R(0)) { *inside = false; return false; }
  R delta = b * b - a * c;
  if (delta < R(0)) { *inside = false; return false; }
  R t = (-b - std::sqrt(delta)) / a;
  if (t <= R(0)) {
    *inside = true;
    *toi = solid ? R(0) : (-b + std::sqrt(delta)) / a;
    return true;
  }
  *inside = false;
  *toi = t;
  return true;
}

// clip_aabb_line.rs:79-185 -> near / far (t, normal); returns false for None.
template <class R>
inline bool clip_aabb_line(const Aabb<R>& aabb, const Vec3<R>& origin, const Vec3<R>& dir, R* tn, Vec3<R>* nn, R* tf, Vec3<R>* nf) {
  R tmax = std::numeric_limits<R>::max();
  R tmin = -tmax;
  int near_side = 0, far_side = 0;
  bool near_diag = false, far_diag = false;
  for (int i = 0; i < 3; ++i) {
    if (dir[i] == R(0)) {
      if (origin[i] < aabb.mins[i] || origin[i] > aabb.maxs[i]) return false;
    } else {
      R denom = R(1) / dir[i];
      bool flip;
      R n = (aabb.mins[i] - origin[i]) * denom;
      R f = (aabb.maxs[i] - origin[i]) * denom;
      if (n > f) { flip = true; std::swap(n, f); } else flip = false;
      if (n > tmin) { tmin = n; near_side = flip ? -(i + 1) : (i + 1); near_diag = false; }
      else if (n == tmin) near_diag = true;
      if (f < tmax) { tmax = f; far_side = !flip ? -(i + 1) : (i + 1); far_diag = false; }
      else if (f == tmax) far_diag = true;
      if (tmax < R(0) || tmin > tmax) return false;
    }
  }
  auto contains = [&]() {
    for (int i = 0; i < 3; ++i) if (origin[i] < aabb.mins[i] || origin[i] > aabb.maxs[i]) return false;
    return true;
  };
  if (near_diag) { *tn = tmin; *nn = -normalize(dir); }
  else {
    if (near_side == 0) {
      if (!contains()) return false;
      *tn = R(0); *nn = Vec3<R>(); *tf = R(0); *nf = Vec3<R>();
      return true;
    }
    Vec3<R> n;
    if (near_side < 0) n[-near_side - 1] = R(1); else n[near_side - 1] = R(-1);
    *tn = tmin; *nn = n;
  }
  if (far_diag) { *tf = tmax; *nf = -normalize(dir); }
  else {
    if (far_side == 0) {
      if (!contains()) return false;
      *tn = R(0); *nn = Vec3<R>(); *tf = R(0); *nf = Vec3<R>();
      return true;
    }
    Vec3<R> n;
    if (far_side < 0) n[-far_side - 1] = R(-1); else n[far_side - 1] = R(1);
    *tf = tmax; *nf = n;
  }
  return true;
}

// ray_aabb.rs:51-92 (cast_local_ray_and_get_normal of an Aabb)
template <class R> inline bool ray_aabb(const Aabb<R>& aabb, const Ray<R>& ray, R max_toi, bool solid, R* toi, Vec3<R>* normal) {
  R tn, tf;
  Vec3<R> nn, nf;
  if (!clip_aabb_line(aabb, ray.origin, ray.dir, &tn, &nn, &tf, &nf)) return false;
  if (tn < R(0)) {
    if (solid) { *toi = R(0); *normal = Vec3<R>(); return true; }
    if (tf <= max_toi) { *toi = tf; *normal = nf; return true; }
    return false;
  }
  if (tn <= max_toi) { *toi = tn; *normal = nn; return true; }
  return false;
}

// ray_halfspace.rs: ray_toi_with_halfspace
template <class R> inline bool ray_toi_with_halfspace(const Vec3<R>& center, const Vec3<R>& normal, const Ray<R>& ray, R* t) {
  Vec3<R> dpos = center - ray.origin;
  R denom = dot(normal, ray.dir);
  if (std::fabs(denom) <= eps_default<R>()) return false;  // relative_eq!(denom, 0.0)
  R tt = dot(normal, dpos) / denom;
  if (tt >= R(0)) { *t = tt; return true; }
  return false;
}

// gjk.rs:660-795 minkowski_ray_cast: ray cast on the Minkowski difference g1 - pos12 * g2. On a hit
// returns the toi (in units of the ray direction's length) and the normal; `simplex` is left as
// the reference leaves it (directional_distance reads its witness points).
template <class R>
inline bool minkowski_ray_cast(const Iso<R>& pos12, const Support<R>& g1, const Support<R>& g2, const Ray<R>& ray, R max_toi,
                               VoronoiSimplex<R>& simplex, R* toi_out, Vec3<R>* n_out) {
  const R eps_tol = gjk_eps_tol<R>();
  const R eps_rel = std::sqrt(eps_tol);
  R ray_length = norm(ray.dir);
  if (std::fabs(ray_length) <= eps_default<R>()) return false;  // relative_eq!(ray_length, 0.0)
  R ltoi = R(0);
  Ray<R> curr{ray.origin, ray.dir / ray_length};
  Vec3<R> dir = -curr.dir;
  Vec3<R> ldir = dir;
  CSOPoint<R> sp = cso_from_shapes(pos12, g1, g2, dir);
  simplex.reset(sp.translate(-curr.origin));
  Vec3<R> proj = simplex.project_origin_and_reduce();
  R max_bound = std::numeric_limits<R>::max();
  int niter = 0;
  bool last_chance = false;
  for (;;) {
    R old_max_bound = max_bound;
    R nb;
    Vec3<R> u;
    if (try_normalize(-proj, eps_tol, &u, &nb)) { dir = u; max_bound = nb; }
    else { *toi_out = ltoi / ray_length; *n_out = ldir; return true; }
    CSOPoint<R> support_point;
    if (max_bound >= old_max_bound) {
      last_chance = true;
      support_point = CSOPoint<R>::single_point(proj + curr.origin);
    } else {
      support_point = cso_from_shapes(pos12, g1, g2, dir);
    }
    if (last_chance && ltoi > R(0)) { *toi_out = ltoi / ray_length; *n_out = ldir; return true; }
    R t;
    if (ray_toi_with_halfspace(support_point.point, dir, curr, &t)) {
      if (dot(dir, curr.dir) < R(0) && t > R(0)) {
        ldir = dir;
        ltoi += t;
        if (ltoi / ray_length > max_toi) return false;
        Vec3<R> shift = curr.dir * t;
        curr.origin += shift;
        max_bound = std::numeric_limits<R>::max();
        for (int i = 0; i <= simplex.dim; ++i) simplex.vertices[i].point += -shift;
        last_chance = false;
      }
    } else {
      if (dot(dir, curr.dir) > eps_tol) return false;
    }
    if (last_chance) return false;
    R min_bound = -dot(dir, support_point.point - curr.origin);
    if (max_bound - min_bound <= eps_rel * max_bound) return false;
    simplex.add_point(support_point.translate(-curr.origin));
    proj = simplex.project_origin_and_reduce();
    if (simplex.dim == 3) {
      if (min_bound >= eps_tol) return false;
      *toi_out = ltoi / ray_length; *n_out = ldir; return true;
    }
    niter += 1;
    if (niter == 100) return false;
  }
}

// gjk.rs:519-534 cast_local_ray: minkowski_ray_cast with pos12 = identity and g2 = ConstantOrigin.
template <class R>
inline bool gjk_cast_local_ray(const Shape<R>& shape, VoronoiSimplex<R>& simplex, const Ray<R>& ray, R max_toi, R* toi_out, Vec3<R>* n_out) {
  Iso<R> id;
  Support<R> g1{&shape}, g2{nullptr};
  return minkowski_ray_cast(id, g1, g2, ray, max_toi, simplex, toi_out, n_out);
}

// ray_support_map.rs:19-71
template <class R>
inline bool ray_support_map(const Shape<R>& shape, const Ray<R>& ray, R max_toi, bool solid, R* toi, Vec3<R>* normal) {
  VoronoiSimplex<R> simplex;
  R t;
  Vec3<R> n;
  if (!gjk_cast_local_ray(shape, simplex, ray, max_toi, &t, &n)) return false;
  if (solid || t != R(0)) { *toi = t; *normal = n; return true; }
  // the ray starts inside a hollow shape: cast back from beyond the exit point
  Vec3<R> ndir = normalize(ray.dir);
  Vec3<R> supp = shape.local_support(ndir);
  R eps = R(0.001);
  R shift = dot(supp - ray.origin, ndir) + eps;
  Ray<R> nr{ray.origin + ndir * shift, -ray.dir};
  VoronoiSimplex<R> s2;
  R t2;
  Vec3<R> n2;
  if (!gjk_cast_local_ray(shape, s2, nr, shift + eps, &t2, &n2)) return false;
  R tt = shift - t2;
  if (!(tt <= max_toi)) return false;
  *toi = tt;
  *normal = -n2;
  return true;
}

// RayCast::cast_local_ray_and_get_normal for one convex shape.
template <class R>
inline bool shape_cast_local_ray(const Shape<R>& s, const Ray<R>& ray, R max_toi, bool solid, R* toi, Vec3<R>* normal) {
  switch (s.type) {
    case SHAPE_BALL: {
      bool inside;
      R t;
      if (!ray_toi_with_ball(s.radius, ray, solid, &inside, &t)) return false;
      Vec3<R> pos = ray.origin + ray.dir * t;  // - center (origin)
      Vec3<R> nn = normalize(pos);
      if (!(t <= max_toi)) return false;
      *toi = t;
      *normal = inside ? -nn : nn;
      return true;
    }
    case SHAPE_CUBOID: return ray_aabb(Aabb<R>(-s.half, s.half), ray, max_toi, solid, toi, normal);
    case SHAPE_TRIANGLE: {
      RayHit<R> h;
      if (!ray_triangle(s.pts[0], s.pts[1], s.pts[2], ray, &h)) return false;
      if (!(h.toi <= max_toi)) return false;
      *toi = h.toi;
      *normal = h.normal;
      return true;
    }
    default: return ray_support_map(s, ray, max_toi, solid, toi, normal);
  }
}

// RayCast::cast_ray_and_get_normal(pose, ray, max_toi, solid) for one shape.
template <class R>
inline bool shape_cast_ray(const Shape<R>& s, const Iso<R>& pose, const Ray<R>& wray, R max_toi, bool solid, R* toi, Vec3<R>* normal) {
  Ray<R> lr{pose.inverse_transform_point(wray.origin), pose.inverse_transform_vector(wray.dir)};
  Vec3<R> n;
  if (!shape_cast_local_ray(s, lr, max_toi, solid, toi, &n)) return false;
  *normal = pose.transform_vector(n);
  return true;
}

// Compound: binned BVH over the parts' world AABBs; find_best with the part ray cast.
template <class R> struct Compound {
  std::vector<Shape<R>> shapes;
  std::vector<Iso<R>> poses;
  std::vector<Vec3<R>> pool;  // convex / triangle vertices the shapes point into
  Bvh<R> bvh;
  void build() {
    std::vector<Aabb<R>> leaves(shapes.size());
    for (size_t i = 0; i < shapes.size(); ++i) leaves[i] = shape_aabb(shapes[i], poses[i]);
    bvh = Bvh<R>::from_leaves(leaves);
  }
  bool cast_local_ray_and_get_normal(const Ray<R>& ray, R max_toi, bool solid, bool lowest_index, uint32_t* part, R* toi,
                                     Vec3<R>* normal, VisitStats* st = nullptr) const {
    auto aabb_cost = [&](const BvhNode<R>& n, R best) { return n.cast_ray(ray, best); };
    auto leaf_cost = [&](uint32_t i, R best, R* cost) {
      R t;
      Vec3<R> n;
      if (!shape_cast_ray(shapes[i], poses[i], ray, best, solid, &t, &n)) return false;
      *cost = t;
      return true;
    };
    uint32_t best;
    bool ok = lowest_index ? bvh.find_best_lowest_index(max_toi, aabb_cost, leaf_cost, &best, st)
                           : bvh.find_best(max_toi, aabb_cost, leaf_cost, &best, st);
    if (!ok) return false;
    // re-evaluate the winner with the bound in force when it was accepted: its own toi
    R t;
    Vec3<R> n;
    shape_cast_ray(shapes[best], poses[best], ray, max_toi, solid, &t, &n);
    *part = best;
    *toi = t;
    *normal = n;
    return true;
  }
};

}  // namespace oracle
