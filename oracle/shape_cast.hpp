// Oracle (test infrastructure only): CPU restatement of parry3d's linear shape casting (time of
// impact under translational motion) for ball and support-map pairs. Paths relative to the parry
// repository:
//   src/query/shape_cast/shape_cast.rs:8-79, 230-286     ShapeCastStatus, ShapeCastHit, ShapeCastOptions, cast_shapes
//   src/query/default_query_dispatcher.rs:434-538        DefaultQueryDispatcher::cast_shapes (ball-ball, support maps)
//   src/query/shape_cast/shape_cast_ball_ball.rs:10-69   cast_shapes_ball_ball
//   src/query/shape_cast/shape_cast_support_map_support_map.rs:12-69
//   src/query/gjk/gjk.rs:632-657                         directional_distance
//   src/shape/round_shape.rs:330-349                     RoundShapeRef support (target_distance > 0)
#pragma once
#include "shape_ray.hpp"

namespace oracle {

enum ShapeCastStatus : uint32_t { CAST_OUT_OF_ITERATIONS = 0, CAST_CONVERGED = 1, CAST_FAILED = 2, CAST_PENETRATING = 3 };

template <class R> struct ShapeCastOptions {
  R max_time_of_impact = std::numeric_limits<R>::max();
  R target_distance = R(0);
  bool stop_at_penetration = true;
  bool compute_impact_geometry_on_penetration = true;
};

template <class R> struct ShapeCastHit {
  R toi;
  Vec3<R> witness1, witness2, normal1, normal2;
  uint32_t status;
};

// gjk.rs:632-657 directional_distance: (toi, normal, witness1, witness2) or None.
template <class R>
inline bool directional_distance(const Iso<R>& pos12, const Support<R>& g1, const Support<R>& g2, const Vec3<R>& dir, R* toi, Vec3<R>* n,
                                 Vec3<R>* w1, Vec3<R>* w2) {
  VoronoiSimplex<R> simplex;
  Ray<R> ray{Vec3<R>(), dir};
  if (!minkowski_ray_cast(pos12, g1, g2, ray, std::numeric_limits<R>::max(), simplex, toi, n)) return false;
  if (*toi != R(0)) {
    gjk_result(simplex, simplex.dim == 3, w1, w2);
  } else {
    *w1 = Vec3<R>();  // penetration: witnesses undefined (origin)
    *w2 = Vec3<R>();
  }
  return true;
}

// shape_cast_support_map_support_map.rs:12-69
template <class R>
inline bool cast_shapes_support_map_support_map(const Iso<R>& pos12, const Vec3<R>& vel12, const Shape<R>& s1, const Shape<R>& s2,
                                                const ShapeCastOptions<R>& opt, ShapeCastHit<R>* hit, GjkStats* st) {
  Support<R> g1{&s1}, g2{&s2};
  if (opt.target_distance > R(0)) { g1.round = true; g1.border = opt.target_distance; }
  R toi;
  Vec3<R> normal1, w1, w2;
  if (!directional_distance(pos12, g1, g2, vel12, &toi, &normal1, &w1, &w2)) return false;
  if (toi > opt.max_time_of_impact) return false;
  if ((opt.compute_impact_geometry_on_penetration || !opt.stop_at_penetration) && toi < R(1.0e-5)) {
    Contact<R> c;
    if (!contact_support_map_support_map(pos12, s1, s2, std::numeric_limits<R>::max(), (const Vec3<R>*)nullptr, &c, st)) return false;
    R normal_vel = dot(c.normal1, vel12);
    if (!opt.stop_at_penetration && normal_vel >= R(0)) return false;
    *hit = ShapeCastHit<R>{toi, c.point1, c.point2, c.normal1, c.normal2, CAST_PENETRATING};
    return true;
  }
  hit->toi = toi;
  hit->normal1 = normal1;
  hit->normal2 = pos12.inverse_transform_vector(-normal1);
  hit->witness1 = w1 - normal1 * opt.target_distance;
  hit->witness2 = pos12.inverse_transform_point(w2);
  hit->status = toi == R(0) ? CAST_PENETRATING : CAST_CONVERGED;
  return true;
}

// shape_cast_ball_ball.rs:10-69
template <class R>
inline bool cast_shapes_ball_ball(const Iso<R>& pos12, const Vec3<R>& vel12, R r1, R r2, const ShapeCastOptions<R>& opt, ShapeCastHit<R>* hit) {
  R rsum = (r1 + r2) + opt.target_distance;
  R radius = rsum;
  Vec3<R> center = -pos12.tra;
  Ray<R> ray{pos12.tra, vel12};  // origin - center with the ray starting at the origin
  bool inside;
  R toi;
  if (!ray_toi_with_ball(radius, ray, true, &inside, &toi)) return false;
  if (toi > opt.max_time_of_impact) return false;
  Vec3<R> dpt = vel12 * toi - center;  // ray.point_at(toi) - center
  Vec3<R> n1, n2, w1, w2;
  if (radius == R(0)) {
    n1 = Vec3<R>(1, 0, 0);
    n2 = pos12.inverse_transform_vector(Vec3<R>(-1, 0, 0));
  } else {
    n1 = dpt / radius;
    n2 = pos12.inverse_transform_vector(-n1);
    w1 = n1 * r1;
    w2 = n2 * r2;
  }
  if (!opt.stop_at_penetration && toi < R(1.0e-5) && dot(n1, vel12) >= R(0)) return false;
  uint32_t status = (inside && norm_squared(center) < rsum * rsum) ? CAST_PENETRATING : CAST_CONVERGED;
  *hit = ShapeCastHit<R>{toi, w1, w2, n1, n2, status};
  return true;
}

// query::cast_shapes(pos1, vel1, g1, pos2, vel2, g2, options) (shape_cast.rs:275-286) through the
// DefaultQueryDispatcher for ball and support-map shapes.
template <class R>
inline bool cast_shapes(const Iso<R>& pos1, const Vec3<R>& vel1, const Shape<R>& g1, const Iso<R>& pos2, const Vec3<R>& vel2,
                        const Shape<R>& g2, const ShapeCastOptions<R>& opt, ShapeCastHit<R>* hit, GjkStats* st) {
  Iso<R> pos12 = pos1.inv_mul(pos2);
  Vec3<R> vel12 = pos1.inverse_transform_vector(vel2 - vel1);
  if (g1.is_ball() && g2.is_ball()) return cast_shapes_ball_ball(pos12, vel12, g1.radius, g2.radius, opt, hit);
  return cast_shapes_support_map_support_map(pos12, vel12, g1, g2, opt, hit, st);
}

}  // namespace oracle
