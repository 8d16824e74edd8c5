// Oracle (test infrastructure only): CPU restatement of parry3d's ray casts against triangle
// meshes. Used by tests/, the smoke check and the bench's CPU-baseline leg as the checker.
//
// Follows (paths relative to the parry repository):
//   src/query/ray/ray_triangle.rs:49-62   Triangle::cast_local_ray_and_get_normal (toi <= max_toi)
//   src/query/ray/ray_triangle.rs:70-152  local_ray_intersection_with_triangle
//   src/query/ray/ray_trimesh.rs:17-35    TriMesh::cast_local_ray_and_get_normal (back face -> Face(i + n))
//   src/query/ray/ray_composite_shape.rs:19-62  CompositeShapeRef cast_local_ray(_and_get_normal)
//   src/query/ray/ray.rs:381-403          RayCast::cast_ray(_and_get_normal) world transform
//   src/shape/trimesh.rs:1159-1171        TriMesh BVH = Binned build over triangle local AABBs
//   src/bounding_volume/aabb_triangle.rs:16-30  Triangle::local_aabb
#pragma once
#include "bvh.hpp"

namespace oracle {

template <class R> struct RayHit {
  R toi;
  Vec3<R> normal;
  uint32_t fid;  // 0 = front face, 1 = back face
};

// ray_triangle.rs:70-152
template <class R>
inline bool ray_triangle(const Vec3<R>& a, const Vec3<R>& b, const Vec3<R>& c, const Ray<R>& ray, RayHit<R>* out) {
  Vec3<R> ab = b - a;
  Vec3<R> ac = c - a;
  Vec3<R> n = cross(ab, ac);
  R d = dot(n, ray.dir);
  if (d == R(0)) return false;
  Vec3<R> ap = ray.origin - a;
  R t = dot(ap, n);
  if ((t < R(0) && d < R(0)) || (t > R(0) && d > R(0))) return false;
  uint32_t fid = d < R(0) ? 0u : 1u;
  d = std::fabs(d);
  Vec3<R> e = -cross(ray.dir, ap);
  R v, w, toi;
  Vec3<R> normal;
  if (t < R(0)) {
    v = -dot(ac, e);
    if (v < R(0) || v > d) return false;
    w = dot(ab, e);
    if (w < R(0) || v + w > d) return false;
    R invd = R(1) / d;
    toi = -t * invd;
    normal = -normalize(n);
  } else {
    v = dot(ac, e);
    if (v < R(0) || v > d) return false;
    w = -dot(ab, e);
    if (w < R(0) || v + w > d) return false;
    R invd = R(1) / d;
    toi = t * invd;
    normal = normalize(n);
  }
  out->toi = toi;
  out->normal = normal;
  out->fid = fid;
  return true;
}

template <class R> struct TriMesh {
  std::vector<Vec3<R>> vertices;
  std::vector<uint32_t> indices;  // 3 per triangle
  Bvh<R> bvh;

  uint32_t num_triangles() const { return (uint32_t)(indices.size() / 3); }
  void triangle(uint32_t i, Vec3<R>* a, Vec3<R>* b, Vec3<R>* c) const {
    *a = vertices[indices[3 * i]]; *b = vertices[indices[3 * i + 1]]; *c = vertices[indices[3 * i + 2]];
  }
  static Aabb<R> tri_aabb(const Vec3<R>& a, const Vec3<R>& b, const Vec3<R>& c) {
    Aabb<R> r;
    for (int d = 0; d < 3; ++d) {
      r.mins[d] = rmin(rmin(a[d], b[d]), c[d]);
      r.maxs[d] = rmax(rmax(a[d], b[d]), c[d]);
    }
    return r;
  }
  void build() {
    std::vector<Aabb<R>> leaves(num_triangles());
    for (uint32_t i = 0; i < num_triangles(); ++i) {
      Vec3<R> a, b, c;
      triangle(i, &a, &b, &c);
      leaves[i] = tri_aabb(a, b, c);
    }
    bvh = Bvh<R>::from_leaves(leaves);
  }

  // TriMesh::cast_local_ray_and_get_normal. feature = tri (front) or tri + n_tris (back face).
  // `lowest_index` selects the lowest-triangle-index rule on exact toi ties instead of parry's
  // first-found rule.
  bool cast_local_ray_and_get_normal(const Ray<R>& ray, R max_toi, bool lowest_index, RayHit<R>* out,
                                     uint32_t* feature, VisitStats* st = nullptr) const {
    auto aabb_cost = [&](const BvhNode<R>& n, R best) { return n.cast_ray(ray, best); };
    RayHit<R> tmp;
    auto leaf_cost = [&](uint32_t tri, R best, R* cost) {
      Vec3<R> a, b, c;
      triangle(tri, &a, &b, &c);
      RayHit<R> h;
      if (!ray_triangle(a, b, c, ray, &h)) return false;
      if (!(h.toi <= best)) return false;
      *cost = h.toi;
      return true;
    };
    uint32_t best;
    bool ok = lowest_index ? bvh.find_best_lowest_index(max_toi, aabb_cost, leaf_cost, &best, st)
                           : bvh.find_best(max_toi, aabb_cost, leaf_cost, &best, st);
    if (!ok) return false;
    Vec3<R> a, b, c;
    triangle(best, &a, &b, &c);
    ray_triangle(a, b, c, ray, &tmp);
    *out = tmp;
    *feature = tmp.fid == 1 ? best + num_triangles() : best;
    return true;
  }

  // RayCast::cast_ray_and_get_normal(m, ray, max_toi, solid): local cast then normal rotated back.
  bool cast_ray_and_get_normal(const Iso<R>& m, const Ray<R>& wray, R max_toi, bool lowest_index, RayHit<R>* out,
                               uint32_t* feature, VisitStats* st = nullptr) const {
    Ray<R> lr;
    lr.origin = m.inverse_transform_point(wray.origin);
    lr.dir = m.inverse_transform_vector(wray.dir);
    if (!cast_local_ray_and_get_normal(lr, max_toi, lowest_index, out, feature, st)) return false;
    out->normal = m.transform_vector(out->normal);
    return true;
  }
};

}  // namespace oracle
