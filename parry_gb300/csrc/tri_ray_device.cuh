// Ray against one triangle, shared by the TriMesh ray casts and the manifold generators
// (src/query/ray/ray_triangle.rs:70-152, path relative to the parry repository): toi and face id
// (0 = front, 1 = back), no normal.
#pragma once
#include "common.cuh"

namespace pg {

struct TriHit {
  float toi;
  uint32_t fid;
};

// local_ray_intersection_with_triangle without the normal (the ray casts recompute it for the winner).
__device__ __forceinline__ bool ray_triangle_toi(V3 a, V3 b, V3 c, V3 o, V3 dir, TriHit* h) {
  V3 ab = b - a;
  V3 ac = c - a;
  V3 n = cross(ab, ac);
  float d = dot(n, dir);
  if (d == 0.0f) return false;
  V3 ap = o - a;
  float t = dot(ap, n);
  if ((t < 0.0f && d < 0.0f) || (t > 0.0f && d > 0.0f)) return false;
  uint32_t fid = d < 0.0f ? 0u : 1u;
  d = fabsf(d);
  V3 e = -cross(dir, ap);
  float v, w;
  if (t < 0.0f) {
    v = -dot(ac, e);
    if (v < 0.0f || v > d) return false;
    w = dot(ab, e);
    if (w < 0.0f || v + w > d) return false;
    float invd = 1.0f / d;
    h->toi = -t * invd;
  } else {
    v = dot(ac, e);
    if (v < 0.0f || v > d) return false;
    w = -dot(ab, e);
    if (w < 0.0f || v + w > d) return false;
    float invd = 1.0f / d;
    h->toi = t * invd;
  }
  h->fid = fid;
  return true;
}

}  // namespace pg
