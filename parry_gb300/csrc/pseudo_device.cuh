// Normal constraints of TriMesh triangles (TriMeshFlags::FIX_INTERNAL_EDGES) on the device. Paths
// relative to the parry repository:
//   src/shape/triangle_pseudo_normals.rs:20-99                TrianglePseudoNormals::project_local_normal_mut
//   src/query/contact_manifolds/normals_constraint.rs:41-125   project_local_normal1 / 2 and the pair rule
// Same evaluation order as the reference (the library is compiled without FMA contraction).
#pragma once
#include "common.cuh"

namespace pg {

// One triangle's pseudo-normals: the face normal and the (unit) pseudo-normals of edges 01, 12, 20.
struct TriPN {
  V3 face;
  V3 e[3];
};

__device__ __forceinline__ bool v3_eq(V3 a, V3 b) { return a.x == b.x && a.y == b.y && a.z == b.z; }

// Vector::try_normalize(min_norm): None when |v| <= min_norm (norm form).
__device__ __forceinline__ bool try_normalize_norm(V3 v, float min_norm, V3* out) {
  float n = norm(v);
  if (n <= min_norm) return false;
  *out = v / n;
  return true;
}

// TrianglePseudoNormals::project_local_normal_mut: projects *dir into the polygonal normal cone
// (closest edge pseudo-normal by dot product, first on ties); false = the contact is discarded.
__device__ __forceinline__ bool project_local_normal_mut(const TriPN& pn, V3* dir) {
  const float dot_face = dot(*dir, pn.face);
  const float d0 = dot(*dir, pn.e[0]), d1 = dot(*dir, pn.e[1]), d2 = dot(*dir, pn.e[2]);
  int ci = 0;
  float m = d0;
  if (d1 > m) { m = d1; ci = 1; }
  if (d2 > m) ci = 2;
  const V3 closest = pn.e[ci];
  if (v3_eq(closest, pn.face)) {
    *dir = pn.face;
    return dot_face >= 0.0f;
  }
  const float dot_edge_face = dot(pn.face, closest);
  const float dot_dir_face = dot(pn.face, *dir);
  const float dot_corrected_dir_face = 2.0f * dot_edge_face * dot_edge_face - 1.0f;
  if (dot_dir_face >= dot_corrected_dir_face) return true;
  const V3 edge_on_normal = pn.face * dot_edge_face;
  const V3 edge_orthogonal = closest - edge_on_normal;
  const V3 dir_on_normal = pn.face * dot_dir_face;
  const V3 dir_orthogonal = *dir - dir_on_normal;
  V3 unit_dir_orthogonal, adjusted;
  if (!try_normalize_norm(dir_orthogonal, 1.0e-6f, &unit_dir_orthogonal)) return dot_face >= 0.0f;
  if (!try_normalize_norm(edge_on_normal + unit_dir_orthogonal * norm(edge_orthogonal), 1.0e-6f, &adjusted)) return dot_face >= 0.0f;
  *dir = adjusted * (2.0f * dot(pn.face, adjusted)) - pn.face;
  return dot_face >= 0.0f;
}

// (Option<&dyn NormalConstraints>, Option<&dyn NormalConstraints>)::project_local_normals: the
// constraints of shape 1 act on n1 (then n2 := -n1 in shape 2's frame), then those of shape 2 on n2
// (then n1 := -n2 in shape 1's frame). Null = None.
__device__ __forceinline__ bool project_local_normals(const TriPN* c1, const TriPN* c2, const Pose& pos12, V3* n1, V3* n2) {
  if (c1) {
    if (!project_local_normal_mut(*c1, n1)) return false;
    *n2 = pose_inv_rotate(pos12, -*n1);
  }
  if (c2) {
    if (!project_local_normal_mut(*c2, n2)) return false;
    *n1 = pose_rotate(pos12, -*n2);
  }
  return true;
}

// Row j of a pseudo-normal table (12 floats: face, e01, e12, e20).
__device__ __forceinline__ TriPN load_tri_pn(const float* __restrict__ table, uint32_t j) {
  const float* q = table + 12 * (size_t)j;
  TriPN p;
  p.face = v3(q[0], q[1], q[2]);
  p.e[0] = v3(q[3], q[4], q[5]);
  p.e[1] = v3(q[6], q[7], q[8]);
  p.e[2] = v3(q[9], q[10], q[11]);
  return p;
}

}  // namespace pg
