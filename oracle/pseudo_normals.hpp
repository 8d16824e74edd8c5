// Oracle (test infrastructure only): CPU restatement of parry3d's triangle pseudo-normals and the
// normal constraints they put on contact manifolds against a TriMesh built with
// TriMeshFlags::FIX_INTERNAL_EDGES. Paths relative to the parry repository:
//   src/shape/triangle_pseudo_normals.rs:20-99        TrianglePseudoNormals, project_local_normal_mut
//   src/query/contact_manifolds/normals_constraint.rs:14-126   project_local_normal1 / 2, the pair rule
//   src/shape/trimesh.rs:1251-1320                    merge_duplicate_vertices (implied by FIX_INTERNAL_EDGES)
//   src/shape/trimesh.rs:1348-1407                    compute_pseudo_normals (edge part)
//   src/shape/trimesh.rs:1911-1931                    triangle_normal_constraints
//   src/shape/triangle.rs:226-228, 324-328            Triangle::normal, scaled_normal
#pragma once
#include "math.hpp"

#include <cstring>
#include <map>
#include <unordered_map>
#include <vector>

namespace oracle {

template <class R> struct TriPseudoNormals {
  Vec3<R> face;
  Vec3<R> edges[3];
};

// Vector::try_normalize(min_norm): None when |v| <= min_norm (the norm form, unlike Unit::try_new).
template <class R> inline bool try_normalize_norm(const Vec3<R>& v, R min_norm, Vec3<R>* out) {
  R n = norm(v);
  if (n <= min_norm) return false;
  *out = v / n;
  return true;
}

// TrianglePseudoNormals::project_local_normal_mut (triangle_pseudo_normals.rs:35-99).
template <class R> inline bool project_local_normal_mut(const TriPseudoNormals<R>& pn, Vec3<R>* dir) {
  const R dot_face = dot(*dir, pn.face);
  Vec3<R> dots(dot(*dir, pn.edges[0]), dot(*dir, pn.edges[1]), dot(*dir, pn.edges[2]));
  const Vec3<R>& closest_edge = pn.edges[imax(dots)];
  if (closest_edge == pn.face) {
    *dir = pn.face;
    return dot_face >= R(0);
  }
  const R dot_edge_face = dot(pn.face, closest_edge);
  const R dot_dir_face = dot(pn.face, *dir);
  const R dot_corrected_dir_face = R(2) * dot_edge_face * dot_edge_face - R(1);
  if (dot_dir_face >= dot_corrected_dir_face) return true;
  Vec3<R> edge_on_normal = pn.face * dot_edge_face;
  Vec3<R> edge_orthogonal_to_normal = closest_edge - edge_on_normal;
  Vec3<R> dir_on_normal = pn.face * dot_dir_face;
  Vec3<R> dir_orthogonal_to_normal = *dir - dir_on_normal;
  Vec3<R> unit_dir_orthogonal;
  if (!try_normalize_norm(dir_orthogonal_to_normal, R(1.0e-6), &unit_dir_orthogonal)) return dot_face >= R(0);
  Vec3<R> adjusted;
  if (!try_normalize_norm(edge_on_normal + unit_dir_orthogonal * norm(edge_orthogonal_to_normal), R(1.0e-6), &adjusted))
    return dot_face >= R(0);
  *dir = adjusted * (R(2) * dot(pn.face, adjusted)) - pn.face;
  return dot_face >= R(0);
}

// NormalConstraints::project_local_normal1 (normals_constraint.rs:41-55): the constraint belongs to
// shape 1; normal2 := -normal1 in shape 2's frame.
template <class R> inline bool project_local_normal1(const TriPseudoNormals<R>& pn, const Iso<R>& pos12, Vec3<R>* n1, Vec3<R>* n2) {
  if (!project_local_normal_mut(pn, n1)) return false;
  *n2 = pos12.inverse_transform_vector(-*n1);
  return true;
}

// NormalConstraints::project_local_normal2 (normals_constraint.rs:66-80): the constraint belongs to
// shape 2; normal1 := -normal2 in shape 1's frame.
template <class R> inline bool project_local_normal2(const TriPseudoNormals<R>& pn, const Iso<R>& pos12, Vec3<R>* n1, Vec3<R>* n2) {
  if (!project_local_normal_mut(pn, n2)) return false;
  *n1 = pos12.transform_vector(-*n2);
  return true;
}

// (Option<&dyn NormalConstraints>, Option<&dyn NormalConstraints>)::project_local_normals
// (normals_constraint.rs:104-125).
template <class R>
inline bool project_local_normals(const TriPseudoNormals<R>* c1, const TriPseudoNormals<R>* c2, const Iso<R>& pos12, Vec3<R>* n1,
                                  Vec3<R>* n2) {
  if (c1 && !project_local_normal1(*c1, pos12, n1, n2)) return false;
  if (c2) return project_local_normal2(*c2, pos12, n1, n2);
  return true;
}

// Triangle::normal(): Unit::try_new((b - a) x (c - a), DEFAULT_EPSILON).
template <class R> inline bool triangle_normal(const Vec3<R>& a, const Vec3<R>& b, const Vec3<R>& c, Vec3<R>* n) {
  return try_normalize(cross(b - a, c - a), std::numeric_limits<R>::epsilon(), n);
}

// TriMesh::triangle_normal_constraints of every triangle of a mesh with FIX_INTERNAL_EDGES:
//   merge_duplicate_vertices: two vertices are one when their coordinates compare equal and hash
//     alike (HashablePartialEq: PartialEq on the values, hash of the bytes), i.e. bit-identical and
//     NaN-free; the vertex numbering it produces does not change any result here.
//   compute_pseudo_normals: the pseudo-normal of an edge (sorted pair of merged vertex ids) is the
//     sum, in triangle order from zero, of the unit normals of the triangles that have a normal and
//     contain that edge.
//   triangle_normal_constraints: Some({face: normal, edges: [e01, e12, e20] each Unit::try_new(.,
//     1e-6)}) if every piece exists, else None.
// out: 12 floats per triangle (face, e01, e12, e20); valid: 1 when Some.
template <class R>
inline void trimesh_pseudo_normals(const float* vtx, uint32_t nv, const uint32_t* idx, uint32_t nt, R* out, uint8_t* valid) {
  struct Key {
    uint32_t w[3];
    bool operator==(const Key& o) const { return w[0] == o.w[0] && w[1] == o.w[1] && w[2] == o.w[2]; }
  };
  struct KeyHash {
    size_t operator()(const Key& k) const { return ((size_t)k.w[0] * 0x9E3779B97F4A7C15ull) ^ ((size_t)k.w[1] * 0xC2B2AE3D27D4EB4Full) ^ k.w[2]; }
  };
  std::unordered_map<Key, uint32_t, KeyHash> ids;
  uint32_t next = 0;
  auto resolve = [&](uint32_t v) -> uint32_t {
    const float* p = vtx + 3 * (size_t)v;
    if (std::isnan(p[0]) || std::isnan(p[1]) || std::isnan(p[2])) return next++;  // NaN never compares equal
    Key k;
    std::memcpy(k.w, p, 12);
    auto it = ids.find(k);
    if (it != ids.end()) return it->second;
    ids.emplace(k, next);
    return next++;
  };
  std::vector<uint32_t> merged((size_t)nt * 3);
  for (size_t i = 0; i < (size_t)nt * 3; ++i) merged[i] = idx[i] < nv ? resolve(idx[i]) : next++;
  auto pos = [&](uint32_t t, int k) {
    const float* p = vtx + 3 * (size_t)idx[3 * (size_t)t + k];
    return Vec3<R>((R)p[0], (R)p[1], (R)p[2]);
  };
  auto sorted = [](uint32_t a, uint32_t b) { return a < b ? std::make_pair(a, b) : std::make_pair(b, a); };
  std::map<std::pair<uint32_t, uint32_t>, Vec3<R>> edge_n;
  std::vector<Vec3<R>> face((size_t)nt);
  std::vector<uint8_t> has_face((size_t)nt, 0);
  for (uint32_t t = 0; t < nt; ++t) {
    has_face[t] = triangle_normal(pos(t, 0), pos(t, 1), pos(t, 2), &face[t]);
    if (!has_face[t]) continue;
    const uint32_t* m = &merged[3 * (size_t)t];
    for (auto e : {sorted(m[0], m[1]), sorted(m[0], m[2]), sorted(m[1], m[2])}) {
      auto it = edge_n.find(e);
      if (it == edge_n.end()) it = edge_n.emplace(e, Vec3<R>()).first;
      it->second += face[t];
    }
  }
  for (uint32_t t = 0; t < nt; ++t) {
    R* o = out + 12 * (size_t)t;
    for (int k = 0; k < 12; ++k) o[k] = R(0);
    valid[t] = 0;
    if (!has_face[t]) continue;
    const uint32_t* m = &merged[3 * (size_t)t];
    std::pair<uint32_t, uint32_t> es[3] = {sorted(m[0], m[1]), sorted(m[1], m[2]), sorted(m[2], m[0])};
    Vec3<R> en[3];
    bool ok = true;
    for (int k = 0; k < 3; ++k) {
      auto it = edge_n.find(es[k]);
      Vec3<R> sum = it == edge_n.end() ? Vec3<R>() : it->second;
      ok = ok && try_normalize(sum, R(1.0e-6), &en[k]);
    }
    if (!ok) continue;
    valid[t] = 1;
    o[0] = face[t].x; o[1] = face[t].y; o[2] = face[t].z;
    for (int k = 0; k < 3; ++k) { o[3 + 3 * k] = en[k].x; o[4 + 3 * k] = en[k].y; o[5 + 3 * k] = en[k].z; }
  }
}

}  // namespace oracle
