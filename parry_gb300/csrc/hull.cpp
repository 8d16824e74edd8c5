// Host-side ConvexPolyhedron construction (input preparation for the contact-manifold kernels).
//
// parry builds a ConvexPolyhedron with ConvexPolyhedron::from_convex_hull(points)
// (src/shape/convex_polyhedron.rs:264-268): a convex hull triangulation, then from_convex_mesh
// (:390-639), which merges coplanar triangles into faces and builds the vertex / edge / face
// adjacency that the polygonal-feature and support-feature queries read.
//
// This file has two parts:
//   * hull_triangles: this library's own incremental hull in double precision. It produces the
//     same triangulation as any exact hull for points in general position, but not parry's
//     quickhull numbering (parry orders its initial simplex by a covariance eigen-decomposition);
//     a caller holding parry's own ConvexPolyhedron passes that topology through the C ABI instead.
//   * remove_unused_points and from_convex_mesh: restated step for step in f32 (src/utils/cleanup.rs:6-34,
//     src/shape/convex_polyhedron.rs:390-639), so the faces, normals and ids follow from the
//     triangles exactly as in the reference.
// Compiled without floating-point contraction (the f32 steps must round as the reference's).
#include "../../include/parry_gpu.h"
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <thread>
#include <atomic>
#include <unordered_map>
#include <unordered_set>
#include <vector>
#include <algorithm>
#include <array>

namespace {

struct D3 {
  double x, y, z;
};
inline D3 dsub(D3 a, D3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline D3 dcross(D3 a, D3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline double ddot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

// Incremental convex hull. Returns outward-oriented triangles (counter-clockwise seen from
// outside, so (b - a) x (c - a) points out), or an empty vector when the points span less than 3-D.
std::vector<std::array<uint32_t, 3>> hull_triangles(const float* pts, uint32_t n) {
  std::vector<std::array<uint32_t, 3>> out;
  if (n < 4) return out;
  std::vector<D3> p(n);
  D3 lo = {1e300, 1e300, 1e300}, hi = {-1e300, -1e300, -1e300};
  for (uint32_t i = 0; i < n; ++i) {
    p[i] = {pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]};
    lo = {std::min(lo.x, p[i].x), std::min(lo.y, p[i].y), std::min(lo.z, p[i].z)};
    hi = {std::max(hi.x, p[i].x), std::max(hi.y, p[i].y), std::max(hi.z, p[i].z)};
  }
  D3 ext = dsub(hi, lo);
  double scale = std::max(ext.x, std::max(ext.y, ext.z));
  if (!(scale > 0.0) || !std::isfinite(scale)) return out;
  const double eps = 1e-10 * scale;  // plane-distance tolerance
  // initial tetrahedron: extreme x, farthest point, farthest from the line, farthest from the plane
  uint32_t i0 = 0;
  for (uint32_t i = 1; i < n; ++i)
    if (p[i].x < p[i0].x) i0 = i;
  uint32_t i1 = i0;
  double best = -1.0;
  for (uint32_t i = 0; i < n; ++i) {
    D3 d = dsub(p[i], p[i0]);
    double l = ddot(d, d);
    if (l > best) { best = l; i1 = i; }
  }
  if (best <= eps * eps) return out;
  D3 e01 = dsub(p[i1], p[i0]);
  uint32_t i2 = i0;
  best = -1.0;
  for (uint32_t i = 0; i < n; ++i) {
    D3 c = dcross(e01, dsub(p[i], p[i0]));
    double l = ddot(c, c);
    if (l > best) { best = l; i2 = i; }
  }
  if (best <= (eps * scale) * (eps * scale)) return out;
  D3 nrm = dcross(e01, dsub(p[i2], p[i0]));
  double nn = std::sqrt(ddot(nrm, nrm));
  uint32_t i3 = i0;
  best = -1.0;
  double side = 0.0;
  for (uint32_t i = 0; i < n; ++i) {
    double d = ddot(nrm, dsub(p[i], p[i0])) / nn;
    if (std::fabs(d) > best) { best = std::fabs(d); i3 = i; side = d; }
  }
  if (best <= eps) return out;

  struct Face {
    uint32_t v[3];
    D3 n;
    double off;
    bool alive;
  };
  std::vector<Face> faces;
  auto add_face = [&](uint32_t a, uint32_t b, uint32_t c) {
    Face f;
    f.v[0] = a; f.v[1] = b; f.v[2] = c;
    D3 fn = dcross(dsub(p[b], p[a]), dsub(p[c], p[a]));
    double l = std::sqrt(ddot(fn, fn));
    f.n = l > 0 ? D3{fn.x / l, fn.y / l, fn.z / l} : D3{0, 0, 0};
    f.off = ddot(f.n, p[a]);
    f.alive = true;
    faces.push_back(f);
  };
  if (side > 0) {  // i3 above plane (i0, i1, i2): that face looks away from i3
    add_face(i0, i2, i1); add_face(i0, i1, i3); add_face(i1, i2, i3); add_face(i2, i0, i3);
  } else {
    add_face(i0, i1, i2); add_face(i0, i3, i1); add_face(i1, i3, i2); add_face(i2, i3, i0);
  }
  std::vector<uint8_t> used(n, 0);
  used[i0] = used[i1] = used[i2] = used[i3] = 1;
  auto key = [](uint32_t a, uint32_t b) { return ((uint64_t)a << 32) | b; };
  std::vector<uint32_t> visible;
  std::unordered_set<uint64_t> vis_edges;
  for (uint32_t pi = 0; pi < n; ++pi) {
    if (used[pi]) continue;
    visible.clear();
    for (uint32_t f = 0; f < faces.size(); ++f)
      if (faces[f].alive && ddot(faces[f].n, p[pi]) - faces[f].off > eps) visible.push_back(f);
    if (visible.empty()) continue;  // inside or on the hull
    vis_edges.clear();
    for (uint32_t f : visible)
      for (int k = 0; k < 3; ++k) vis_edges.insert(key(faces[f].v[k], faces[f].v[(k + 1) % 3]));
    std::vector<std::pair<uint32_t, uint32_t>> horizon;
    for (uint32_t f : visible) {
      for (int k = 0; k < 3; ++k) {
        uint32_t a = faces[f].v[k], b = faces[f].v[(k + 1) % 3];
        if (!vis_edges.count(key(b, a))) horizon.push_back({a, b});
      }
      faces[f].alive = false;
    }
    for (auto& e : horizon) add_face(e.first, e.second, pi);
    used[pi] = 1;
  }
  for (auto& f : faces)
    if (f.alive) out.push_back({f.v[0], f.v[1], f.v[2]});
  return out;
}

// --- f32 restatement of the reference's cleanup and from_convex_mesh ---
struct F3 {
  float x, y, z;
};
inline F3 fsub(F3 a, F3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline float fdot(F3 a, F3 b) {
  float p0 = a.x * b.x, p1 = a.y * b.y, p2 = a.z * b.z;
  return (p0 + p1) + p2;
}
inline F3 fcross(F3 a, F3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline bool unit_try_new(F3 v, float min_norm, F3* out) {
  float sq = fdot(v, v);
  if (sq > min_norm * min_norm) {
    float l = std::sqrt(sq);
    *out = {v.x / l, v.y / l, v.z / l};
    return true;
  }
  return false;
}
constexpr float F32_EPS = 1.1920929e-7f;

// utils::remove_unused_points (src/utils/cleanup.rs:6-34)
void remove_unused_points(std::vector<F3>& points, std::vector<std::array<uint32_t, 3>>& idx) {
  std::vector<uint8_t> used(points.size(), 0);
  std::vector<size_t> remap(points.size());
  for (size_t i = 0; i < remap.size(); ++i) remap[i] = i;
  for (auto& t : idx) used[t[0]] = used[t[1]] = used[t[2]] = 1;
  size_t i = 0;
  while (i != points.size()) {
    if (!used[i]) {
      points[i] = points.back();  // swap_remove
      points.pop_back();
      remap[points.size()] = i;
      used[i] = used[points.size()];
    } else {
      ++i;
    }
  }
  for (auto& t : idx)
    for (int k = 0; k < 3; ++k) t[k] = (uint32_t)remap[t[k]];
}

struct Polyhedron {
  std::vector<F3> points;
  std::vector<F3> face_normals;
  std::vector<uint32_t> face_first, face_count;   // into face_vertices / face_edges
  std::vector<uint32_t> face_vertices, face_edges;
  std::vector<uint32_t> vertex_first, vertex_count;  // into vertex_faces / vertex_edges
  std::vector<uint32_t> vertex_faces, vertex_edges;
  std::vector<F3> edge_dirs;
  std::vector<uint32_t> edge_vertices;  // 2 per edge
};

// ConvexPolyhedron::from_convex_mesh (src/shape/convex_polyhedron.rs:390-639). False for the
// reference's None.
bool from_convex_mesh(std::vector<F3> points, const std::vector<std::array<uint32_t, 3>>& indices, Polyhedron* out) {
  const float eps = std::sqrt(F32_EPS);
  struct Edge {
    uint32_t v[2];
    uint32_t faces[2];
    F3 dir;
    bool deleted;
  };
  struct Tri {
    uint32_t v[3], e[3];
    F3 normal;
    int64_t parent;
  };
  std::vector<Edge> edges;
  std::vector<Tri> tris;
  std::unordered_map<uint64_t, uint32_t> edge_map;
  if (points.size() + indices.size() <= 2) return false;
  for (auto& idx : indices) {
    Tri t;
    uint32_t face_id = (uint32_t)tris.size();
    if (idx[0] == idx[1] || idx[0] == idx[2] || idx[1] == idx[2]) return false;
    for (int i1 = 0; i1 < 3; ++i1) {
      int i2 = (i1 + 1) % 3;
      uint32_t a = std::min(idx[i1], idx[i2]), b = std::max(idx[i1], idx[i2]);
      uint64_t k = ((uint64_t)a << 32) | b;
      auto it = edge_map.find(k);
      if (it != edge_map.end()) {
        Edge& e = edges[it->second];
        if (e.faces[1] == UINT32_MAX) {
          t.e[i1] = it->second;
          e.faces[1] = face_id;
        } else {
          return false;  // t-junction
        }
      } else {
        uint32_t id = (uint32_t)edges.size();
        edge_map.emplace(k, id);
        t.e[i1] = id;
        F3 d;
        bool ok = unit_try_new(fsub(points[idx[i2]], points[idx[i1]]), F32_EPS, &d);
        edges.push_back(Edge{{idx[i1], idx[i2]}, {face_id, UINT32_MAX}, ok ? d : F3{1.f, 0.f, 0.f}, !ok});
      }
    }
    F3 n;
    bool ok = unit_try_new(fcross(fsub(points[idx[1]], points[idx[0]]), fsub(points[idx[2]], points[idx[0]])), F32_EPS, &n);
    for (int k = 0; k < 3; ++k) t.v[k] = idx[k];
    t.normal = ok ? n : F3{0.f, 0.f, 0.f};
    t.parent = -1;
    tris.push_back(t);
  }
  for (auto& e : edges) {
    if (e.faces[0] >= tris.size() || e.faces[1] >= tris.size()) return false;
    if (fdot(tris[e.faces[0]].normal, tris[e.faces[1]].normal) > 1.0f - eps) e.deleted = true;
  }
  auto next_edge_id = [&](const Tri& t, uint32_t id) -> int {
    for (int i = 0; i < 3; ++i)
      if (t.e[i] == id) return (i + 1) % 3;
    return -1;
  };
  struct FaceRec {
    uint32_t first, num;
    F3 normal;
  };
  std::vector<FaceRec> faces;
  for (size_t i = 0; i < tris.size(); ++i) {
    if (tris[i].parent >= 0) continue;
    for (int j1 = 0; j1 < 3; ++j1) {
      if (edges[tris[i].e[j1]].deleted) continue;
      uint32_t new_face_id = (uint32_t)faces.size();
      FaceRec nf{(uint32_t)out->face_edges.size(), 1, tris[i].normal};
      out->face_edges.push_back(tris[i].e[j1]);
      out->face_vertices.push_back(tris[i].v[j1]);
      int j2 = (j1 + 1) % 3;
      uint32_t start_vertex = tris[i].v[j1];
      size_t curr_tri = i;
      int curr_edge_id = j2;
      size_t guard = 0;
      while (tris[curr_tri].v[curr_edge_id] != start_vertex) {
        if (++guard > 4 * (tris.size() + 3)) return false;  // malformed topology
        uint32_t curr_edge = tris[curr_tri].e[curr_edge_id];
        uint32_t curr_vertex = tris[curr_tri].v[curr_edge_id];
        tris[curr_tri].parent = new_face_id;
        if (!edges[curr_edge].deleted) {
          out->face_edges.push_back(curr_edge);
          out->face_vertices.push_back(curr_vertex);
          nf.num += 1;
          curr_edge_id = (curr_edge_id + 1) % 3;
        } else {
          const Edge& e = edges[curr_edge];
          curr_tri = e.faces[0] == curr_tri ? e.faces[1] : e.faces[0];
          curr_edge_id = next_edge_id(tris[curr_tri], curr_edge);
          if (curr_edge_id < 0 || tris[curr_tri].v[curr_edge_id] != curr_vertex) return false;
        }
      }
      // Degenerate faces (an isolated edge left by rounding) are dropped, as in the reference;
      // their entries stay in the adjacency arrays there too.
      if (nf.num > 2) faces.push_back(nf);
      break;
    }
  }
  for (auto& e : edges) {
    if (tris[e.faces[0]].parent >= 0) e.faces[0] = (uint32_t)tris[e.faces[0]].parent;
    if (tris[e.faces[1]].parent >= 0) e.faces[1] = (uint32_t)tris[e.faces[1]].parent;
  }
  size_t nv = points.size();
  out->vertex_first.assign(nv, 0);
  out->vertex_count.assign(nv, 0);
  for (auto& f : faces)
    for (uint32_t k = f.first; k < f.first + f.num; ++k) out->vertex_count[out->face_vertices[k]] += 1;
  uint32_t total = 0;
  for (size_t v = 0; v < nv; ++v) {
    out->vertex_first[v] = total;
    total += out->vertex_count[v];
  }
  out->vertex_faces.assign(total, 0);
  out->vertex_edges.assign(total, 0);
  std::fill(out->vertex_count.begin(), out->vertex_count.end(), 0u);
  for (size_t fi = 0; fi < faces.size(); ++fi) {
    const FaceRec& f = faces[fi];
    for (uint32_t k = f.first; k < f.first + f.num; ++k) {
      uint32_t v = out->face_vertices[k];
      uint32_t slot = out->vertex_first[v] + out->vertex_count[v];
      out->vertex_faces[slot] = (uint32_t)fi;
      out->vertex_edges[slot] = out->face_edges[k];
      out->vertex_count[v] += 1;
    }
  }
  for (auto& f : faces) {
    out->face_normals.push_back(f.normal);
    out->face_first.push_back(f.first);
    out->face_count.push_back(f.num);
  }
  for (auto& e : edges) {
    out->edge_dirs.push_back(e.dir);
    out->edge_vertices.push_back(e.v[0]);
    out->edge_vertices.push_back(e.v[1]);
  }
  out->points = std::move(points);
  return true;
}

}  // namespace

struct parrygpu_polyhedra_builder {
  std::vector<Polyhedron> hulls;
  std::vector<uint8_t> ok;
};

extern "C" {

parrygpu_status parrygpu_polyhedra_build(const float* points, const uint32_t* first, const uint32_t* count, uint64_t n_hulls,
                                         uint32_t threads, parrygpu_polyhedra_builder** out) {
  if (!out || (n_hulls && (!points || !first || !count))) return PARRYGPU_INVALID_ARG;
  auto* b = new parrygpu_polyhedra_builder();
  b->hulls.resize(n_hulls);
  b->ok.assign(n_hulls, 0);
  std::atomic<uint64_t> next{0};
  auto work = [&]() {
    for (;;) {
      uint64_t h = next.fetch_add(1);
      if (h >= n_hulls) break;
      const float* p = points + 3 * (size_t)first[h];
      uint32_t n = count[h];
      std::vector<std::array<uint32_t, 3>> tris = hull_triangles(p, n);
      std::vector<F3> pts(n);
      for (uint32_t i = 0; i < n; ++i) pts[i] = {p[3 * i], p[3 * i + 1], p[3 * i + 2]};
      if (tris.empty()) {
        b->hulls[h].points = pts;  // degenerate cloud: no topology
        continue;
      }
      remove_unused_points(pts, tris);
      Polyhedron poly;
      if (from_convex_mesh(pts, tris, &poly)) {
        b->hulls[h] = std::move(poly);
        b->ok[h] = 1;
      } else {
        b->hulls[h] = Polyhedron();
        b->hulls[h].points = pts;
      }
    }
  };
  uint32_t nt = threads ? threads : std::max(1u, std::thread::hardware_concurrency());
  if (nt > 64) nt = 64;
  if (n_hulls < 64) nt = 1;
  std::vector<std::thread> ts;
  for (uint32_t t = 1; t < nt; ++t) ts.emplace_back(work);
  work();
  for (auto& t : ts) t.join();
  *out = b;
  return PARRYGPU_OK;
}

parrygpu_status parrygpu_polyhedra_sizes(const parrygpu_polyhedra_builder* b, uint64_t* sizes) {
  if (!b || !sizes) return PARRYGPU_INVALID_ARG;
  uint64_t s[5] = {0, 0, 0, 0, 0};
  for (auto& h : b->hulls) {
    s[0] += h.points.size();
    s[1] += h.face_normals.size();
    s[2] += h.face_vertices.size();
    s[3] += h.vertex_faces.size();
    s[4] += h.edge_dirs.size();
  }
  std::memcpy(sizes, s, sizeof(s));
  return PARRYGPU_OK;
}

parrygpu_status parrygpu_polyhedra_copy(const parrygpu_polyhedra_builder* b, float* points, uint32_t* hulls, float* face_normals,
                                        uint32_t* face_ranges, uint32_t* face_vertices, uint32_t* face_edges, uint32_t* vertex_ranges,
                                        uint32_t* vertex_faces, uint32_t* vertex_edges, float* edge_dirs) {
  if (!b || !points || !hulls) return PARRYGPU_INVALID_ARG;
  uint64_t vp = 0, fp = 0, fe = 0, ve = 0, ep = 0;
  for (size_t h = 0; h < b->hulls.size(); ++h) {
    const Polyhedron& P = b->hulls[h];
    uint32_t* r = hulls + 8 * h;
    r[0] = (uint32_t)vp; r[1] = (uint32_t)P.points.size();
    r[2] = (uint32_t)fp; r[3] = (uint32_t)P.face_normals.size();
    r[4] = (uint32_t)ep; r[5] = (uint32_t)P.edge_dirs.size();
    r[6] = b->ok[h]; r[7] = 0;
    for (size_t i = 0; i < P.points.size(); ++i) {
      points[3 * (vp + i)] = P.points[i].x; points[3 * (vp + i) + 1] = P.points[i].y; points[3 * (vp + i) + 2] = P.points[i].z;
      if (vertex_ranges) {
        bool has = i < P.vertex_first.size();
        vertex_ranges[2 * (vp + i)] = has ? (uint32_t)(ve + P.vertex_first[i]) : (uint32_t)ve;
        vertex_ranges[2 * (vp + i) + 1] = has ? P.vertex_count[i] : 0u;
      }
    }
    for (size_t f = 0; f < P.face_normals.size(); ++f) {
      if (face_normals) {
        face_normals[3 * (fp + f)] = P.face_normals[f].x; face_normals[3 * (fp + f) + 1] = P.face_normals[f].y;
        face_normals[3 * (fp + f) + 2] = P.face_normals[f].z;
      }
      if (face_ranges) { face_ranges[2 * (fp + f)] = (uint32_t)(fe + P.face_first[f]); face_ranges[2 * (fp + f) + 1] = P.face_count[f]; }
    }
    for (size_t k = 0; k < P.face_vertices.size(); ++k) {
      if (face_vertices) face_vertices[fe + k] = P.face_vertices[k];
      if (face_edges) face_edges[fe + k] = P.face_edges[k];
    }
    for (size_t k = 0; k < P.vertex_faces.size(); ++k) {
      if (vertex_faces) vertex_faces[ve + k] = P.vertex_faces[k];
      if (vertex_edges) vertex_edges[ve + k] = P.vertex_edges[k];
    }
    for (size_t e = 0; e < P.edge_dirs.size(); ++e)
      if (edge_dirs) { edge_dirs[3 * (ep + e)] = P.edge_dirs[e].x; edge_dirs[3 * (ep + e) + 1] = P.edge_dirs[e].y; edge_dirs[3 * (ep + e) + 2] = P.edge_dirs[e].z; }
    vp += P.points.size(); fp += P.face_normals.size(); fe += P.face_vertices.size(); ve += P.vertex_faces.size(); ep += P.edge_dirs.size();
  }
  return PARRYGPU_OK;
}

void parrygpu_polyhedra_builder_destroy(parrygpu_polyhedra_builder* b) { delete b; }

}  // extern "C"
