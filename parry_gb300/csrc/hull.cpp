// Host-side ConvexPolyhedron construction (ConvexPolyhedron::from_convex_hull for many clouds on
// the CPU threads): the same algorithm as the GPU builder (hull_build.cu), from hull_core.hpp, with
// stride-1 workspaces. Compiled without floating-point contraction, like the device code.
#include "../../include/parry_gpu.h"
#include "hull_core.hpp"

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

using namespace hullcore;

namespace {

// One thread's workspace, sized for clouds of up to `n` points.
struct HostWs {
  HullCaps caps;
  std::vector<D3> pts;
  std::vector<HFace> faces;
  std::vector<uint32_t> visible, horizon, tris, used, remap;
  std::vector<F3> fpts;
  std::vector<HEdge> edges;
  std::vector<uint64_t> hkeys;
  std::vector<uint32_t> hvals;
  std::vector<HTri> htris;
  std::vector<HFaceRec> frecs;
  std::vector<uint32_t> face_edges, face_vertices, vertex_first, vertex_count, vertex_faces, vertex_edges;
  HullWs ws;

  void reserve(uint32_t n) {
    caps = HullCaps::of(n);
    pts.resize(n); faces.resize(caps.faces); visible.resize(caps.faces); horizon.resize(HORIZON_WORDS * caps.horizon);
    tris.resize(3 * caps.tris); used.resize(n); remap.resize(n); fpts.resize(n); edges.resize(caps.edges);
    hkeys.resize(caps.hash); hvals.resize(caps.hash); htris.resize(caps.tris); frecs.resize(caps.tris);
    face_edges.resize(caps.entries); face_vertices.resize(caps.entries); vertex_first.resize(n); vertex_count.resize(n);
    vertex_faces.resize(caps.entries); vertex_edges.resize(caps.entries);
    ws = HullWs{{pts.data(), 1}, {faces.data(), 1}, {visible.data(), 1}, {horizon.data(), 1}, {tris.data(), 1},
                {used.data(), 1}, {remap.data(), 1}, {fpts.data(), 1}, {edges.data(), 1}, {hkeys.data(), 1},
                {hvals.data(), 1}, {htris.data(), 1}, {frecs.data(), 1}, {face_edges.data(), 1}, {face_vertices.data(), 1},
                {vertex_first.data(), 1}, {vertex_count.data(), 1}, {vertex_faces.data(), 1}, {vertex_edges.data(), 1}};
  }
};

// One built hull, copied out of the workspace in the output layout (offsets relative to the hull).
struct HostHull {
  HullOut r;
  std::vector<float> points, face_normals, edge_dirs;
  std::vector<uint32_t> face_ranges, face_vertices, face_edges, vertex_ranges, vertex_faces, vertex_edges;
  std::vector<uint32_t> triangles;
};

}  // namespace

struct parrygpu_polyhedra_builder {
  std::vector<HostHull> hulls;
};

extern "C" {

parrygpu_status parrygpu_polyhedra_build(const float* points, const uint32_t* first, const uint32_t* count, uint64_t n_hulls,
                                         uint32_t threads, parrygpu_polyhedra_builder** out) {
  if (!out || (n_hulls && (!points || !first || !count))) return PARRYGPU_INVALID_ARG;
  auto* b = new parrygpu_polyhedra_builder();
  b->hulls.resize(n_hulls);
  std::atomic<uint64_t> next{0};
  auto work = [&]() {
    HostWs w;
    uint32_t cap = 0;
    for (;;) {
      uint64_t h = next.fetch_add(1);
      if (h >= n_hulls) break;
      const uint32_t n = count[h];
      if (n > cap || cap == 0) { cap = std::max(n, 64u); w.reserve(cap); }
      const float* p = points + 3 * (size_t)first[h];
      HostHull& H = b->hulls[h];
      H.r = build_one(p, n, w.caps, w.ws);
      H.points.resize(3 * (size_t)H.r.npts);
      H.vertex_ranges.resize(2 * (size_t)H.r.npts);
      const uint32_t nf = H.r.ok ? H.r.nfaces : 0, nfe = H.r.ok ? H.r.nfentries : 0, nve = H.r.ok ? H.r.nventries : 0,
                     ne = H.r.ok ? H.r.nedges : 0;
      H.face_normals.resize(3 * (size_t)nf); H.face_ranges.resize(2 * (size_t)nf);
      H.face_vertices.resize(nfe); H.face_edges.resize(nfe); H.vertex_faces.resize(nve); H.vertex_edges.resize(nve);
      H.edge_dirs.resize(3 * (size_t)ne);
      H.triangles.resize(3 * (size_t)H.r.ntris);
      PolyOut o{H.points.data(), nullptr, H.face_normals.data(), H.face_ranges.data(), H.face_vertices.data(), H.face_edges.data(),
                H.vertex_ranges.data(), H.vertex_faces.data(), H.vertex_edges.data(), H.edge_dirs.data(), H.triangles.data()};
      emit(w.ws, H.r, 0, 0, 0, 0, 0, 0, o);
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
    s[0] += h.r.npts;
    s[1] += h.face_normals.size() / 3;
    s[2] += h.face_vertices.size();
    s[3] += h.vertex_faces.size();
    s[4] += h.edge_dirs.size() / 3;
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
    const HostHull& H = b->hulls[h];
    const uint32_t np = H.r.npts, nf = (uint32_t)(H.face_normals.size() / 3), nfe = (uint32_t)H.face_vertices.size(),
                   nve = (uint32_t)H.vertex_faces.size(), ne = (uint32_t)(H.edge_dirs.size() / 3);
    uint32_t* r = hulls + 8 * h;
    r[0] = (uint32_t)vp; r[1] = np; r[2] = (uint32_t)fp; r[3] = nf; r[4] = (uint32_t)ep; r[5] = ne; r[6] = H.r.ok ? 1u : 0u; r[7] = 0;
    std::memcpy(points + 3 * vp, H.points.data(), H.points.size() * 4);
    if (vertex_ranges)
      for (uint32_t i = 0; i < np; ++i) {
        vertex_ranges[2 * (vp + i)] = (uint32_t)(ve + H.vertex_ranges[2 * i]);
        vertex_ranges[2 * (vp + i) + 1] = H.vertex_ranges[2 * i + 1];
      }
    if (face_normals && nf) std::memcpy(face_normals + 3 * fp, H.face_normals.data(), H.face_normals.size() * 4);
    if (face_ranges)
      for (uint32_t f = 0; f < nf; ++f) {
        face_ranges[2 * (fp + f)] = (uint32_t)(fe + H.face_ranges[2 * f]);
        face_ranges[2 * (fp + f) + 1] = H.face_ranges[2 * f + 1];
      }
    if (face_vertices && nfe) std::memcpy(face_vertices + fe, H.face_vertices.data(), (size_t)nfe * 4);
    if (face_edges && nfe) std::memcpy(face_edges + fe, H.face_edges.data(), (size_t)nfe * 4);
    if (vertex_faces && nve) std::memcpy(vertex_faces + ve, H.vertex_faces.data(), (size_t)nve * 4);
    if (vertex_edges && nve) std::memcpy(vertex_edges + ve, H.vertex_edges.data(), (size_t)nve * 4);
    if (edge_dirs && ne) std::memcpy(edge_dirs + 3 * ep, H.edge_dirs.data(), H.edge_dirs.size() * 4);
    vp += np; fp += nf; fe += nfe; ve += nve; ep += ne;
  }
  return PARRYGPU_OK;
}

parrygpu_status parrygpu_polyhedra_triangles(const parrygpu_polyhedra_builder* b, uint64_t* n_triangles, uint32_t* tri_ranges,
                                             uint32_t* triangles) {
  if (!b) return PARRYGPU_INVALID_ARG;
  uint64_t tp = 0;
  for (size_t h = 0; h < b->hulls.size(); ++h) {
    const HostHull& H = b->hulls[h];
    const uint32_t nt = (uint32_t)(H.triangles.size() / 3);
    if (tri_ranges) { tri_ranges[2 * h] = (uint32_t)tp; tri_ranges[2 * h + 1] = nt; }
    if (triangles && nt) std::memcpy(triangles + 3 * tp, H.triangles.data(), H.triangles.size() * 4);
    tp += nt;
  }
  if (n_triangles) *n_triangles = tp;
  return PARRYGPU_OK;
}

void parrygpu_polyhedra_builder_destroy(parrygpu_polyhedra_builder* b) { delete b; }

}  // extern "C"
