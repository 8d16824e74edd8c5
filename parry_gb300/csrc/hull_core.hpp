// ConvexPolyhedron construction shared by the host builder (hull.cpp) and the GPU builder
// (hull_build.cu): one code path, so both produce the same bytes. parry builds a ConvexPolyhedron
// with ConvexPolyhedron::from_convex_hull(points) (src/shape/convex_polyhedron.rs:264-268, paths
// relative to the parry repository): a convex hull triangulation, then from_convex_mesh (:390-639),
// which merges coplanar triangles into faces and builds the vertex / edge / face adjacency.
//
//   hull_triangles: this library's own incremental hull in double precision. It produces the same
//     triangulation as any exact hull for points in general position, but not parry's quickhull
//     numbering (parry orders its initial simplex by a covariance eigen-decomposition); a caller
//     holding parry's own ConvexPolyhedron passes that topology through the C ABI instead.
//   remove_unused_points and from_convex_mesh: restated step for step in f32 (src/utils/cleanup.rs:6-34,
//     src/shape/convex_polyhedron.rs:390-639), so the faces, normals and ids follow from the
//     triangles exactly as in the reference.
//
// Every array lives in a caller-provided workspace reached through strided spans: the host passes
// stride 1, a GPU thread its own lane of arrays interleaved across threads (coalesced when the
// threads of a warp walk the same step). Capacities follow from the point count n (HullCaps). The
// arithmetic is written without contraction-sensitive forms; both builds compile it without FMA.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cmath>

#if defined(__CUDACC__)
#define HC_FN __host__ __device__ inline
#else
#define HC_FN inline
#endif

namespace hullcore {

template <class T> struct Span {
  T* p;
  size_t stride;
  HC_FN T& operator[](size_t i) const { return p[i * stride]; }
};

struct D3 {
  double x, y, z;
};
HC_FN D3 dsub(D3 a, D3 b) { return D3{a.x - b.x, a.y - b.y, a.z - b.z}; }
HC_FN D3 dcross(D3 a, D3 b) { return D3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
HC_FN double ddot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
HC_FN double dmin(double a, double b) { return (b < a) ? b : a; }  // std::min
HC_FN double dmax(double a, double b) { return (a < b) ? b : a; }  // std::max

struct F3 {
  float x, y, z;
};
HC_FN F3 fsub(F3 a, F3 b) { return F3{a.x - b.x, a.y - b.y, a.z - b.z}; }
HC_FN float fdot(F3 a, F3 b) {
  float p0 = a.x * b.x, p1 = a.y * b.y, p2 = a.z * b.z;
  return (p0 + p1) + p2;
}
HC_FN F3 fcross(F3 a, F3 b) { return F3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
// Unit::try_new(v, min_norm)
HC_FN bool unit_try_new(F3 v, float min_norm, F3* out) {
  float sq = fdot(v, v);
  if (sq > min_norm * min_norm) {
    float l = sqrtf(sq);
    *out = F3{v.x / l, v.y / l, v.z / l};
    return true;
  }
  return false;
}
constexpr float F32_EPS = 1.1920929e-7f;
constexpr uint32_t NONE = 0xffffffffu;

struct HFace {
  uint32_t v[3];
  uint32_t alive;
  D3 n;
  double off;
};

struct HEdge {
  uint32_t v[2];
  uint32_t faces[2];
  F3 dir;
  uint32_t deleted;
};

struct HTri {
  uint32_t v[3], e[3];
  F3 normal;
  uint32_t parent;  // NONE = not yet in a face
};

struct HFaceRec {
  uint32_t first, num;
  F3 normal;
};

// Capacities for a cloud of n points: a closed triangulated hull has at most 2n - 4 triangles and
// 3n - 6 edges, and the horizon of a point seen from outside is one cycle of hull edges; the
// incremental hull keeps dead faces until it compacts them.
struct HullCaps {
  uint32_t n, faces, horizon, tris, edges, hash, entries;
  HC_FN static HullCaps of(uint32_t n) {
    HullCaps c;
    c.n = n;
    c.faces = 4 * n + 16;
    c.horizon = 2 * n + 16;
    c.tris = 2 * n + 4;
    c.edges = 3 * n + 8;
    uint32_t h = 16;
    while (h < 2 * c.edges) h <<= 1;
    c.hash = h;
    c.entries = 3 * c.tris;
    return c;
  }
};

// The workspace of one hull (every span sized by HullCaps of the largest cloud it serves).
struct HullWs {
  Span<D3> pts;              // n
  Span<HFace> faces;         // caps.faces
  Span<uint32_t> visible;    // caps.faces
  Span<uint32_t> horizon;    // 2 x caps.horizon
  Span<uint32_t> tris;       // 3 x caps.tris
  Span<uint32_t> used;       // n
  Span<uint32_t> remap;      // n
  Span<F3> fpts;             // n
  Span<HEdge> edges;         // caps.edges
  Span<uint64_t> hkeys;      // caps.hash
  Span<uint32_t> hvals;      // caps.hash
  Span<HTri> htris;          // caps.tris
  Span<HFaceRec> frecs;      // caps.tris
  Span<uint32_t> face_edges, face_vertices;    // caps.entries
  Span<uint32_t> vertex_first, vertex_count;   // n
  Span<uint32_t> vertex_faces, vertex_edges;   // caps.entries
};

// Incremental convex hull of pts[0..n) (x, y, z floats). Writes the outward-oriented triangles
// (counter-clockwise seen from outside, so (b - a) x (c - a) points out) to ws.tris and returns
// their count; 0 when the points span less than 3-D (or, on inputs whose rounding breaks the
// hull's manifold structure, when a capacity would overflow).
HC_FN uint32_t hull_triangles(const float* in, uint32_t n, const HullCaps& caps, HullWs& ws) {
  if (n < 4) return 0;
  D3 lo = {1e300, 1e300, 1e300}, hi = {-1e300, -1e300, -1e300};
  for (uint32_t i = 0; i < n; ++i) {
    D3 p = D3{(double)in[3 * i], (double)in[3 * i + 1], (double)in[3 * i + 2]};
    ws.pts[i] = p;
    lo = D3{dmin(lo.x, p.x), dmin(lo.y, p.y), dmin(lo.z, p.z)};
    hi = D3{dmax(hi.x, p.x), dmax(hi.y, p.y), dmax(hi.z, p.z)};
  }
  D3 ext = dsub(hi, lo);
  double scale = dmax(ext.x, dmax(ext.y, ext.z));
  if (!(scale > 0.0) || !((scale - scale) == 0.0)) return 0;  // not positive, or not finite
  const double eps = 1e-10 * scale;  // plane-distance tolerance
  // initial tetrahedron: extreme x, farthest point, farthest from the line, farthest from the plane
  uint32_t i0 = 0;
  for (uint32_t i = 1; i < n; ++i)
    if (ws.pts[i].x < ws.pts[i0].x) i0 = i;
  const D3 p0 = ws.pts[i0];
  uint32_t i1 = i0;
  double best = -1.0;
  for (uint32_t i = 0; i < n; ++i) {
    D3 d = dsub(ws.pts[i], p0);
    double l = ddot(d, d);
    if (l > best) { best = l; i1 = i; }
  }
  if (best <= eps * eps) return 0;
  D3 e01 = dsub(ws.pts[i1], p0);
  uint32_t i2 = i0;
  best = -1.0;
  for (uint32_t i = 0; i < n; ++i) {
    D3 c = dcross(e01, dsub(ws.pts[i], p0));
    double l = ddot(c, c);
    if (l > best) { best = l; i2 = i; }
  }
  if (best <= (eps * scale) * (eps * scale)) return 0;
  D3 nrm = dcross(e01, dsub(ws.pts[i2], p0));
  double nn = sqrt(ddot(nrm, nrm));
  uint32_t i3 = i0;
  best = -1.0;
  double side = 0.0;
  for (uint32_t i = 0; i < n; ++i) {
    double d = ddot(nrm, dsub(ws.pts[i], p0)) / nn;
    if (fabs(d) > best) { best = fabs(d); i3 = i; side = d; }
  }
  if (best <= eps) return 0;

  uint32_t nf = 0;
  auto add_face = [&](uint32_t a, uint32_t b, uint32_t c) {
    HFace f;
    f.v[0] = a; f.v[1] = b; f.v[2] = c;
    const D3 pa = ws.pts[a];
    D3 fn = dcross(dsub(ws.pts[b], pa), dsub(ws.pts[c], pa));
    double l = sqrt(ddot(fn, fn));
    f.n = l > 0 ? D3{fn.x / l, fn.y / l, fn.z / l} : D3{0, 0, 0};
    f.off = ddot(f.n, pa);
    f.alive = 1;
    ws.faces[nf++] = f;
  };
  if (side > 0) {  // i3 above plane (i0, i1, i2): that face looks away from i3
    add_face(i0, i2, i1); add_face(i0, i1, i3); add_face(i1, i2, i3); add_face(i2, i0, i3);
  } else {
    add_face(i0, i1, i2); add_face(i0, i3, i1); add_face(i1, i3, i2); add_face(i2, i3, i0);
  }
  for (uint32_t pi = 0; pi < n; ++pi) {
    if (pi == i0 || pi == i1 || pi == i2 || pi == i3) continue;
    const D3 pp = ws.pts[pi];
    uint32_t nvis = 0;
    for (uint32_t f = 0; f < nf; ++f) {
      const HFace& F = ws.faces[f];
      if (F.alive && ddot(F.n, pp) - F.off > eps) ws.visible[nvis++] = f;
    }
    if (nvis == 0) continue;  // inside or on the hull
    // horizon: directed edges of visible faces whose reverse belongs to no visible face
    uint32_t nh = 0;
    for (uint32_t i = 0; i < nvis; ++i) {
      const HFace& F = ws.faces[ws.visible[i]];
      for (int k = 0; k < 3; ++k) {
        const uint32_t a = F.v[k], b = F.v[(k + 1) % 3];
        bool shared = false;
        for (uint32_t j = 0; j < nvis && !shared; ++j) {
          const HFace& G = ws.faces[ws.visible[j]];
          for (int kk = 0; kk < 3; ++kk)
            if (G.v[kk] == b && G.v[(kk + 1) % 3] == a) { shared = true; break; }
        }
        if (!shared) {
          if (nh >= caps.horizon) return 0;
          ws.horizon[2 * nh] = a;
          ws.horizon[2 * nh + 1] = b;
          ++nh;
        }
      }
    }
    for (uint32_t i = 0; i < nvis; ++i) ws.faces[ws.visible[i]].alive = 0;
    if (nf + nh > caps.faces) {  // drop dead faces, keeping the creation order of the live ones
      uint32_t k = 0;
      for (uint32_t f = 0; f < nf; ++f)
        if (ws.faces[f].alive) {
          if (k != f) ws.faces[k] = ws.faces[f];
          ++k;
        }
      nf = k;
      if (nf + nh > caps.faces) return 0;
    }
    for (uint32_t h = 0; h < nh; ++h) add_face(ws.horizon[2 * h], ws.horizon[2 * h + 1], pi);
  }
  uint32_t nt = 0;
  for (uint32_t f = 0; f < nf; ++f) {
    const HFace& F = ws.faces[f];
    if (!F.alive) continue;
    if (nt >= caps.tris) return 0;
    ws.tris[3 * nt] = F.v[0];
    ws.tris[3 * nt + 1] = F.v[1];
    ws.tris[3 * nt + 2] = F.v[2];
    ++nt;
  }
  return nt;
}

// The result of one cloud in ws: points (fpts[0..npts)), and with ok the topology of
// from_convex_mesh (frecs / face_edges / face_vertices, vertex_first / vertex_count / vertex_faces /
// vertex_edges, edges).
struct HullOut {
  uint32_t npts = 0, nfaces = 0;
  uint32_t nfentries = 0;  // face entries, those of dropped degenerate faces included
  uint32_t nventries = 0;  // vertex entries (from the kept faces)
  uint32_t nedges = 0;
  bool ok = false;
};

// utils::remove_unused_points (src/utils/cleanup.rs:6-34): swap_remove of the points no triangle uses.
HC_FN uint32_t remove_unused_points(uint32_t n, uint32_t nt, HullWs& ws) {
  for (uint32_t i = 0; i < n; ++i) { ws.used[i] = 0; ws.remap[i] = i; }
  for (uint32_t t = 0; t < 3 * nt; ++t) ws.used[ws.tris[t]] = 1;
  uint32_t size = n, i = 0;
  while (i != size) {
    if (!ws.used[i]) {
      ws.fpts[i] = ws.fpts[size - 1];  // swap_remove
      --size;
      ws.remap[size] = i;
      ws.used[i] = ws.used[size];
    } else {
      ++i;
    }
  }
  for (uint32_t t = 0; t < 3 * nt; ++t) ws.tris[t] = ws.remap[ws.tris[t]];
  return size;
}

// Edge id of the sorted pair (a, b) in the open-addressing table, or NONE; *slot = where it is or
// would go.
HC_FN uint32_t edge_lookup(const HullWs& ws, uint32_t hash_cap, uint64_t key, uint32_t* slot) {
  uint32_t h = (uint32_t)((key * 0x9E3779B97F4A7C15ull) >> 40) & (hash_cap - 1);
  for (uint32_t probe = 0; probe < hash_cap; ++probe) {
    const uint64_t k = ws.hkeys[h];
    if (k == key) { *slot = h; return ws.hvals[h]; }
    if (k == ~0ull) { *slot = h; return NONE; }
    h = (h + 1) & (hash_cap - 1);
  }
  *slot = NONE;
  return NONE;
}

// ConvexPolyhedron::from_convex_mesh (src/shape/convex_polyhedron.rs:390-639) over the npts points
// in ws.fpts and nt triangles in ws.tris. False for the reference's None.
HC_FN bool from_convex_mesh(uint32_t npts, uint32_t nt, const HullCaps& caps, HullWs& ws, HullOut* out) {
  const float eps = sqrtf(F32_EPS);
  if (npts + nt <= 2) return false;
  for (uint32_t h = 0; h < caps.hash; ++h) ws.hkeys[h] = ~0ull;
  uint32_t ne = 0;
  for (uint32_t t = 0; t < nt; ++t) {
    HTri T;
    const uint32_t idx[3] = {ws.tris[3 * t], ws.tris[3 * t + 1], ws.tris[3 * t + 2]};
    if (idx[0] == idx[1] || idx[0] == idx[2] || idx[1] == idx[2]) return false;
    for (int i1 = 0; i1 < 3; ++i1) {
      const int i2 = (i1 + 1) % 3;
      const uint32_t a = idx[i1] < idx[i2] ? idx[i1] : idx[i2], b = idx[i1] < idx[i2] ? idx[i2] : idx[i1];
      const uint64_t key = ((uint64_t)a << 32) | b;
      uint32_t slot;
      const uint32_t id = edge_lookup(ws, caps.hash, key, &slot);
      if (id != NONE) {
        HEdge& e = ws.edges[id];
        if (e.faces[1] == NONE) {
          T.e[i1] = id;
          e.faces[1] = t;
        } else {
          return false;  // t-junction
        }
      } else {
        if (slot == NONE || ne >= caps.edges) return false;
        ws.hkeys[slot] = key;
        ws.hvals[slot] = ne;
        T.e[i1] = ne;
        F3 d;
        const bool ok = unit_try_new(fsub(ws.fpts[idx[i2]], ws.fpts[idx[i1]]), F32_EPS, &d);
        HEdge e;
        e.v[0] = idx[i1]; e.v[1] = idx[i2];
        e.faces[0] = t; e.faces[1] = NONE;
        e.dir = ok ? d : F3{1.f, 0.f, 0.f};
        e.deleted = ok ? 0u : 1u;
        ws.edges[ne++] = e;
      }
    }
    F3 nrm;
    const F3 p0 = ws.fpts[idx[0]];
    const bool ok = unit_try_new(fcross(fsub(ws.fpts[idx[1]], p0), fsub(ws.fpts[idx[2]], p0)), F32_EPS, &nrm);
    for (int k = 0; k < 3; ++k) T.v[k] = idx[k];
    T.normal = ok ? nrm : F3{0.f, 0.f, 0.f};
    T.parent = NONE;
    ws.htris[t] = T;
  }
  for (uint32_t i = 0; i < ne; ++i) {
    HEdge& e = ws.edges[i];
    if (e.faces[0] >= nt || e.faces[1] >= nt) return false;
    if (fdot(ws.htris[e.faces[0]].normal, ws.htris[e.faces[1]].normal) > 1.0f - eps) e.deleted = 1;
  }
  uint32_t nfaces = 0, nentries = 0;
  for (uint32_t i = 0; i < nt; ++i) {
    if (ws.htris[i].parent != NONE) continue;
    for (int j1 = 0; j1 < 3; ++j1) {
      if (ws.edges[ws.htris[i].e[j1]].deleted) continue;
      const uint32_t new_face_id = nfaces;
      HFaceRec nf;
      nf.first = nentries;
      nf.num = 1;
      nf.normal = ws.htris[i].normal;
      ws.face_edges[nentries] = ws.htris[i].e[j1];
      ws.face_vertices[nentries] = ws.htris[i].v[j1];
      ++nentries;
      const uint32_t start_vertex = ws.htris[i].v[j1];
      uint32_t curr_tri = i;
      int curr_edge_id = (j1 + 1) % 3;
      uint32_t guard = 0;
      while (ws.htris[curr_tri].v[curr_edge_id] != start_vertex) {
        if (++guard > 4 * (nt + 3)) return false;  // malformed topology
        const uint32_t curr_edge = ws.htris[curr_tri].e[curr_edge_id];
        const uint32_t curr_vertex = ws.htris[curr_tri].v[curr_edge_id];
        ws.htris[curr_tri].parent = new_face_id;
        if (!ws.edges[curr_edge].deleted) {
          if (nentries >= caps.entries) return false;
          ws.face_edges[nentries] = curr_edge;
          ws.face_vertices[nentries] = curr_vertex;
          ++nentries;
          nf.num += 1;
          curr_edge_id = (curr_edge_id + 1) % 3;
        } else {
          const HEdge& e = ws.edges[curr_edge];
          curr_tri = e.faces[0] == curr_tri ? e.faces[1] : e.faces[0];
          int next = -1;
          for (int k = 0; k < 3; ++k)
            if (ws.htris[curr_tri].e[k] == curr_edge) { next = (k + 1) % 3; break; }
          curr_edge_id = next;
          if (curr_edge_id < 0 || ws.htris[curr_tri].v[curr_edge_id] != curr_vertex) return false;
        }
      }
      // Degenerate faces (an isolated edge left by rounding) are dropped, as in the reference;
      // their entries stay in the adjacency arrays there too.
      if (nf.num > 2) ws.frecs[nfaces++] = nf;
      break;
    }
  }
  for (uint32_t i = 0; i < ne; ++i) {
    HEdge& e = ws.edges[i];
    if (ws.htris[e.faces[0]].parent != NONE) e.faces[0] = ws.htris[e.faces[0]].parent;
    if (ws.htris[e.faces[1]].parent != NONE) e.faces[1] = ws.htris[e.faces[1]].parent;
  }
  for (uint32_t v = 0; v < npts; ++v) { ws.vertex_first[v] = 0; ws.vertex_count[v] = 0; }
  for (uint32_t f = 0; f < nfaces; ++f) {
    const HFaceRec r = ws.frecs[f];
    for (uint32_t k = r.first; k < r.first + r.num; ++k) ws.vertex_count[ws.face_vertices[k]] += 1;
  }
  uint32_t total = 0;
  for (uint32_t v = 0; v < npts; ++v) {
    ws.vertex_first[v] = total;
    total += ws.vertex_count[v];
    ws.vertex_count[v] = 0;
  }
  if (total > caps.entries) return false;
  for (uint32_t f = 0; f < nfaces; ++f) {
    const HFaceRec r = ws.frecs[f];
    for (uint32_t k = r.first; k < r.first + r.num; ++k) {
      const uint32_t v = ws.face_vertices[k];
      const uint32_t slot = ws.vertex_first[v] + ws.vertex_count[v];
      ws.vertex_faces[slot] = f;
      ws.vertex_edges[slot] = ws.face_edges[k];
      ws.vertex_count[v] += 1;
    }
  }
  out->npts = npts;
  out->nfaces = nfaces;
  out->nfentries = nentries;
  out->nventries = total;
  out->nedges = ne;
  out->ok = true;
  return true;
}

// ConvexPolyhedron::from_convex_hull for one cloud: the hull, then (if it has one) the cleanup and
// the topology; a cloud without a 3-D hull keeps all its points and no topology, one whose mesh
// from_convex_mesh rejects keeps the hull's points.
HC_FN HullOut build_one(const float* in, uint32_t n, const HullCaps& caps, HullWs& ws) {
  HullOut out;
  const uint32_t nt = hull_triangles(in, n, caps, ws);
  for (uint32_t i = 0; i < n; ++i) ws.fpts[i] = F3{in[3 * i], in[3 * i + 1], in[3 * i + 2]};
  if (nt == 0) {
    out.npts = n;
    return out;
  }
  const uint32_t m = remove_unused_points(n, nt, ws);
  if (!from_convex_mesh(m, nt, caps, ws, &out)) {
    out = HullOut();
    out.npts = m;
  }
  return out;
}

// Output arrays of a batch (the parrygpu_polyhedra layout) and the offsets of one hull in them.
struct PolyOut {
  float* points;
  uint32_t* hulls;
  float* face_normals;
  uint32_t *face_ranges, *face_vertices, *face_edges, *vertex_ranges, *vertex_faces, *vertex_edges;
  float* edge_dirs;
};

// Writes one hull's result (in ws, described by r) at offsets vp / fp / fe / ve / ep; null arrays
// are skipped.
HC_FN void emit(const HullWs& ws, const HullOut& r, uint64_t h, uint64_t vp, uint64_t fp, uint64_t fe, uint64_t ve, uint64_t ep,
                const PolyOut& o) {
  if (o.hulls) {
    uint32_t* rec = o.hulls + 8 * h;
    rec[0] = (uint32_t)vp; rec[1] = r.npts;
    rec[2] = (uint32_t)fp; rec[3] = r.ok ? r.nfaces : 0u;
    rec[4] = (uint32_t)ep; rec[5] = r.ok ? r.nedges : 0u;
    rec[6] = r.ok ? 1u : 0u; rec[7] = 0;
  }
  for (uint32_t i = 0; i < r.npts; ++i) {
    const F3 p = ws.fpts[i];
    if (o.points) { o.points[3 * (vp + i)] = p.x; o.points[3 * (vp + i) + 1] = p.y; o.points[3 * (vp + i) + 2] = p.z; }
    if (o.vertex_ranges) {
      o.vertex_ranges[2 * (vp + i)] = r.ok ? (uint32_t)(ve + ws.vertex_first[i]) : (uint32_t)ve;
      o.vertex_ranges[2 * (vp + i) + 1] = r.ok ? ws.vertex_count[i] : 0u;
    }
  }
  if (!r.ok) return;
  for (uint32_t f = 0; f < r.nfaces; ++f) {
    const HFaceRec fr = ws.frecs[f];
    if (o.face_normals) {
      o.face_normals[3 * (fp + f)] = fr.normal.x; o.face_normals[3 * (fp + f) + 1] = fr.normal.y;
      o.face_normals[3 * (fp + f) + 2] = fr.normal.z;
    }
    if (o.face_ranges) { o.face_ranges[2 * (fp + f)] = (uint32_t)(fe + fr.first); o.face_ranges[2 * (fp + f) + 1] = fr.num; }
  }
  // face entries: every entry the faces walked, dropped degenerate faces included (their entries
  // stay in the arrays, as in the reference)
  for (uint32_t k = 0; k < r.nfentries; ++k) {
    if (o.face_vertices) o.face_vertices[fe + k] = ws.face_vertices[k];
    if (o.face_edges) o.face_edges[fe + k] = ws.face_edges[k];
  }
  for (uint32_t k = 0; k < r.nventries; ++k) {
    if (o.vertex_faces) o.vertex_faces[ve + k] = ws.vertex_faces[k];
    if (o.vertex_edges) o.vertex_edges[ve + k] = ws.vertex_edges[k];
  }
  for (uint32_t e = 0; e < r.nedges; ++e) {
    const F3 d = ws.edges[e].dir;
    if (o.edge_dirs) { o.edge_dirs[3 * (ep + e)] = d.x; o.edge_dirs[3 * (ep + e) + 1] = d.y; o.edge_dirs[3 * (ep + e) + 2] = d.z; }
  }
}

}  // namespace hullcore
