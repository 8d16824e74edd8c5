// ConvexPolyhedron construction shared by the host builder (hull.cpp) and the GPU builder
// (hull_build.cu): one code path, so both produce the same bytes. parry builds a ConvexPolyhedron
// with ConvexPolyhedron::from_convex_hull(points) (src/shape/convex_polyhedron.rs:264-268, paths
// relative to the parry repository): a convex hull triangulation, then from_convex_mesh (:390-639),
// which merges coplanar triangles into faces and builds the vertex / edge / face adjacency.
//
//   hull_triangles: this library's own incremental hull in double precision. It produces the same
//     triangulation as any exact hull for points in general position, but not parry's quickhull
//     numbering (parry orders its initial simplex by a covariance eigen-decomposition); a caller
//     holding parry's own ConvexPolyhedron passes that topology through the C ABI instead. Like
//     parry's convex_hull it always returns a closed 2-manifold that transformation::
//     check_convex_hull accepts (src/transformation/convex_hull3/validation.rs:33-108): the faces a
//     new point sees are grown from the face it sees best through face adjacency, a point whose
//     seen region is not bounded by one simple cycle of edges (rounding on nearly coplanar faces) is
//     left out as lying on the hull, and a cloud whose points are coplanar gets the double-sided
//     polygon parry builds for it (src/transformation/convex_hull3/initial_mesh.rs).
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
#include <cstring>

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
  uint32_t alive;   // 0 dead, 1 live, 2 live and seen from the point being inserted
  uint32_t adj[3];  // the face across edge (v[k], v[k + 1])
  float off;        // unit normal and offset rounded to f32: a filter for the exact test
  float n[3];
  float tol;        // bound on the error of n . p - off (evaluated in f32) over the cloud
};

// ---- exact orientation ----------------------------------------------------------------------
// The hull decides visibility with the exact sign of orientation determinants (Shewchuk, "Adaptive
// Precision Floating-Point Arithmetic and Fast Robust Geometric Predicates", 1997): a rounded
// evaluation settles the sign when it clears an error bound, else an error-free expansion of the
// determinant decides. Coordinates are f32 values held in doubles, so their differences are exact
// (for coordinates within a factor 2^29 of one another, or zero) and the expansion gives the true
// sign. With exact signs the incremental hull stays convex and manifold on coplanar and repeated
// points, where tolerance-based tests fold faces over.
HC_FN void two_sum(double a, double b, double* s, double* e) {
  const double x = a + b, bv = x - a, av = x - bv;
  *s = x;
  *e = (a - av) + (b - bv);
}
HC_FN void two_prod(double a, double b, double* p, double* e) {
  const double x = a * b;
  *p = x;
  *e = fma(a, b, -x);
}
// Sign of the exact sum of x[0..m) (m <= 24): a nonoverlapping expansion grown one term at a time
// (Grow-Expansion), whose most significant nonzero component carries the sign.
HC_FN int exact_sum_sign(const double* x, int m) {
  double e[24];
  int ne = 0;
  for (int i = 0; i < m; ++i) {
    double q = x[i];
    for (int j = 0; j < ne; ++j) {
      double sum, err;
      two_sum(q, e[j], &sum, &err);
      e[j] = err;
      q = sum;
    }
    e[ne++] = q;
  }
  for (int j = ne - 1; j >= 0; --j)
    if (e[j] != 0.0) return e[j] > 0.0 ? 1 : -1;
  return 0;
}
// Sign of (x0 * y0 - x1 * y1), exactly.
HC_FN int diff_of_products_sign(double x0, double y0, double x1, double y1) {
  double t[4];
  two_prod(x0, y0, &t[0], &t[1]);
  two_prod(-x1, y1, &t[2], &t[3]);
  return exact_sum_sign(t, 4);
}
// Sign of ((b - a) x (c - a)) . (p - a): positive when p lies on the side the right-handed normal of
// triangle (a, b, c) points to.
HC_FN int orient3d_sign(D3 a, D3 b, D3 c, D3 p) {
  const D3 u = dsub(b, a), v = dsub(c, a), w = dsub(p, a);
  const double m1 = v.y * w.z - v.z * w.y, m2 = v.z * w.x - v.x * w.z, m3 = v.x * w.y - v.y * w.x;
  const double det = u.x * m1 + u.y * m2 + u.z * m3;
  const double perm = fabs(u.x) * (fabs(v.y * w.z) + fabs(v.z * w.y)) + fabs(u.y) * (fabs(v.z * w.x) + fabs(v.x * w.z)) +
                      fabs(u.z) * (fabs(v.x * w.y) + fabs(v.y * w.x));
  const double bound = 1e-15 * perm;  // above the rounding of det (7.8e-16 x perm)
  if (det > bound) return 1;
  if (det < -bound) return -1;
  double t[24];
  int k = 0;
  auto triple = [&](double x, double y, double z, bool neg) {
    double p, pe, q0, q1, r0, r1;
    two_prod(x, y, &p, &pe);
    two_prod(p, z, &q0, &q1);
    two_prod(pe, z, &r0, &r1);
    const double sg = neg ? -1.0 : 1.0;
    t[k++] = sg * q0; t[k++] = sg * q1; t[k++] = sg * r0; t[k++] = sg * r1;
  };
  triple(u.x, v.y, w.z, false); triple(u.x, v.z, w.y, true);
  triple(u.y, v.z, w.x, false); triple(u.y, v.x, w.z, true);
  triple(u.z, v.x, w.y, false); triple(u.z, v.y, w.x, true);
  return exact_sum_sign(t, 24);
}
// True when (b - a) x (c - a) is exactly the zero vector (a, b, c collinear or repeated).
HC_FN bool collinear_exact(D3 a, D3 b, D3 c) {
  const D3 u = dsub(b, a), v = dsub(c, a);
  return diff_of_products_sign(u.y, v.z, u.z, v.y) == 0 && diff_of_products_sign(u.z, v.x, u.x, v.z) == 0 &&
         diff_of_products_sign(u.x, v.y, u.y, v.x) == 0;
}

// Words per horizon entry: edge start, edge end, the unseen face across the edge.
constexpr uint32_t HORIZON_WORDS = 3;

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
  Span<uint32_t> horizon;    // HORIZON_WORDS x caps.horizon
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

// Double-sided polygon of a coplanar cloud (what parry's convex_hull returns for one): the 2-D hull
// of the points on the two coordinates other than the dominant axis of the plane's normal (an exact
// projection), by Andrew's monotone chain with exact turn signs (collinear points dropped),
// triangulated as a fan from its first vertex on one side and a fan from its second vertex on the
// other side, so that no diagonal is shared by the two sides. Returns the triangle count (0 when
// fewer than 3 points are extreme).
HC_FN uint32_t planar_triangles(uint32_t n, uint32_t i0, uint32_t i1, uint32_t i2, const HullCaps& caps, HullWs& ws) {
  const D3 p0 = ws.pts[i0];
  const D3 nrm = dcross(dsub(ws.pts[i1], p0), dsub(ws.pts[i2], p0));
  const double ax = fabs(nrm.x), ay = fabs(nrm.y), az = fabs(nrm.z);
  const int drop = (ax >= ay && ax >= az) ? 0 : (ay >= az ? 1 : 2);
  auto X = [&](uint32_t i) { const D3 p = ws.pts[i]; return drop == 0 ? p.y : (drop == 1 ? p.z : p.x); };
  auto Y = [&](uint32_t i) { const D3 p = ws.pts[i]; return drop == 0 ? p.z : (drop == 1 ? p.x : p.y); };
  // point indices sorted by (X, Y) in ws.remap with a heap sort (repeated points: the first kept)
  uint32_t m = 0;
  for (uint32_t i = 0; i < n; ++i)
    if (!ws.remap[i]) ws.used[m++] = i;
  for (uint32_t i = 0; i < m; ++i) ws.remap[i] = ws.used[i];
  auto less = [&](uint32_t a, uint32_t b) {
    return X(a) < X(b) || (X(a) == X(b) && (Y(a) < Y(b) || (Y(a) == Y(b) && a < b)));
  };
  auto sift = [&](uint32_t root, uint32_t end) {
    while (2 * root + 1 < end) {
      uint32_t child = 2 * root + 1;
      if (child + 1 < end && less(ws.remap[child], ws.remap[child + 1])) ++child;
      if (!less(ws.remap[root], ws.remap[child])) return;
      const uint32_t t = ws.remap[root]; ws.remap[root] = ws.remap[child]; ws.remap[child] = t;
      root = child;
    }
  };
  for (uint32_t i = m / 2; i-- > 0;) sift(i, m);
  for (uint32_t end = m; end-- > 1;) {
    const uint32_t t = ws.remap[0]; ws.remap[0] = ws.remap[end]; ws.remap[end] = t;
    sift(0, end);
  }
  auto left_turn = [&](uint32_t o, uint32_t a, uint32_t b) {  // o -> a -> b counter-clockwise in (X, Y)
    return diff_of_products_sign(X(a) - X(o), Y(b) - Y(o), Y(a) - Y(o), X(b) - X(o)) > 0;
  };
  // the chain, counter-clockwise in (X, Y), in ws.visible
  uint32_t k = 0;
  for (uint32_t i = 0; i < m; ++i) {
    const uint32_t p = ws.remap[i];
    while (k >= 2 && !left_turn(ws.visible[k - 2], ws.visible[k - 1], p)) --k;
    ws.visible[k++] = p;
  }
  for (uint32_t i = m - 1, lower = k + 1; i-- > 0;) {
    const uint32_t p = ws.remap[i];
    while (k >= lower && !left_turn(ws.visible[k - 2], ws.visible[k - 1], p)) --k;
    ws.visible[k++] = p;
  }
  const uint32_t h = k - 1;  // the last point repeats the first
  if (h < 3 || 2 * (h - 2) > caps.tris) return 0;
  uint32_t nt = 0;
  for (uint32_t i = 1; i + 1 < h; ++i) {  // one side: fan from the first vertex
    ws.tris[3 * nt] = ws.visible[0]; ws.tris[3 * nt + 1] = ws.visible[i]; ws.tris[3 * nt + 2] = ws.visible[i + 1];
    ++nt;
  }
  for (uint32_t j = 2; j < h; ++j) {  // other side: fan from the second vertex, reversed
    ws.tris[3 * nt] = ws.visible[1]; ws.tris[3 * nt + 1] = ws.visible[(j + 1) % h]; ws.tris[3 * nt + 2] = ws.visible[j];
    ++nt;
  }
  return nt;
}

// Incremental convex hull of pts[0..n) (x, y, z floats) with exact visibility. Writes the
// outward-oriented triangles (counter-clockwise seen from outside, so (b - a) x (c - a) points out)
// to ws.tris and returns their count; a coplanar cloud gets its double-sided polygon; 0 when the
// points span less than 2-D.
HC_FN uint32_t hull_triangles(const float* in, uint32_t n, const HullCaps& caps, HullWs& ws) {
  if (n < 3) return 0;
  D3 lo = {1e300, 1e300, 1e300}, hi = {-1e300, -1e300, -1e300};
  double rmax = 0.0;
  for (uint32_t i = 0; i < n; ++i) {
    D3 p = D3{(double)in[3 * i], (double)in[3 * i + 1], (double)in[3 * i + 2]};
    ws.pts[i] = p;
    lo = D3{dmin(lo.x, p.x), dmin(lo.y, p.y), dmin(lo.z, p.z)};
    hi = D3{dmax(hi.x, p.x), dmax(hi.y, p.y), dmax(hi.z, p.z)};
    rmax = dmax(rmax, dmax(fabs(p.x), dmax(fabs(p.y), fabs(p.z))));
  }
  D3 ext = dsub(hi, lo);
  double scale = dmax(ext.x, dmax(ext.y, ext.z));
  if (!(scale > 0.0) || !((scale - scale) == 0.0)) return 0;  // all points equal, or not finite
  // a point equal to an earlier one (f32 ==) never enters the hull: ws.remap[i] = 1 marks it, found
  // through the open-addressing table (free until from_convex_mesh)
  for (uint32_t h = 0; h < caps.hash; ++h) ws.hkeys[h] = ~0ull;
  for (uint32_t i = 0; i < n; ++i) {
    const float* q = in + 3 * i;
    uint64_t key = 0x9E3779B97F4A7C15ull;
    for (int k = 0; k < 3; ++k) {
      uint32_t b;
      const float c = q[k] == 0.0f ? 0.0f : q[k];  // -0 == +0
      memcpy(&b, &c, 4);
      key = (key ^ b) * 0xBF58476D1CE4E5B9ull;
      key ^= key >> 31;
    }
    if (key == ~0ull) key = 0;
    uint32_t h = (uint32_t)(key >> 40) & (caps.hash - 1);
    ws.remap[i] = 0;
    while (ws.hkeys[h] != ~0ull) {
      const float* o = in + 3 * ws.hvals[h];
      if (ws.hkeys[h] == key && o[0] == q[0] && o[1] == q[1] && o[2] == q[2]) { ws.remap[i] = 1; break; }
      h = (h + 1) & (caps.hash - 1);
    }
    if (!ws.remap[i]) { ws.hkeys[h] = key; ws.hvals[h] = i; }
  }
  // initial tetrahedron: extreme x, farthest point, farthest from the line, farthest from the plane
  // (each an exact decision: the largest rounded measure, else the first point that is exactly off)
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
  D3 e01 = dsub(ws.pts[i1], p0);
  uint32_t i2 = i0;
  best = -1.0;
  for (uint32_t i = 0; i < n; ++i) {
    D3 c = dcross(e01, dsub(ws.pts[i], p0));
    double l = ddot(c, c);
    if (l > best) { best = l; i2 = i; }
  }
  if (collinear_exact(p0, ws.pts[i1], ws.pts[i2])) {
    i2 = NONE;
    for (uint32_t i = 0; i < n && i2 == NONE; ++i)
      if (!collinear_exact(p0, ws.pts[i1], ws.pts[i])) i2 = i;
    if (i2 == NONE) return 0;  // collinear cloud
  }
  D3 nrm = dcross(e01, dsub(ws.pts[i2], p0));
  uint32_t i3 = i0;
  best = -1.0;
  for (uint32_t i = 0; i < n; ++i) {
    double d = fabs(ddot(nrm, dsub(ws.pts[i], p0)));
    if (d > best) { best = d; i3 = i; }
  }
  int side = orient3d_sign(p0, ws.pts[i1], ws.pts[i2], ws.pts[i3]);
  for (uint32_t i = 0; i < n && side == 0; ++i) {
    side = orient3d_sign(p0, ws.pts[i1], ws.pts[i2], ws.pts[i]);
    i3 = i;
  }
  if (side == 0) return planar_triangles(n, i0, i1, i2, caps, ws);

  uint32_t nf = 0;
  auto add_face = [&](uint32_t a, uint32_t b, uint32_t c, uint32_t f0, uint32_t f1, uint32_t f2) {
    HFace f;
    f.v[0] = a; f.v[1] = b; f.v[2] = c;
    f.adj[0] = f0; f.adj[1] = f1; f.adj[2] = f2;
    const D3 pa = ws.pts[a], u = dsub(ws.pts[b], pa), v = dsub(ws.pts[c], pa);
    D3 fn = dcross(u, v);
    double l = sqrt(ddot(fn, fn));
    const D3 nd = l > 0 ? D3{fn.x / l, fn.y / l, fn.z / l} : D3{0, 0, 0};
    f.n[0] = (float)nd.x; f.n[1] = (float)nd.y; f.n[2] = (float)nd.z;
    f.off = (float)ddot(nd, pa);
    // the f32 evaluation (products, sums, and the rounding of the normal and offset to f32: about
    // 9 f32 epsilons of the cloud's radius) plus the normal's direction error in double (relative to
    // how thin the face is) times the cloud's extent, with margin; infinite for a degenerate face
    const double cond = l > 0 ? sqrt(ddot(u, u) * ddot(v, v)) / l : 1e300;
    f.tol = (float)(1e-6 * (rmax + scale * (1.0 + cond)));
    f.alive = 1;
    ws.faces[nf++] = f;
  };
  // the f32 filter's signed distance of point pf from face F's plane
  auto dist = [](const HFace& F, const F3& pf) { return ((F.n[0] * pf.x + F.n[1] * pf.y) + F.n[2] * pf.z) - F.off; };
  // whether face F sees p (p strictly above its plane), exactly (pf: p's f32 coordinates)
  auto sees = [&](const HFace& F, const F3& pf, const D3& p) {
    const float d = dist(F, pf);
    if (d > F.tol) return true;
    if (d < -F.tol) return false;
    return orient3d_sign(ws.pts[F.v[0]], ws.pts[F.v[1]], ws.pts[F.v[2]], p) > 0;
  };
  // faces 0-3 with their neighbours: face k's edge j borders the face listed at [k][j]
  if (side > 0) {  // i3 above plane (i0, i1, i2): that face looks away from i3
    add_face(i0, i2, i1, 3, 2, 1); add_face(i0, i1, i3, 0, 2, 3); add_face(i1, i2, i3, 0, 3, 1); add_face(i2, i0, i3, 0, 1, 2);
  } else {
    add_face(i0, i1, i2, 1, 2, 3); add_face(i0, i3, i1, 3, 2, 0); add_face(i1, i3, i2, 1, 3, 0); add_face(i2, i3, i0, 2, 1, 0);
  }
  for (uint32_t pi = 0; pi < n; ++pi) {
    if (pi == i0 || pi == i1 || pi == i2 || pi == i3 || ws.remap[pi]) continue;
    if (nf + caps.horizon > caps.faces) {  // drop dead faces (creation order kept), renumbering links
      uint32_t k = 0;
      for (uint32_t f = 0; f < nf; ++f) ws.visible[f] = ws.faces[f].alive ? k++ : NONE;
      k = 0;
      for (uint32_t f = 0; f < nf; ++f)
        if (ws.faces[f].alive) {
          HFace F = ws.faces[f];
          for (int j = 0; j < 3; ++j) F.adj[j] = ws.visible[F.adj[j]];
          ws.faces[k++] = F;
        }
      nf = k;
      if (nf + caps.horizon > caps.faces) return 0;  // more live faces than a closed hull of n points has
    }
    const D3 pp = ws.pts[pi];
    const F3 pf = F3{in[3 * pi], in[3 * pi + 1], in[3 * pi + 2]};
    // the face that sees pp at the largest (filter) distance, then every face that sees pp connected
    // to it (for a convex hull and an exact test, that is every face that sees pp)
    uint32_t seed = NONE;
    float bestd = 0.0f;
    for (uint32_t f = 0; f < nf; ++f) {
      const HFace& F = ws.faces[f];
      if (!F.alive) continue;
      const float d = dist(F, pf);  // NaN (overflowing coordinates): left to the exact test
      if (!(d < -F.tol) && (seed == NONE || d > bestd) && sees(F, pf, pp)) { bestd = d; seed = f; }
    }
    if (seed == NONE) continue;  // inside or on the hull
    uint32_t nvis = 0;
    ws.visible[nvis++] = seed;
    ws.faces[seed].alive = 2;
    for (uint32_t i = 0; i < nvis; ++i) {
      for (int j = 0; j < 3; ++j) {
        const uint32_t g = ws.faces[ws.visible[i]].adj[j];
        HFace& G = ws.faces[g];
        if (G.alive == 1 && sees(G, pf, pp)) {
          G.alive = 2;
          ws.visible[nvis++] = g;
        }
      }
    }
    // horizon: edges of seen faces whose other face is unseen, chained into one cycle
    uint32_t nh = 0;
    bool simple = true;
    for (uint32_t i = 0; i < nvis && simple; ++i) {
      const HFace& F = ws.faces[ws.visible[i]];
      for (int j = 0; j < 3; ++j) {
        if (ws.faces[F.adj[j]].alive == 2) continue;
        if (nh >= caps.horizon) { simple = false; break; }
        ws.horizon[HORIZON_WORDS * nh] = F.v[j];
        ws.horizon[HORIZON_WORDS * nh + 1] = F.v[(j + 1) % 3];
        ws.horizon[HORIZON_WORDS * nh + 2] = F.adj[j];
        ++nh;
      }
    }
    for (uint32_t h = 0; h + 1 < nh && simple; ++h) {
      uint32_t next = NONE;
      for (uint32_t g = h + 1; g < nh; ++g)
        if (ws.horizon[HORIZON_WORDS * g] == ws.horizon[HORIZON_WORDS * h + 1]) { next = g; break; }
      if (next == NONE) { simple = false; break; }
      for (uint32_t w = 0; w < HORIZON_WORDS; ++w) {
        const uint32_t t = ws.horizon[HORIZON_WORDS * (h + 1) + w];
        ws.horizon[HORIZON_WORDS * (h + 1) + w] = ws.horizon[HORIZON_WORDS * next + w];
        ws.horizon[HORIZON_WORDS * next + w] = t;
      }
    }
    if (simple && (nh < 3 || ws.horizon[HORIZON_WORDS * (nh - 1) + 1] != ws.horizon[0])) simple = false;
    if (simple) {  // one cycle through distinct vertices (no pinch)
      for (uint32_t h = 0; h < nh; ++h) ws.used[ws.horizon[HORIZON_WORDS * h]] = 0;
      for (uint32_t h = 0; h < nh && simple; ++h) {
        uint32_t& mark = ws.used[ws.horizon[HORIZON_WORDS * h]];
        if (mark) simple = false;
        mark = 1;
      }
    }
    if (!simple) {  // cannot happen with exact signs on a convex hull; kept as a guard (pp left out)
      for (uint32_t i = 0; i < nvis; ++i) ws.faces[ws.visible[i]].alive = 1;
      continue;
    }
    for (uint32_t i = 0; i < nvis; ++i) ws.faces[ws.visible[i]].alive = 0;
    const uint32_t first = nf;
    for (uint32_t h = 0; h < nh; ++h) {
      const uint32_t a = ws.horizon[HORIZON_WORDS * h], b = ws.horizon[HORIZON_WORDS * h + 1];
      const uint32_t out = ws.horizon[HORIZON_WORDS * h + 2];
      add_face(a, b, pi, out, first + (h + 1) % nh, first + (h + nh - 1) % nh);
      HFace& O = ws.faces[out];
      for (int j = 0; j < 3; ++j)
        if (O.v[j] == b && O.v[(j + 1) % 3] == a) O.adj[j] = first + h;
    }
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
  uint32_t ntris = 0;  // triangles of the hull (transformation::convex_hull's indices), in ws.tris
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
  out.ntris = nt;
  return out;
}

// Output arrays of a batch (the parrygpu_polyhedra layout) and the offsets of one hull in them.
struct PolyOut {
  float* points;
  uint32_t* hulls;
  float* face_normals;
  uint32_t *face_ranges, *face_vertices, *face_edges, *vertex_ranges, *vertex_faces, *vertex_edges;
  float* edge_dirs;
  uint32_t* triangles;  // 3 hull-local vertex ids per triangle (may be null)
};

// Writes one hull's result (in ws, described by r) at offsets vp / fp / fe / ve / ep / tp (tp in
// triangles); null arrays are skipped.
HC_FN void emit(const HullWs& ws, const HullOut& r, uint64_t h, uint64_t vp, uint64_t fp, uint64_t fe, uint64_t ve, uint64_t ep,
                const PolyOut& o, uint64_t tp = 0) {
  if (o.triangles)
    for (uint32_t k = 0; k < 3 * r.ntris; ++k) o.triangles[3 * tp + k] = ws.tris[k];
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
