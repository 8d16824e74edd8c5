// The GJK Voronoi simplex held in registers, for kernels that inline one GJK loop.
//
// gjk_device.cuh's Simplex is an array indexed at run time (vertex swaps by the projected feature's
// id, appends at index dim), so it lives in local memory, and the out-of-line projection shares one
// copy between kernels. RegSimplex names its four vertices and moves them with constant indices, so
// a kernel that inlines the loop keeps the whole simplex in registers. Every value is computed as
// simplex_reset / simplex_add / simplex_project_origin_and_reduce / gjk_result compute it (the
// projections are the same inline bodies), so a loop written over RegSimplex gives the same bits.
//
// WIT = false keeps only the vertex positions (a ray cast needs nothing else); WIT = true also
// carries each vertex's two support points and the barycentric coordinates of the current and of
// the previous projection (VoronoiSimplex::proj / prev_proj), for the witness points.
#pragma once
#include "gjk_device.cuh"

namespace pg {

template <bool WIT>
struct RegSimplex {
  V3 p0, p1, p2, p3;          // CSO points
  V3 a0, a1, a2, a3;          // support points on shape 1 (WIT)
  V3 b0, b1, b2, b3;          // support points on shape 2 (WIT)
  float c0, c1, c2;           // proj (WIT)
  float q0, q1, q2;           // prev_proj (WIT)
  int dim, prev_dim;
};

template <bool W>
__device__ __forceinline__ CSO rs_get(const RegSimplex<W>& s, int i) {
  if (i == 0) return CSO{s.p0, s.a0, s.b0};
  if (i == 1) return CSO{s.p1, s.a1, s.b1};
  if (i == 2) return CSO{s.p2, s.a2, s.b2};
  return CSO{s.p3, s.a3, s.b3};
}

// Vertex slot `i` (a constant at every call site) <- c.
template <bool W>
__device__ __forceinline__ void rs_put(RegSimplex<W>& s, int i, const CSO& c) {
  if (i == 0) { s.p0 = c.p; if constexpr (W) { s.a0 = c.o1; s.b0 = c.o2; } }
  else if (i == 1) { s.p1 = c.p; if constexpr (W) { s.a1 = c.o1; s.b1 = c.o2; } }
  else if (i == 2) { s.p2 = c.p; if constexpr (W) { s.a2 = c.o1; s.b2 = c.o2; } }
  else { s.p3 = c.p; if constexpr (W) { s.a3 = c.o1; s.b3 = c.o2; } }
}

// Barycentric coordinates of a face / of an edge (the third coordinate keeps its value, as the
// array form leaves proj[2] when it reduces to an edge).
template <bool W>
__device__ __forceinline__ void rs_proj3(RegSimplex<W>& s, float x, float y, float z) {
  if constexpr (W) { s.c0 = x; s.c1 = y; s.c2 = z; }
}
template <bool W>
__device__ __forceinline__ void rs_proj2(RegSimplex<W>& s, float x, float y) {
  if constexpr (W) { s.c0 = x; s.c1 = y; }
}

// VoronoiSimplex::reset.
template <bool W>
__device__ __forceinline__ void rs_reset(RegSimplex<W>& s, const CSO& c) {
  s.dim = 0;
  s.prev_dim = 0;
  rs_put(s, 0, c);
  if constexpr (W) { s.c0 = s.c1 = s.c2 = 0.0f; s.q0 = s.q1 = s.q2 = 0.0f; }
}

// VoronoiSimplex::add_point: refused (vertices unchanged) when the point is affinely dependent; the
// previous projection is saved either way.
template <bool W>
__device__ __forceinline__ bool rs_add(RegSimplex<W>& s, const CSO& pt) {
  s.prev_dim = s.dim;
  if constexpr (W) { s.q0 = s.c0; s.q1 = s.c1; s.q2 = s.c2; }
  if (s.dim == 0) {
    V3 d = s.p0 - pt.p;
    if (dot(d, d) < GJK_EPS_TOL) return false;
  } else if (s.dim == 1) {
    V3 ab = s.p1 - s.p0, ac = pt.p - s.p0;
    V3 c = cross(ab, ac);
    if (dot(c, c) < GJK_EPS_TOL) return false;
  } else if (s.dim == 2) {
    V3 ab = s.p1 - s.p0, ac = s.p2 - s.p0, ap = pt.p - s.p0;
    V3 n = normalize(cross(ab, ac));
    if (fabsf(dot(n, ap)) < GJK_EPS_TOL) return false;
  }
  s.dim += 1;
  if (s.dim == 1) rs_put(s, 1, pt);
  else if (s.dim == 2) rs_put(s, 2, pt);
  else rs_put(s, 3, pt);
  return true;
}

// Every vertex position of the simplex moved by `d` (the ray cast's origin shift).
template <bool W>
__device__ __forceinline__ void rs_translate(RegSimplex<W>& s, V3 d) {
  s.p0 = s.p0 + d;
  if (s.dim >= 1) s.p1 = s.p1 + d;
  if (s.dim >= 2) s.p2 = s.p2 + d;
  if (s.dim >= 3) s.p3 = s.p3 + d;
}

// VoronoiSimplex::project_origin_and_reduce: the projection of the origin; the vertices of the
// feature that holds it move to the front in the order the array form's swaps leave them, with
// their barycentric coordinates, and dim shrinks to that feature's. (Vertices past dim are not
// kept: nothing reads them before an add overwrites them.)
template <bool W>
__device__ __forceinline__ V3 rs_project_origin_and_reduce(RegSimplex<W>& s) {
  const V3 o = v3(0.f, 0.f, 0.f);
  Loc loc;
  if (s.dim == 0) {
    if constexpr (W) s.c0 = 1.0f;
    return s.p0;
  }
  if (s.dim == 1) {
    V3 p = project_segment(s.p0, s.p1, o, &loc);
    if (loc.kind == LOC_VERTEX) {
      if (loc.id != 0) rs_put(s, 0, rs_get(s, 1));
      if constexpr (W) s.c0 = 1.0f;
      s.dim = 0;
    } else {
      rs_proj2(s, loc.bc[0], loc.bc[1]);
    }
    return p;
  }
  if (s.dim == 2) {
    V3 p = project_triangle_inl(s.p0, s.p1, s.p2, o, &loc);
    if (loc.kind == LOC_VERTEX) {
      rs_put(s, 0, rs_get(s, loc.id));
      if constexpr (W) s.c0 = 1.0f;
      s.dim = 0;
    } else if (loc.kind == LOC_EDGE) {
      if (loc.id == 0) {
        rs_proj2(s, loc.bc[0], loc.bc[1]);
      } else if (loc.id == 1) {  // swap(0, 2)
        rs_put(s, 0, rs_get(s, 2));
        rs_proj2(s, loc.bc[1], loc.bc[0]);
      } else {  // swap(1, 2)
        rs_put(s, 1, rs_get(s, 2));
        rs_proj2(s, loc.bc[0], loc.bc[1]);
      }
      s.dim = 1;
    } else if (loc.kind == LOC_FACE) {
      rs_proj3(s, loc.bc[0], loc.bc[1], loc.bc[2]);
    }
    return p;
  }
  V3 p = project_tetrahedron_inl(s.p0, s.p1, s.p2, s.p3, o, &loc);
  if (loc.kind == LOC_VERTEX) {
    rs_put(s, 0, rs_get(s, loc.id));
    if constexpr (W) s.c0 = 1.0f;
    s.dim = 0;
  } else if (loc.kind == LOC_EDGE) {
    const CSO c = rs_get(s, 2), d = rs_get(s, 3);
    switch (loc.id) {
      case 1: rs_put(s, 1, c); break;                     // swap(1, 2)
      case 2: rs_put(s, 1, d); break;                     // swap(1, 3)
      case 3: rs_put(s, 0, c); break;                     // swap(0, 2)
      case 4: rs_put(s, 0, d); break;                     // swap(0, 3)
      case 5: rs_put(s, 0, c); rs_put(s, 1, d); break;    // swap(0, 2), swap(1, 3)
      default: break;
    }
    if (loc.id == 3 || loc.id == 4) rs_proj2(s, loc.bc[1], loc.bc[0]);
    else rs_proj2(s, loc.bc[0], loc.bc[1]);
    s.dim = 1;
  } else if (loc.kind == LOC_FACE) {
    const CSO d = rs_get(s, 3);
    if (loc.id == 0) rs_proj3(s, loc.bc[0], loc.bc[1], loc.bc[2]);
    else if (loc.id == 1) { rs_put(s, 2, d); rs_proj3(s, loc.bc[0], loc.bc[1], loc.bc[2]); }
    else if (loc.id == 2) { rs_put(s, 1, d); rs_proj3(s, loc.bc[0], loc.bc[2], loc.bc[1]); }
    else { rs_put(s, 0, d); rs_proj3(s, loc.bc[2], loc.bc[0], loc.bc[1]); }
    s.dim = 2;
  }
  return p;
}

// gjk_result: the witness points of the current projection, or (prev) of the projection before the
// last added point. `prev` is only asked for right after an add that reached a tetrahedron and a
// projection that kept it (no vertex moved), so the previous vertices are the first prev_dim + 1.
__device__ __forceinline__ void rs_witness(const RegSimplex<true>& s, bool prev, V3* w1, V3* w2) {
  const int n = prev ? s.prev_dim : s.dim;
  const float k0 = prev ? s.q0 : s.c0, k1 = prev ? s.q1 : s.c1, k2 = prev ? s.q2 : s.c2;
  V3 a = v3(0.f, 0.f, 0.f), b = v3(0.f, 0.f, 0.f);
  a = a + s.a0 * k0;
  b = b + s.b0 * k0;
  if (n >= 1) { a = a + s.a1 * k1; b = b + s.b1 * k1; }
  if (n >= 2) { a = a + s.a2 * k2; b = b + s.b2 * k2; }  // n <= 2: a reduced simplex or the one before the last add
  *w1 = a;
  *w2 = b;
}

}  // namespace pg
