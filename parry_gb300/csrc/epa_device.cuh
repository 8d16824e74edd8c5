// Device-side EPA (src/query/epa/epa3.rs:17-675, path relative to the parry repository).
//
// The polytope lives in a per-thread workspace slot in global memory, one contiguous block of
// words per slot: the lanes of a warp work on different faces and heap positions at any moment,
// so records are laid out for one lane's accesses. A vertex's CSO point is one 16-byte word group
// (read with one vector load); its two witness points, used only for the final closest points,
// sit in a separate array; a face is 8 words, one 32-byte sector. Fixed capacities replace the
// reference's Vecs; exceeding one aborts the pair and raises a capacity error. Vertices are bounded
// by the 100 expansions (at most 105); faces are not: observed maxima over 1,048,576 pairs are 243
// faces (8-256-vertex hulls) and 512 (hulls mixed with cuboids, where flat contacts run all 100
// expansions), so the face capacity is 1,024, with silhouettes of at most 13 edges. The reference's
// recursive silhouette walk becomes an explicit stack visiting faces in the same order, and its
// BinaryHeap is restated with the same sift operations so that ties between face distances pop
// in the same order.
#pragma once
#include "gjk_device.cuh"

namespace pg {

// Fixed capacities and word offsets of one polytope workspace. FW = words per face record: 8 (one
// 32-byte sector, for per-thread workspaces in global memory) or 6 (the record without padding,
// for workspaces in shared memory).
template <int MV, int MF, int MS, int MSTK, int FW = 8>
struct EpaLayout {
  static constexpr int MAX_VERTS = MV, MAX_FACES = MF, MAX_SIL = MS, STACK = MSTK, FACE_WORDS = FW;
  static constexpr int W_VP = 0;                          // 4 words per vertex: CSO point (x, y, z, -)
  static constexpr int W_VO = W_VP + 4 * MV;              // 6 words per vertex: witness points orig1, orig2
  static constexpr int W_FACES = W_VO + 6 * MV;           // FW words per face
  // the heap (MF entries of 2 words) lives in the thread's local memory up to 1,024 entries, else at
  // the end of the workspace; the silhouette walk's stack and edge list (MSTK, MS) in local memory
  static constexpr bool HEAP_LOCAL = MF <= 1024;
  static constexpr int W_HEAP = W_FACES + FW * MF;
  static constexpr int WORDS = W_HEAP + (HEAP_LOCAL ? 0 : 2 * MF);  // words per workspace
  static_assert(FW != 8 || (W_FACES % 8 == 0 && WORDS % 8 == 0), "faces and slots start on 32-byte boundaries");
  static_assert(FW == 8 || FW == 6, "face records of 8 or 6 words");
};
// Per-thread workspaces in global memory.
using EpaGlobalLayout = EpaLayout<128, 1024, 64, 256>;

constexpr int EPA_MAX_VERTS = EpaGlobalLayout::MAX_VERTS;
constexpr int EPA_MAX_FACES = EpaGlobalLayout::MAX_FACES;
constexpr int EPA_WORDS = EpaGlobalLayout::WORDS;                     // words per slot
constexpr size_t EPA_SLOT_BYTES = (size_t)EPA_WORDS * 4;             // bytes per slot

// A workspace view over one slot (word i at base[i]; base 32-byte aligned).
template <class L>
struct EpaWsT {
  using Layout = L;
  uint32_t* base;
  __device__ __forceinline__ uint32_t& w(int i) const { return base[i]; }
  __device__ __forceinline__ float& f(int i) const { return reinterpret_cast<float&>(base[i]); }
  // vertices
  __device__ __forceinline__ void set_vert(int v, const CSO& c) const {
    *reinterpret_cast<float4*>(base + L::W_VP + 4 * v) = make_float4(c.p.x, c.p.y, c.p.z, 0.0f);
    float2* o = reinterpret_cast<float2*>(base + L::W_VO + 6 * v);  // 8-byte aligned: W_VO and 6 v are even
    o[0] = make_float2(c.o1.x, c.o1.y);
    o[1] = make_float2(c.o1.z, c.o2.x);
    o[2] = make_float2(c.o2.y, c.o2.z);
  }
  __device__ __forceinline__ V3 vp(int v) const {
    float4 q = *reinterpret_cast<const float4*>(base + L::W_VP + 4 * v);
    return v3(q.x, q.y, q.z);
  }
  __device__ __forceinline__ V3 vo1(int v) const { int o = L::W_VO + 6 * v; return v3(f(o), f(o + 1), f(o + 2)); }
  __device__ __forceinline__ V3 vo2(int v) const { int o = L::W_VO + 6 * v + 3; return v3(f(o), f(o + 1), f(o + 2)); }
  // faces: word0 = pts (3 x u8) | deleted << 24; word1 = adj0 | adj1 << 16; word2 = adj2; 3-5 normal
  __device__ __forceinline__ int fo(int fid) const { return L::W_FACES + L::FACE_WORDS * fid; }
  __device__ __forceinline__ int pt(int fid, int k) const { return (w(fo(fid)) >> (8 * k)) & 0xff; }
  __device__ __forceinline__ bool deleted(int fid) const { return (w(fo(fid)) >> 24) != 0; }
  __device__ __forceinline__ void set_deleted(int fid) const { w(fo(fid)) |= 0x01000000u; }
  __device__ __forceinline__ int adj(int fid, int k) const {
    return k == 0 ? (int)(w(fo(fid) + 1) & 0xffff) : (k == 1 ? (int)(w(fo(fid) + 1) >> 16) : (int)w(fo(fid) + 2));
  }
  __device__ __forceinline__ void set_adj(int fid, int k, int v) const {
    if (k == 0) w(fo(fid) + 1) = (w(fo(fid) + 1) & 0xffff0000u) | (uint32_t)v;
    else if (k == 1) w(fo(fid) + 1) = (w(fo(fid) + 1) & 0xffffu) | ((uint32_t)v << 16);
    else w(fo(fid) + 2) = (uint32_t)v;
  }
  __device__ __forceinline__ V3 normal(int fid) const { int o = fo(fid) + 3; return v3(f(o), f(o + 1), f(o + 2)); }
  // words 0-5 of a face record (pts | deleted flag, adj0 | adj1, adj2, normal) in vector loads
  struct Rec {
    uint32_t w0, w1, w2;
    V3 n;
  };
  __device__ __forceinline__ Rec rec(int fid) const {
    if constexpr (L::FACE_WORDS == 8) {
      const uint4 a = *reinterpret_cast<const uint4*>(base + fo(fid));
      const uint2 b = *reinterpret_cast<const uint2*>(base + fo(fid) + 4);
      return Rec{a.x, a.y, a.z, v3(__uint_as_float(a.w), __uint_as_float(b.x), __uint_as_float(b.y))};
    } else {
      const uint2* q = reinterpret_cast<const uint2*>(base + fo(fid));
      const uint2 a = q[0], b = q[1], c = q[2];
      return Rec{a.x, a.y, b.x, v3(__uint_as_float(b.y), __uint_as_float(c.x), __uint_as_float(c.y))};
    }
  }
  // writes words 0-5 of a face record in vector stores
  __device__ __forceinline__ void put_rec(int fid, uint32_t w0, uint32_t w1, uint32_t w2, V3 n) const {
    if constexpr (L::FACE_WORDS == 8) {
      *reinterpret_cast<uint4*>(base + fo(fid)) = make_uint4(w0, w1, w2, __float_as_uint(n.x));
      *reinterpret_cast<uint2*>(base + fo(fid) + 4) = make_uint2(__float_as_uint(n.y), __float_as_uint(n.z));
    } else {
      uint2* q = reinterpret_cast<uint2*>(base + fo(fid));
      q[0] = make_uint2(w0, w1);
      q[1] = make_uint2(w2, __float_as_uint(n.x));
      q[2] = make_uint2(__float_as_uint(n.y), __float_as_uint(n.z));
    }
  }
  // set_deleted for a face whose word 0 the caller already holds
  __device__ __forceinline__ void set_deleted_word(int fid, uint32_t w0) const { w(fo(fid)) = w0 | 0x01000000u; }
  // set_adj for a face whose word 1 the caller already holds
  __device__ __forceinline__ void set_adj_held(int fid, int k, int v, uint32_t w1) const {
    if (k == 0) w(fo(fid) + 1) = (w1 & 0xffff0000u) | (uint32_t)v;
    else if (k == 1) w(fo(fid) + 1) = (w1 & 0xffffu) | ((uint32_t)v << 16);
    else w(fo(fid) + 2) = (uint32_t)v;
  }
};
using EpaWs = EpaWsT<EpaGlobalLayout>;
// The workspace of slot `slot` in a pool of EPA_WORDS-word slots.
__device__ __forceinline__ EpaWs epa_slot(uint32_t* pool, uint32_t slot) { return EpaWs{pool + (size_t)slot * EPA_WORDS}; }

// Large workspaces for the few pairs whose polytope outgrows the regular slot (a second pass over
// those pairs only, on a small pool of these slots).
using EpaBigLayout = EpaLayout<128, 8192, 64, 1024>;
using EpaWsBig = EpaWsT<EpaBigLayout>;
constexpr size_t EPA_BIG_SLOT_BYTES = (size_t)EpaBigLayout::WORDS * 4;
constexpr uint32_t EPA_BIG_SLOTS = 640;  // 10 blocks of 64 threads: 216 MB
__device__ __forceinline__ EpaWsBig epa_slot_big(uint32_t* pool, uint32_t slot) {
  return EpaWsBig{pool + (size_t)slot * EpaBigLayout::WORDS};
}

template <class WS>
struct EpaHeap {
  uint2* h;  // (face id, distance bits) per entry, in the thread's local memory
  int len;
  __device__ __forceinline__ uint32_t id(int i) const { return h[i].x; }
  __device__ __forceinline__ uint2 ent(int i) const { return h[i]; }
  __device__ __forceinline__ void put(int i, uint2 e) const { h[i] = e; }
  static __device__ __forceinline__ float dist_of(uint2 e) { return __uint_as_float(e.y); }
  // FaceId::cmp: -1 / 0 / 1 (NaN -> 0)
  static __device__ __forceinline__ int cmp(float a, float b) { return a < b ? -1 : (a > b ? 1 : 0); }
  // BinaryHeap::sift_up of entry e, held in registers, from slot pos
  __device__ int sift_up(int start, int pos, uint2 e) {
    const float ed = dist_of(e);
    while (pos > start) {
      int parent = (pos - 1) / 2;
      const uint2 pe = ent(parent);
      if (cmp(ed, dist_of(pe)) <= 0) break;
      put(pos, pe);
      pos = parent;
    }
    put(pos, e);
    return pos;
  }
  __device__ void push(uint32_t fid, float d) {
    int old = len;
    len += 1;
    sift_up(0, old, make_uint2(fid, __float_as_uint(d)));
  }
  // BinaryHeap::sift_down_to_bottom of entry e from slot pos
  __device__ void sift_down_to_bottom(int pos, uint2 e) {
    int end = len, start = pos;
    int child = 2 * pos + 1;
    while (end >= 2 && child <= end - 2) {
      const uint2 c0 = ent(child), c1 = ent(child + 1);
      const bool right = cmp(dist_of(c0), dist_of(c1)) <= 0;
      child += right ? 1 : 0;
      put(pos, right ? c1 : c0);
      pos = child;
      child = 2 * pos + 1;
    }
    if (child == end - 1) {
      put(pos, ent(child));
      pos = child;
    }
    sift_up(start, pos, e);
  }
  // BinaryHeap::pop: the last entry moves to the root and sinks
  __device__ bool pop(uint32_t* fid, float* d) {
    if (len == 0) return false;
    len -= 1;
    uint2 out = ent(len);
    if (len > 0) {
      const uint2 root = ent(0);
      sift_down_to_bottom(0, out);
      out = root;
    }
    *fid = out.x;
    *d = dist_of(out);
    return true;
  }
};

// The barycentric part of Face::new (epa3.rs:90-118): the projection of the origin on triangle
// (A, B, C) as barycentric coordinates, and whether the origin projects inside it. A face's
// coordinates are not stored: they are recomputed from its vertices by this same function (same
// inputs, same operations, same bits) for the one face whose closest points are returned.
static __device__ __noinline__ bool epa_face_bcoords(V3 A, V3 B, V3 C, float bc[3]) {
  Loc loc;
  V3 proj = project_triangle(A, B, C, v3(0.f, 0.f, 0.f), &loc);
  bc[0] = 0.f; bc[1] = 0.f; bc[2] = 0.f;
  if (loc.kind == LOC_VERTEX || loc.kind == LOC_EDGE) {
    if (loc.kind == LOC_VERTEX) bc[loc.id] = 1.0f;
    else {
      int i0 = loc.id == 1 ? 1 : 0;
      int i1 = loc.id == 0 ? 1 : 2;
      bc[i0] = loc.bc[0];
      bc[i1] = loc.bc[1];
    }
    bool is_inside = fabsf(proj.x) <= EPS && fabsf(proj.y) <= EPS && fabsf(proj.z) <= EPS;
    float tol = EPS * 100.0f;
    return is_inside || dot(proj, proj) < tol * tol;
  } else if (loc.kind == LOC_FACE) {
    bc[0] = loc.bc[0]; bc[1] = loc.bc[1]; bc[2] = loc.bc[2];
    return true;
  }
  return false;
}

// The `inside` answer of epa_face_bcoords alone: the face region needs neither its barycentric
// coordinates nor their division, and a vertex or edge region only its projected point.
static __device__ __noinline__ bool epa_face_inside(V3 A, V3 B, V3 C) {
  const TriRegion r = tri_region(A, B, C, v3(0.f, 0.f, 0.f));
  if (r.region >= 6) return r.region == 6;
  V3 proj;
  if (r.region < 3) {
    proj = r.region == 0 ? A : (r.region == 1 ? B : C);
  } else {
    float t;
    proj = tri_edge_point(r, A, B, &t);
  }
  bool is_inside = fabsf(proj.x) <= EPS && fabsf(proj.y) <= EPS && fabsf(proj.z) <= EPS;
  float tol = EPS * 100.0f;
  return is_inside || dot(proj, proj) < tol * tol;
}

// Face::new (epa3.rs:90-118): writes face `fid`; returns whether the origin projects inside it and
// the face's distance from the origin along its normal, measured at its first vertex (the value the
// expansion loop pushes on the heap).
struct NewFace {
  float dist;
  bool inside;
};
template <class WS>
static __device__ __noinline__ NewFace epa_new_face(const WS& ws, int fid, int p0, int p1, int p2, int a0, int a1, int a2) {
  V3 A = ws.vp(p0), B = ws.vp(p1), C = ws.vp(p2);
  bool inside = epa_face_inside(A, B, C);
  V3 n;
  if (!try_normalize(cross(B - A, C - A), EPS, &n)) n = v3(0.f, 0.f, 0.f);
  ws.put_rec(fid, (uint32_t)p0 | ((uint32_t)p1 << 8) | ((uint32_t)p2 << 16), (uint32_t)a0 | ((uint32_t)a1 << 16), (uint32_t)a2, n);
  return NewFace{dot(n, A), inside};
}

// Face::closest_points (epa3.rs:120-129) for the face with vertices (a, b, c).
template <class WS>
__device__ __forceinline__ void epa_closest_points_of(const WS& ws, int a, int b, int c, V3* p1, V3* p2) {
  float bc[3];
  epa_face_bcoords(ws.vp(a), ws.vp(b), ws.vp(c), bc);
  *p1 = (ws.vo1(a) * bc[0] + ws.vo1(b) * bc[1]) + ws.vo1(c) * bc[2];
  *p2 = (ws.vo2(a) * bc[0] + ws.vo2(b) * bc[1]) + ws.vo2(c) * bc[2];
}

template <class WS>
__device__ __forceinline__ void epa_face_closest_points(const WS& ws, int fid, V3* p1, V3* p2) {
  epa_closest_points_of(ws, ws.pt(fid, 0), ws.pt(fid, 1), ws.pt(fid, 2), p1, p2);
}

template <class WS>
// `pt` is the point's position (the expansion's support point, in registers); the edge's two
// vertices are read only when the plane test does not settle it.
__device__ __forceinline__ bool epa_can_be_seen_by(const WS& ws, uint32_t w0, V3 fn, V3 pt, int opp) {
  const int i0 = (int)((w0 >> (8 * opp)) & 0xff);
  V3 p0 = ws.vp(i0);
  if (dot(pt - p0, fn) >= -GJK_EPS_TOL) return true;
  const int o1 = (opp + 1) % 3, o2 = (opp + 2) % 3;
  V3 p1 = ws.vp((int)((w0 >> (8 * o1)) & 0xff));
  V3 p2 = ws.vp((int)((w0 >> (8 * o2)) & 0xff));
  float e = EPS * 100.0f;
  V3 c = cross(p2 - p1, pt - p1);
  return fabsf(dot(c, c)) <= e * e;
}

enum : int { EPA_NONE = 0, EPA_OK = 1, EPA_OVERFLOW = 2 };

// EPA::closest_points. `iters` counts support evaluations. Returns EPA_OK with (p1, p2, n),
// EPA_NONE for the reference's None, EPA_OVERFLOW when a fixed capacity was exceeded. `sup(dir)`
// is CSOPoint::from_shapes(pos12, g1, g2, dir).
template <class WS, class Sup>
__device__ __forceinline__ int epa_closest_points_t(const WS& ws, Sup sup, const Simplex& simplex, V3* p1, V3* p2, V3* n, uint32_t* iters) {
  using L = typename WS::Layout;
  const float eps_tol = EPS * 100.0f;
  int nverts = simplex.dim + 1;
  for (int i = 0; i < nverts; ++i) ws.set_vert(i, simplex.v[i]);
  int nfaces = 0;
  // the heap in local memory (interleaved across a warp's lanes, whose sifts touch the same top
  // slots), or for large capacities in the workspace
  uint2 heap_local[L::HEAP_LOCAL ? L::MAX_FACES : 1];
  EpaHeap<WS> heap{L::HEAP_LOCAL ? heap_local : reinterpret_cast<uint2*>(&ws.w(L::W_HEAP)), 0};
  if (simplex.dim == 0) {
    *p1 = v3(0.f, 0.f, 0.f); *p2 = v3(0.f, 0.f, 0.f); *n = v3(0.f, 1.f, 0.f);
    return EPA_OK;
  } else if (simplex.dim == 3) {
    V3 dp1 = ws.vp(1) - ws.vp(0), dp2 = ws.vp(2) - ws.vp(0), dp3 = ws.vp(3) - ws.vp(0);
    if (dot(cross(dp1, dp2), dp3) > 0.0f) {
      CSO t1 = simplex.v[1], t2 = simplex.v[2];
      ws.set_vert(1, t2);
      ws.set_vert(2, t1);
    }
    bool in0 = epa_new_face(ws, 0, 0, 1, 2, 3, 1, 2).inside;
    bool in1 = epa_new_face(ws, 1, 1, 3, 2, 3, 2, 0).inside;
    bool in2 = epa_new_face(ws, 2, 0, 2, 3, 0, 1, 3).inside;
    bool in3 = epa_new_face(ws, 3, 0, 3, 1, 2, 1, 0).inside;
    nfaces = 4;
    bool ins[4] = {in0, in1, in2, in3};
    for (int k = 0; k < 4; ++k) {
      if (ins[k]) {
        float dist = dot(ws.normal(k), ws.vp(k));
        if (-dist > GJK_EPS_TOL) return EPA_NONE;
        heap.push((uint32_t)k, -dist);
      }
    }
    if (!(in0 || in1 || in2 || in3)) return EPA_NONE;
  } else {
    if (simplex.dim == 1) {
      V3 v = ws.vp(1) - ws.vp(0);
      V3 a = fabsf(v.x) > fabsf(v.y) ? v3(v.z, 0.0f, -v.x) : v3(0.0f, -v.z, v.y);
      a = normalize(a);
      ws.set_vert(2, sup(cross(a, v)));
      nverts = 3;
    }
    epa_new_face(ws, 0, 0, 1, 2, 1, 1, 1);
    epa_new_face(ws, 1, 0, 2, 1, 0, 0, 0);
    nfaces = 2;
    heap.push(0u, 0.0f);
    heap.push(1u, 0.0f);
  }
  int niter = 0;
  float max_dist = FLT_MAX;
  uint32_t best_id = heap.id(0);
  float old_dist = 0.0f;
  uint32_t fid_u;
  float neg;
  while (heap.pop(&fid_u, &neg)) {
    int fid = (int)fid_u;
    const auto F = ws.rec(fid);  // copy of the popped face (its fields are modified below)
    if (F.w0 >> 24) continue;     // deleted
    (*iters)++;
    int fpts[3] = {(int)(F.w0 & 0xff), (int)((F.w0 >> 8) & 0xff), (int)((F.w0 >> 16) & 0xff)};
    int fadj[3] = {(int)(F.w1 & 0xffff), (int)(F.w1 >> 16), (int)F.w2};
    V3 fnormal = F.n;
    if (nverts >= L::MAX_VERTS) return EPA_OVERFLOW;
    CSO cso = sup(fnormal);
    int support_id = nverts;
    ws.set_vert(nverts++, cso);
    float candidate = dot(cso.p, fnormal);
    if (candidate < max_dist) { best_id = fid_u; max_dist = candidate; }
    float curr_dist = -neg;
    if (max_dist - curr_dist < eps_tol || (fabsf(curr_dist - old_dist) < EPS && candidate < max_dist)) {
      epa_face_closest_points(ws, (int)best_id, p1, p2);
      *n = ws.normal((int)best_id);
      return EPA_OK;
    }
    old_dist = curr_dist;
    ws.set_deleted_word(fid, F.w0);
    // silhouette: depth-first walk restated with an explicit stack (same visiting order). An entry
    // holds the face and the vertex whose next_ccw gives the opposite corner, resolved when the entry
    // is popped and the face's record read anyway (a face's corners never change).
    int nsil = 0;
    int sp = 0;
    uint32_t stk[L::STACK], sil[L::MAX_SIL];  // local memory: a warp's lanes touch the same few slots
    auto next_ccw_of = [](uint32_t w0, int vid) {
      if ((int)(w0 & 0xff) == vid) return 1;
      if ((int)((w0 >> 8) & 0xff) == vid) return 2;
      return 0;
    };
    for (int k = 2; k >= 0; --k) stk[sp++] = (uint32_t)fadj[k] | ((uint32_t)fpts[k] << 16);
    while (sp > 0) {
      uint32_t e = stk[--sp];
      int id = (int)(e & 0xffff);
      const auto R = ws.rec(id);
      if (R.w0 >> 24) continue;  // deleted
      const int opp = next_ccw_of(R.w0, (int)(e >> 16));
      if (!epa_can_be_seen_by(ws, R.w0, R.n, cso.p, opp)) {
        if (nsil >= L::MAX_SIL) return EPA_OVERFLOW;
        sil[nsil++] = (uint32_t)id | ((uint32_t)opp << 16);
      } else {
        ws.set_deleted_word(id, R.w0);
        int a1 = (opp + 2) % 3, a2 = opp;
        auto adj_of = [&](int k) { return k == 0 ? (int)(R.w1 & 0xffff) : (k == 1 ? (int)(R.w1 >> 16) : (int)R.w2); };
        int adj1 = adj_of(a1), adj2 = adj_of(a2);
        if (sp + 2 > L::STACK) return EPA_OVERFLOW;
        stk[sp++] = (uint32_t)adj2 | (((R.w0 >> (8 * a2)) & 0xffu) << 16);
        stk[sp++] = (uint32_t)adj1 | (((R.w0 >> (8 * a1)) & 0xffu) << 16);
      }
    }
    int first_new = nfaces;
    if (nsil == 0) return EPA_NONE;
    for (int s = 0; s < nsil; ++s) {
      uint32_t e = sil[s];
      int sfid = (int)(e & 0xffff), opp = (int)(e >> 16);
      const uint2 w01 = *reinterpret_cast<const uint2*>(&ws.w(ws.fo(sfid)));  // pts | deleted, adj0 | adj1
      if (w01.x >> 24) continue;  // deleted
      if (nfaces >= L::MAX_FACES || heap.len >= L::MAX_FACES) return EPA_OVERFLOW;
      int new_id = nfaces;
      int pt1 = (int)((w01.x >> (8 * ((opp + 2) % 3))) & 0xff);
      int pt2 = (int)((w01.x >> (8 * ((opp + 1) % 3))) & 0xff);
      const NewFace nf = epa_new_face(ws, new_id, pt1, pt2, support_id, sfid, new_id + 1, new_id - 1);
      ws.set_adj_held(sfid, (opp + 1) % 3, new_id, w01.y);
      nfaces++;
      if (nf.inside) {
        const float dist = nf.dist;  // dot(normal, first vertex), as Face::new's caller computes it
        if (dist < curr_dist) {
          epa_closest_points_of(ws, fpts[0], fpts[1], fpts[2], p1, p2);
          *n = fnormal;
          return EPA_OK;
        }
        if (-dist > GJK_EPS_TOL) return EPA_NONE;
        heap.push((uint32_t)new_id, -dist);
      }
    }
    if (first_new == nfaces) return EPA_NONE;
    ws.set_adj(first_new, 2, nfaces - 1);
    ws.set_adj(nfaces - 1, 1, first_new);
    niter += 1;
    if (niter > 100) break;
  }
  epa_face_closest_points(ws, (int)best_id, p1, p2);
  *n = ws.normal((int)best_id);
  return EPA_OK;
}

// The per-thread form over a global-memory slot.
template <class WS>
static __device__ __noinline__ int epa_closest_points(const WS& ws, const Pose& pos12, const ShapeDev& g1, const ShapeDev& g2,
                                                      const Simplex& simplex, V3* p1, V3* p2, V3* n, uint32_t* iters) {
  return epa_closest_points_t(ws, [&](V3 d) { return cso_from_shapes(pos12, g1, g2, d); }, simplex, p1, p2, n, iters);
}

}  // namespace pg
