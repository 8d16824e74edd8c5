// Device-side pieces shared by the batched contact and contact-manifold kernels: the shape-array
// view, pair validation, point projections on cuboids and capsules, and the EPA work queue.
//   point projections  src/query/point/point_aabb.rs:9-132, src/query/point/point_capsule.rs:7-51
// (paths relative to the parry repository).
#pragma once
#include "internal.hpp"
#include "gjk_device.cuh"

namespace pg {

constexpr int QUEUE_WORDS = 40;  // pair, dim, 4 x CSO (9 words), pad

// ConvexPolyhedron topology on the device (parrygpu_polyhedra); all null when absent.
struct PolyArrays {
  const uint32_t* hulls;          // x8: first vertex, vertex count, first face, face count, first edge, edge count, ok, 0
  const float* face_normals;      // x3
  const uint32_t* face_ranges;    // x2
  const uint32_t* face_vertices;
  const uint32_t* face_edges;
  const uint32_t* vertex_ranges;  // x2, parallel to the vertex pool
  const uint32_t* vertex_faces;
  const uint32_t* vertex_edges;
  const float* edge_dirs;         // x3
  uint64_t n_hulls, n_faces, n_face_entries, n_vertex_entries, n_edges;
};

struct ShapeArrays {
  const uint32_t* types;
  const float4* params;
  const float* poses;
  const float* pool;
  uint64_t n_shapes;
  uint64_t n_vertices;
  PolyArrays poly;
  // Normal constraints (TrianglePseudoNormals rows of 12 floats) of a TriMesh's triangles: a
  // triangle shape of index >= pseudo_first whose params word 2 holds j > 0 uses row j - 1.
  const float* pseudo = nullptr;
  uint64_t pseudo_first = 0;
};

// Rejects out-of-range pair indices and vertex ranges (reported as a capacity / argument error
// through the context's error word; the pair reports no contact).
__device__ __forceinline__ bool valid_pair(const ShapeArrays& sh, uint32_t a, uint32_t b) {
  if (a >= sh.n_shapes || b >= sh.n_shapes) return false;
  uint32_t ids[2] = {a, b};
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    uint32_t t = sh.types[ids[k]];
    if (t > SH_TRIANGLE) return false;
    if (t == SH_CONVEX || t == SH_TRIANGLE) {
      float4 p = sh.params[ids[k]];
      uint64_t first = __float_as_uint(p.x), cnt = __float_as_uint(p.y);
      if (cnt == 0 || first + cnt > sh.n_vertices || (t == SH_TRIANGLE && cnt != 3)) return false;
    }
  }
  return true;
}

struct PointProj {
  bool inside;
  V3 point;
  int face;
  V3 shift;  // cuboid: the shift of do_project_local_point (point = pt + shift)
};

// point_aabb.rs:9-132 on [-h, h] with solid = false.
__device__ __forceinline__ PointProj project_cuboid(V3 h, V3 pt) {
  V3 mins = -h, maxs = h;
  V3 mins_pt = mins - pt, pt_maxs = pt - maxs;
  V3 z = v3(0.f, 0.f, 0.f);
  V3 shift = vmax(mins_pt, z) - vmax(pt_maxs, z);
  bool inside = shift.x == 0.0f && shift.y == 0.0f && shift.z == 0.0f;
  PointProj out;
  V3 ls;
  if (!inside) {
    ls = pt + shift;
    out.inside = false;
  } else {
    float best = -FLT_MAX;
    bool is_mins = false;
    int best_id = 0;
    float mp[3] = {mins_pt.x, mins_pt.y, mins_pt.z}, pm[3] = {pt_maxs.x, pt_maxs.y, pt_maxs.z};
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      if (mp[i] < pm[i]) {
        if (pm[i] > best) { best_id = i; is_mins = false; best = pm[i]; }
      } else if (mp[i] > best) { best_id = i; is_mins = true; best = mp[i]; }
    }
    float s[3] = {0.f, 0.f, 0.f};
    s[best_id] = is_mins ? best : -best;
    shift = v3(s[0], s[1], s[2]);
    ls = pt + shift;
    out.inside = true;
  }
  out.point = ls;
  out.shift = shift;
  out.face = -1;
  float sh[3] = {shift.x, shift.y, shift.z}, l[3] = {ls.x, ls.y, ls.z}, mn[3] = {mins.x, mins.y, mins.z}, mx[3] = {maxs.x, maxs.y, maxs.z};
  int nz = 0, last_nz = 0;
#pragma unroll
  for (int i = 0; i < 3; ++i) { if (sh[i] == 0.0f) nz++; else last_nz = i; }
  if (nz == 3) {
    for (int i = 0; i < 3; ++i) {
      if (l[i] > mx[i] - EPS) { out.face = i; break; }
      if (l[i] <= mn[i] + EPS) { out.face = i + 3; break; }
    }
  } else if (nz == 2) {
    float center = (mn[last_nz] + mx[last_nz]) * 0.5f;
    out.face = l[last_nz] < center ? last_nz + 3 : last_nz;
  }
  return out;
}

// point_capsule.rs:7-51 with solid = false.
__device__ __forceinline__ PointProj project_capsule(float hh, float radius, V3 pt) {
  Loc loc;
  V3 a = v3(0.f, -hh, 0.f), b = v3(0.f, hh, 0.f);
  V3 proj = project_segment(a, b, pt, &loc);
  V3 dir;
  float dist;
  PointProj out;
  out.face = -1;
  if (try_normalize(pt - proj, EPS, &dir, &dist)) {
    out.inside = dist <= radius;
    out.point = proj + dir * radius;
    return out;
  }
  V3 sd;
  out.inside = true;
  if (try_normalize(b - a, EPS, &sd)) {
    float sign = copysignf(1.0f, sd.z);
    float aa = -1.0f / (sign + sd.z);
    float bb = sd.x * sd.y * aa;
    V3 t = v3(1.0f + sign * sd.x * sd.x * aa, sign * bb, -sign * sd.x);
    out.point = proj + t * radius;
  } else {
    out.point = proj + v3(0.f, radius, 0.f);
  }
  return out;
}

// Appends (pair k, simplex) to the EPA queue; `tag` (word 39) tells the EPA kernel which query the
// pair came from.
__device__ __forceinline__ void enqueue(uint32_t* __restrict__ queue, unsigned long long* __restrict__ qcount, uint64_t k, const Simplex& s,
                                        uint32_t tag = 0) {
  unsigned long long slot = atomicAdd(qcount, 1ull);
  uint32_t* e = queue + (size_t)slot * QUEUE_WORDS;
  e[0] = (uint32_t)k;
  e[QUEUE_WORDS - 1] = tag;
  e[1] = (uint32_t)s.dim;
  for (int i = 0; i <= s.dim; ++i) {
    float* f = reinterpret_cast<float*>(e + 2 + 9 * i);
    f[0] = s.v[i].p.x; f[1] = s.v[i].p.y; f[2] = s.v[i].p.z;
    f[3] = s.v[i].o1.x; f[4] = s.v[i].o1.y; f[5] = s.v[i].o1.z;
    f[6] = s.v[i].o2.x; f[7] = s.v[i].o2.y; f[8] = s.v[i].o2.z;
  }
}

// Queue entry layout: pair index, simplex dimension, then dim + 1 CSO points (p, o1, o2).
__device__ __forceinline__ void dequeue(const uint32_t* __restrict__ e, uint64_t* k, Simplex* s) {
  *k = e[0];
  simplex_reset(*s, CSO{});
  s->dim = (int)e[1];
  for (int i = 0; i <= s->dim; ++i) {
    const float* f = reinterpret_cast<const float*>(e + 2 + 9 * i);
    s->v[i] = CSO{v3(f[0], f[1], f[2]), v3(f[3], f[4], f[5]), v3(f[6], f[7], f[8])};
  }
}

// Stages a parrygpu_shapes description on the device (host arrays are copied, device arrays used in place).
// defer_pool: a host vertex pool only gets its device buffer (out->pool), the caller copies it.
parrygpu_status stage_shapes(parrygpu_ctx* ctx, const parrygpu_shapes* s, ShapeArrays* out, bool defer_pool = false);

// Launchers on device buffers, no allocation and no host synchronisation (graph-capturable):
// Shape::compute_aabb(pos).loosened(margin) for n shapes (contact.cu);
// Shape::compute_aabb(pos) (aabb_ball.rs:7-33, aabb_cuboid.rs:9-14 with isometry_ops.rs:16-18,
// aabb_capsule.rs:8-20, aabb_utils.rs:58-86 for a point cloud).
__device__ __forceinline__ void shape_world_aabb(const ShapeDev& s, const Pose& p, V3* mn, V3* mx) {
  if (s.type == SH_BALL) {
    *mn = p.t + v3(-s.a, -s.a, -s.a);
    *mx = p.t + v3(s.a, s.a, s.a);
  } else if (s.type == SH_CUBOID) {
    // |R| h with R = to_rotation_matrix (isometry_ops.rs:14-19), row r = (|m_r0| hx + |m_r1| hy) + |m_r2| hz
    float ww = p.qw * p.qw, ii = p.qi * p.qi, jj = p.qj * p.qj, kk = p.qk * p.qk;
    float ij = p.qi * p.qj * 2.0f, wk = p.qw * p.qk * 2.0f, wj = p.qw * p.qj * 2.0f;
    float ik = p.qi * p.qk * 2.0f, jk = p.qj * p.qk * 2.0f, wi = p.qw * p.qi * 2.0f;
    float m00 = ww + ii - jj - kk, m01 = ij - wk, m02 = wj + ik;
    float m10 = wk + ij, m11 = ww - ii + jj - kk, m12 = jk - wi;
    float m20 = ik - wj, m21 = wi + jk, m22 = ww - ii - jj + kk;
    V3 he = v3((fabsf(m00) * s.a + fabsf(m01) * s.b) + fabsf(m02) * s.c, (fabsf(m10) * s.a + fabsf(m11) * s.b) + fabsf(m12) * s.c,
               (fabsf(m20) * s.a + fabsf(m21) * s.b) + fabsf(m22) * s.c);
    *mn = p.t - he;
    *mx = p.t + he;
  } else if (s.type == SH_CAPSULE) {
    V3 a = pose_point(p, v3(0.f, -s.a, 0.f)), b = pose_point(p, v3(0.f, s.a, 0.f));
    *mn = vmin(a, b) - v3(s.b, s.b, s.b);
    *mx = vmax(a, b) + v3(s.b, s.b, s.b);
  } else {
    *mn = pose_point(p, ldv(s.pts));
    *mx = *mn;
    for (uint32_t j = 1; j < s.npts; ++j) {
      V3 q = pose_point(p, ldv(s.pts + 3 * j));
      *mn = vmin(*mn, q);
      *mx = vmax(*mx, q);
    }
  }
}

parrygpu_status launch_shape_aabbs(parrygpu_ctx* ctx, const ShapeArrays& sh, uint64_t n, float margin, float* d_out);
// contact manifolds of the first min(cap, *d_count) pairs (manifold.cu) with caller-owned scratch
// sized by manifolds_reserve(cap).
parrygpu_status manifolds_reserve(parrygpu_ctx* ctx, uint64_t cap, MfScratch& scratch);
// The frame pipeline's learned GJK start directions (mlp.cu): per-shape descriptors computed once,
// a snapshot of the network's weights, and per-pair buffers sized for the pair capacity. The
// manifold classification lists the polyhedral pairs whose record holds no cached normal; their
// features and the network's directions are computed on the device before the polyhedral kernel.
struct LearnedSeed {
  const float* desc = nullptr;  // n_shapes x 16 descriptors
  const void* wb = nullptr;     // BF16 weights in the network's parameter layout
  const float* wf = nullptr;    // FP32 parameters (the biases are read from here)
  float* feat = nullptr;        // cap x PARRYGPU_MLP_IN features, 16-byte aligned
  uint32_t* list = nullptr;     // cap pair indices
  float* dirs = nullptr;        // cap x 3 directions, row = pair index
};
// Features and tcgen05 inference of the pairs list[0 .. min(cap, *d_count)), writing their rows of
// seed.dirs; no host synchronisation (graph-capturable).
parrygpu_status launch_seed_dirs(parrygpu_ctx* ctx, const ShapeArrays& sh, const uint32_t* d_pairs, const LearnedSeed& seed,
                                 const unsigned long long* d_count, uint64_t cap);
// The shape descriptors (desc: n x 16 floats) and a snapshot of the network's BF16 weights and FP32
// parameters into wb / wf; asynchronous on the context stream.
parrygpu_status seed_prepare(parrygpu_ctx* ctx, const parrygpu_mlp* mlp, const ShapeArrays& sh, DevBuf& desc, DevBuf& wb, DevBuf& wf);
// d_count may be null (then all `cap` pairs); returns after queuing the launches. init_dirs (may be
// null): per-pair GJK start directions of the polyhedral generator where a record holds no cached
// normal; with `seed`, the network computes them for the pairs that need one (init_dirs ignored).
parrygpu_status launch_manifolds(parrygpu_ctx* ctx, const ShapeArrays& sh, const uint32_t* d_pairs, uint64_t cap,
                                 const unsigned long long* d_count, float prediction, uint32_t* d_recs, MfScratch& scratch,
                                 const float* init_dirs = nullptr, const LearnedSeed* seed = nullptr);

}  // namespace pg
