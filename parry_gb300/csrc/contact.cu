// Batched query::contact for convex shapes (balls, cuboids, capsules, convex polyhedra, triangles)
// and per-shape AABBs.
//
// Pipeline (one stream, no host round trip):
//   k_pair_cost_keys + radix sort   pairs binned by support-scan cost (vertices one support
//                    evaluation scans), ascending.
//   k_contacts_fused one persistent launch over work items taken from an atomic counter:
//                    - the pairs at the top of the cost order (cost >= the configured threshold), one
//                      warp per pair, dearest first: both hulls staged into shared memory by the TMA
//                      unit (cp.async.bulk), support points by a lane-parallel scan reduced with warp
//                      shuffles (first index on ties), GJK and then EPA with the polytope in the warp's
//                      shared memory (a polytope that outgrows it goes to the per-thread EPA pass);
//                    - then the others, 32 consecutive pairs per item, one thread per pair: dispatch
//                      of DefaultQueryDispatcher::contact (src/query/default_query_dispatcher.rs:
//                      302-356): ball-ball analytic, ball-convex by point projection, otherwise GJK
//                      (gjk_device.cuh). Pairs whose GJK ends inside the Minkowski difference append
//                      (pair, final simplex) to an EPA queue.
//   k_contacts_epa   persistent grid-stride loop over the EPA queue, one polytope workspace slot per
//                    thread (epa_device.cuh), finishing those pairs exactly as the reference does.
// Every path runs the reference's steps in the same order on the same values, so the answers do not
// depend on which path a pair takes. Results are written in world space (contact_shape_shape.rs:
// 123-138).
// the support scan's loop unrolled as the compiler chooses (faster here than any explicit factor)
#define PG_SCAN_UNROLL 0
#include "internal.hpp"
#include "epa_device.cuh"
#include "contact_device.cuh"
#include "bulk_copy.cuh"
#include <algorithm>
#include <cstring>

using namespace pg;

namespace {

constexpr int EPA_THREADS = 64;

struct ContactOut {
  V3 p1, p2, n1, n2;
  float dist;
};

// contact_ball_ball.rs:9-42
__device__ __forceinline__ bool contact_ball_ball(const Pose& pos12, float r1, float r2, float prediction, ContactOut* c) {
  V3 center = pos12.t;
  float d2 = dot(center, center);
  float sum = r1 + r2;
  float sum_err = sum + prediction;
  if (!(d2 < sum_err * sum_err)) return false;
  V3 n1 = d2 != 0.0f ? normalize(center) : v3(1.f, 0.f, 0.f);
  V3 n2 = -pose_inv_rotate(pos12, n1);
  c->p1 = n1 * r1;
  c->p2 = n2 * r2;
  c->n1 = n1;
  c->n2 = n2;
  c->dist = sqrtf(d2) - sum;
  return true;
}

// Finishes contact_convex_polyhedron_ball (contact_ball_convex_polyhedron.rs:26-63) from a projection.
__device__ __forceinline__ bool finish_convex_ball(const Pose& pos12, const ShapeDev& s1, const PointProj& proj, float r2, float prediction,
                                                   ContactOut* c) {
  V3 center = pos12.t;
  float dist;
  V3 n1, dir1;
  float len;
  if (try_normalize(proj.point - center, EPS, &dir1, &len)) {
    if (proj.inside) { dist = -len - r2; n1 = dir1; }
    else { dist = len - r2; n1 = -dir1; }
  } else {
    dist = -r2;
    if (s1.type == SH_CUBOID && proj.face >= 0) {
      float d[3] = {0.f, 0.f, 0.f};
      if (proj.face < 3) d[proj.face] = 1.0f; else d[proj.face - 3] = -1.0f;
      n1 = v3(d[0], d[1], d[2]);
    } else if (!try_normalize(proj.point, EPS, &n1)) {
      n1 = v3(0.f, 1.f, 0.f);
    }
  }
  if (!(dist <= prediction)) return false;
  V3 n2 = pose_inv_rotate(pos12, -n1);
  c->p1 = proj.point;
  c->p2 = n2 * r2;
  c->n1 = n1;
  c->n2 = n2;
  c->dist = dist;
  return true;
}

// contact_support_map_support_map: ClosestPoints -> Contact
__device__ __forceinline__ void finish_support_pair(const Pose& pos12, V3 p1, V3 p2, V3 n1, ContactOut* c) {
  c->dist = dot(p2 - p1, n1);
  c->p1 = p1;
  c->p2 = pose_inv_point(pos12, p2);
  c->n1 = n1;
  c->n2 = pose_inv_rotate(pos12, -n1);
}

__device__ __forceinline__ void write_out(float* __restrict__ out, uint8_t* __restrict__ has, uint64_t k, bool ok, const ContactOut& c,
                                          const Pose& pa, const Pose& pb) {
  float* o = out + 13 * k;
  if (ok) {
    V3 p1 = pose_point(pa, c.p1), p2 = pose_point(pb, c.p2), n1 = pose_rotate(pa, c.n1), n2 = pose_rotate(pb, c.n2);
    o[0] = p1.x; o[1] = p1.y; o[2] = p1.z;
    o[3] = p2.x; o[4] = p2.y; o[5] = p2.z;
    o[6] = n1.x; o[7] = n1.y; o[8] = n1.z;
    o[9] = n2.x; o[10] = n2.y; o[11] = n2.z;
    o[12] = c.dist;
  } else {
#pragma unroll
    for (int j = 0; j < 13; ++j) o[j] = 0.0f;
  }
  has[k] = ok ? 1 : 0;
}

// Which path a pair takes in DefaultQueryDispatcher::contact.
enum : int { PATH_BALL_BALL = 0, PATH_BALL_FIRST = 1, PATH_BALL_SECOND = 2, PATH_SUPPORT = 3 };

struct PairSetup {
  ShapeDev s1, s2;
  Pose pa, pb, pos12;
  int path;
  // for the ball paths: the convex shape, the pose used for the projection and the ball radius
  Pose cpos;
  const ShapeDev* convex;
  float radius;
};

__device__ __forceinline__ void setup_pair(const ShapeArrays& sh, uint32_t a, uint32_t b, PairSetup* ps) {
  ps->s1 = load_shape(sh.types, sh.params, sh.pool, a);
  ps->s2 = load_shape(sh.types, sh.params, sh.pool, b);
  ps->pa = load_pose(sh.poses, a);
  ps->pb = load_pose(sh.poses, b);
  ps->pos12 = pose_inv_mul(ps->pa, ps->pb);
  bool b1 = ps->s1.type == SH_BALL, b2 = ps->s2.type == SH_BALL;
  if (b1 && b2) ps->path = PATH_BALL_BALL;
  else if (b1) { ps->path = PATH_BALL_FIRST; ps->cpos = pose_inverse(ps->pos12); ps->convex = &ps->s2; ps->radius = ps->s1.a; }
  else if (b2) { ps->path = PATH_BALL_SECOND; ps->cpos = ps->pos12; ps->convex = &ps->s1; ps->radius = ps->s2.a; }
  else ps->path = PATH_SUPPORT;
}

__device__ __forceinline__ void flip(ContactOut* c) {
  V3 t = c->p1; c->p1 = c->p2; c->p2 = t;
  t = c->n1; c->n1 = c->n2; c->n2 = t;
}

// Binning key of a pair: the vertices one support evaluation of the pair scans (vertex count of
// a convex / triangle shape, 1 for the others, summed over the two shapes; capped at 1023).
// Threads of a warp then run pairs of similar cost, and so do the EPA queue entries they append.
// Keys of pairs base .. base + n - 1, values their indices.
__global__ void k_pair_cost_keys(ShapeArrays sh, const uint32_t* __restrict__ pairs, uint32_t base, uint32_t n, uint32_t* __restrict__ keys,
                                 uint32_t* __restrict__ vals) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const size_t k = (size_t)base + i;
  uint32_t a = pairs[2 * k], b = pairs[2 * k + 1];
  uint32_t c = 2;
  if (a < sh.n_shapes && b < sh.n_shapes) {
    uint32_t ta = sh.types[a], tb = sh.types[b];
    uint32_t ca = (ta == SH_CONVEX || ta == SH_TRIANGLE) ? __float_as_uint(sh.params[a].y) : 1u;
    uint32_t cb = (tb == SH_CONVEX || tb == SH_TRIANGLE) ? __float_as_uint(sh.params[b].y) : 1u;
    c = (ca > 1023u ? 1023u : ca) + (cb > 1023u ? 1023u : cb);
  }
  keys[i] = c > 1023u ? 1023u : c;
  vals[i] = (uint32_t)k;
}

// For chunk c of `chunk` consecutive pairs (a multiple of 32): the end (exclusive) of the
// vertex-pool range that the chunk's shapes reference, maximised into ends[c] (zeroed by the
// caller). Invalid shape indices are skipped (the contact kernels report them).
__global__ void k_chunk_vertex_ends(ShapeArrays sh, const uint32_t* __restrict__ pairs, uint64_t n, uint64_t chunk,
                                    unsigned long long* __restrict__ ends) {
  const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  unsigned long long e = 0;
  if (i < n) {
    for (int j = 0; j < 2; ++j) {
      const uint32_t s = pairs[2 * i + j];
      if (s >= sh.n_shapes) continue;
      const uint32_t t = sh.types[s];
      if (t == SH_CONVEX || t == SH_TRIANGLE) {
        const float4 p = sh.params[s];
        const unsigned long long end = (unsigned long long)__float_as_uint(p.x) + __float_as_uint(p.y);
        e = end > e ? end : e;
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long x = __shfl_xor_sync(0xffffffffu, e, o);
    e = x > e ? x : e;
  }
  if ((threadIdx.x & 31) == 0 && e && i < n) atomicMax(&ends[i / chunk], e);
}

// EPA for pair k from GJK's final simplex s, finishing query::contact as the reference does (the
// support-map pair's closest points, or the projection of a ball's centre onto a convex shape).
// Returns EPA_OVERFLOW when the workspace is too small (nothing written, *iters unchanged), else
// writes the pair's result.
template <class WS>
__device__ __forceinline__ int epa_pair(const WS& ws, const PairSetup& ps, uint64_t k, const Simplex& s, float prediction,
                                        float* __restrict__ out, uint8_t* __restrict__ has, float* __restrict__ final_dirs,
                                        uint32_t* iters) {
  ContactOut c;
  bool ok = false;
  V3 p1, p2, nn;
  uint32_t it = 0;
  int r;
  if (ps.path == PATH_SUPPORT) {
    r = epa_closest_points(ws, ps.pos12, ps.s1, ps.s2, s, &p1, &p2, &nn, &it);
    if (r == EPA_OVERFLOW) return r;
    if (r == EPA_OK) { ok = true; finish_support_pair(ps.pos12, p1, p2, nn, &c); }
    if (final_dirs) {
      V3 fd = r == EPA_OK ? nn : v3(1.f, 0.f, 0.f);  // GJKResult::NoIntersection(x) when EPA fails
      final_dirs[3 * k] = fd.x; final_dirs[3 * k + 1] = fd.y; final_dirs[3 * k + 2] = fd.z;
    }
  } else {
    const ShapeDev& cs = *ps.convex;
    V3 center = ps.cpos.t;
    Pose m{0.f, 0.f, 0.f, 1.f, -center};
    Pose minv = pose_inverse(m);
    ShapeDev origin;
    origin.type = SH_ORIGIN;
    PointProj proj;
    proj.face = -1;
    proj.inside = true;
    r = epa_closest_points(ws, minv, cs, origin, s, &p1, &p2, &nn, &it);
    if (r == EPA_OVERFLOW) return r;
    proj.point = r == EPA_OK ? p1 : center;
    ok = finish_convex_ball(ps.cpos, cs, proj, ps.radius, prediction, &c);
    if (ok && ps.path == PATH_BALL_FIRST) flip(&c);
  }
  *iters += it;
  write_out(out, has, k, ok, c, ps.pa, ps.pb);
  return r;
}

// Where a pair's EPA goes once its GJK ends inside the Minkowski difference: the queue of the
// per-thread EPA pass (ws = NULL), or this thread's own workspace slot right away (ws set: the
// hulls GJK just read are still in cache), a polytope outgrowing that slot going to the
// large-slot pass through the overflow list.
struct LaneEpa {
  const EpaWs* ws;
  uint32_t* ovf;
  unsigned long long* ovf_count;
  uint32_t iters = 0, calls = 0;
};

__device__ __forceinline__ void lane_epa(LaneEpa& le, const PairSetup& ps, uint64_t k, const Simplex& s, float prediction,
                                         float* __restrict__ out, uint8_t* __restrict__ has, float* __restrict__ final_dirs,
                                         uint32_t* __restrict__ queue, unsigned long long* __restrict__ qcount) {
  if (!le.ws) { enqueue(queue, qcount, k, s); return; }
  if (epa_pair(*le.ws, ps, k, s, prediction, out, has, final_dirs, &le.iters) == EPA_OVERFLOW) {
    const unsigned long long e = atomicAdd(qcount, 1ull);
    uint32_t* q = queue + (size_t)e * QUEUE_WORDS;
    q[0] = (uint32_t)k;
    q[QUEUE_WORDS - 1] = 0;
    q[1] = (uint32_t)s.dim;
    for (int i = 0; i <= s.dim; ++i) {
      float* f = reinterpret_cast<float*>(q + 2 + 9 * i);
      f[0] = s.v[i].p.x; f[1] = s.v[i].p.y; f[2] = s.v[i].p.z;
      f[3] = s.v[i].o1.x; f[4] = s.v[i].o1.y; f[5] = s.v[i].o1.z;
      f[6] = s.v[i].o2.x; f[7] = s.v[i].o2.y; f[8] = s.v[i].o2.z;
    }
    le.ovf[atomicAdd(le.ovf_count, 1ull)] = (uint32_t)e;
    return;
  }
  le.calls++;
}

// query::contact for pair k on this thread alone (EPA as `le` says). Adds its GJK support
// evaluations to *iters.
__device__ __forceinline__ void contact_pair_lane(const ShapeArrays& sh, const uint32_t* __restrict__ pairs, uint64_t k, float prediction,
                                                  const float* __restrict__ init_dirs, float* __restrict__ out, uint8_t* __restrict__ has,
                                                  uint32_t* __restrict__ queue, unsigned long long* __restrict__ qcount,
                                                  uint32_t* __restrict__ err, float* __restrict__ final_dirs, uint32_t* iters_out,
                                                  LaneEpa& le) {
  uint32_t iters = 0;
  if (!valid_pair(sh, pairs[2 * k], pairs[2 * k + 1])) {
    atomicOr(err, ERR_CAPACITY);
    float* o = out + 13 * k;
    for (int j = 0; j < 13; ++j) o[j] = 0.0f;
    has[k] = 0;
  } else {
    PairSetup ps;
    setup_pair(sh, pairs[2 * k], pairs[2 * k + 1], &ps);
    ContactOut c;
    bool ok = false, done = true;
    if (ps.path == PATH_BALL_BALL) {
      ok = contact_ball_ball(ps.pos12, ps.s1.a, ps.s2.a, prediction, &c);
    } else if (ps.path != PATH_SUPPORT) {
      const ShapeDev& cs = *ps.convex;
      PointProj proj;
      V3 center = ps.cpos.t;
      if (cs.type == SH_CUBOID) proj = project_cuboid(v3(cs.a, cs.b, cs.c), center);
      else if (cs.type == SH_CAPSULE) proj = project_capsule(cs.a, cs.b, center);
      else {
        // point_support_map.rs:17-57: GJK projection of the origin onto shape - center
        Pose m{0.f, 0.f, 0.f, 1.f, -center};
        Pose minv = pose_inverse(m);
        Pose m_inv{0.f, 0.f, 0.f, 1.f, center};
        ShapeDev origin;
        origin.type = SH_ORIGIN;
        V3 dir;
        if (!try_normalize(-m.t, EPS, &dir)) dir = v3(1.f, 0.f, 0.f);
        Simplex s;
        simplex_reset(s, cso_from_shapes(m_inv, cs, origin, dir));
        GjkOut g = gjk_closest_points(minv, cs, origin, FLT_MAX, s, &iters);
        if (g.kind == GJK_CLOSEST) {
          proj.inside = false;
          proj.point = g.p1;
          proj.face = -1;
        } else {
          lane_epa(le, ps, k, s, prediction, out, has, final_dirs, queue, qcount);
          done = false;
        }
      }
      if (done) {
        ok = finish_convex_ball(ps.cpos, cs, proj, ps.radius, prediction, &c);
        if (ok && ps.path == PATH_BALL_FIRST) flip(&c);
      }
    } else {
      V3 dir;
      if (init_dirs) dir = v3(init_dirs[3 * k], init_dirs[3 * k + 1], init_dirs[3 * k + 2]);
      else if (!try_normalize(ps.pos12.t, EPS, &dir)) dir = v3(1.f, 0.f, 0.f);
      Simplex s;
      simplex_reset(s, cso_from_shapes(ps.pos12, ps.s1, ps.s2, dir));
      GjkOut g = gjk_closest_points(ps.pos12, ps.s1, ps.s2, prediction, s, &iters);
      if (g.kind == GJK_CLOSEST) {
        ok = true;
        finish_support_pair(ps.pos12, g.p1, g.p2, g.dir, &c);
      } else if (g.kind == GJK_INTERSECTION) {
        lane_epa(le, ps, k, s, prediction, out, has, final_dirs, queue, qcount);
        done = false;
      }
      if (final_dirs && g.kind != GJK_INTERSECTION) {
        final_dirs[3 * k] = g.dir.x; final_dirs[3 * k + 1] = g.dir.y; final_dirs[3 * k + 2] = g.dir.z;
      }
    }
    if (final_dirs && ps.path != PATH_SUPPORT) {
      final_dirs[3 * k] = 0.0f; final_dirs[3 * k + 1] = 0.0f; final_dirs[3 * k + 2] = 0.0f;
    }
    if (done) write_out(out, has, k, ok, c, ps.pa, ps.pb);
  }
  *iters_out += iters;
}

// ---- one warp per pair ----

// point_cloud_support_point (src/utils/point_cloud_support_point.rs:5-19) with the warp's 32 lanes:
// lane l scans vertices l, l + 32, ... keeping the first index of its largest dot product (NaN
// products never count), and a shuffle reduction keeps the largest value, then the smallest index.
// That is the sequential scan's answer (best = 0, then strict `>`), whose seed only matters when
// vertex 0's product is NaN: then nothing replaces it. Every lane returns the same vertex.
__device__ __forceinline__ V3 warp_convex_support(const float* pts, uint32_t n, V3 dir) {
  const uint32_t lane = threadIdx.x & 31;
  float bd = 0.0f;
  uint32_t bi = 0xffffffffu;
  bool nan0 = false;  // vertex 0's product is NaN (lane 0 scans vertex 0)
  for (uint32_t i = lane; i < n; i += 32) {
    const float d = dot(v3(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]), dir);
    if (i == 0 && d != d) nan0 = true;
    if (bi == 0xffffffffu ? !(d != d) : d > bd) { bd = d; bi = i; }
  }
  nan0 = __shfl_sync(0xffffffffu, nan0, 0);
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const float od = __shfl_xor_sync(0xffffffffu, bd, off);
    const uint32_t oi = __shfl_xor_sync(0xffffffffu, bi, off);
    if (oi != 0xffffffffu && (bi == 0xffffffffu || od > bd || (od == bd && oi < bi))) { bd = od; bi = oi; }
  }
  if (nan0 || bi == 0xffffffffu) bi = 0;
  return v3(pts[3 * bi], pts[3 * bi + 1], pts[3 * bi + 2]);
}

__device__ __forceinline__ V3 warp_local_support(const ShapeDev& s, V3 dir) {
  return s.type == SH_CONVEX ? warp_convex_support(s.pts, s.npts, dir) : local_support(s, dir);
}

// Polytope of one warp-per-pair EPA in shared memory: 64 vertices, 256 faces (24-byte records),
// silhouettes of 32 edges, a walk stack of 128 (an EPA call that outgrows it finishes in the
// per-thread pass).
using EpaSmemLayout = EpaLayout<64, 256, 32, 128, 6>;
using EpaWsSmem = EpaWsT<EpaSmemLayout>;
// Hull vertices staged per shape (larger hulls are scanned where they lie in global memory); 4
// spare floats absorb the shift that keeps the bulk-copied body 16-byte aligned.
constexpr uint32_t STAGE_VERTS = 256;
constexpr uint32_t STAGE_FLOATS = 3 * STAGE_VERTS + 4;
constexpr int FUSED_WARPS = 4;
constexpr int FUSED_THREADS = 32 * FUSED_WARPS;
constexpr uint32_t MBAR_WAIT_POLLS = 1u << 24;

struct __align__(16) WarpSmem {
  uint32_t epa[EpaSmemLayout::WORDS];
  float hull[2][STAGE_FLOATS];
  uint64_t bar;
  uint64_t pad;
};
static_assert(sizeof(WarpSmem) % 16 == 0 && (EpaSmemLayout::WORDS * 4) % 16 == 0 && (STAGE_FLOATS * 4) % 16 == 0,
              "16-byte aligned shared-memory regions");

// Stages shape s's vertices into `dst` (16-byte aligned) when it is a convex polyhedron of at most
// STAGE_VERTS vertices: the 16-byte-aligned body of its byte range by one bulk copy issued by lane 0
// (bytes added to *tx), the ragged head and tail (at most 3 floats each) by plain loads of lanes
// 0-5. Points s.pts at the staged copy. Returns false (nothing staged) otherwise.
__device__ __forceinline__ bool stage_hull(ShapeDev& s, float* dst, uint64_t* bar, uint32_t* tx) {
  if (s.type != SH_CONVEX || s.npts > STAGE_VERTS || s.npts == 0) return false;
  const uint32_t lane = threadIdx.x & 31;
  const uintptr_t start = reinterpret_cast<uintptr_t>(s.pts), end = start + 12u * (uintptr_t)s.npts;
  const uintptr_t base = start & ~(uintptr_t)15;         // dst[0] mirrors this address
  const uintptr_t b0 = (start + 15) & ~(uintptr_t)15, b1 = end & ~(uintptr_t)15;
  float* vdst = dst + (start - base) / 4;                 // where vertex 0 lands
  if (b1 > b0) {
    if (lane == 0) {
      const uint32_t bytes = (uint32_t)(b1 - b0);
      bulk_copy_g2s(dst + (b0 - base) / 4, reinterpret_cast<const void*>(b0), bytes, bar);
      *tx += bytes;
    }
    const uint32_t head = (uint32_t)(b0 - start) / 4, tail = (uint32_t)(end - b1) / 4;
    if (lane < head) vdst[lane] = s.pts[lane];
    else if (lane >= 8 && lane < 8 + tail) {
      const uint32_t j = (uint32_t)(b1 - start) / 4 + (lane - 8);
      vdst[j] = s.pts[j];
    }
  } else {
    for (uint32_t j = lane; j < 3 * s.npts; j += 32) vdst[j] = s.pts[j];
  }
  s.pts = vdst;
  return true;
}

// query::contact for pair k (a PATH_SUPPORT pair) with the whole warp; every lane runs the
// reference's steps on the same values (uniform control flow), the support scans lane-parallel.
// Returns false when the staging wait timed out (the warp must stop).
__device__ bool contact_pair_warp(const PairSetup& ps0, uint64_t k, float prediction, const float* __restrict__ init_dirs,
                                  float* __restrict__ out, uint8_t* __restrict__ has, uint32_t* __restrict__ queue,
                                  unsigned long long* __restrict__ qcount, uint32_t* __restrict__ err, float* __restrict__ final_dirs,
                                  WarpSmem* w, uint32_t* phase, uint32_t* gjk_iters, uint32_t* epa_iters, uint32_t* epa_calls) {
  const uint32_t lane = threadIdx.x & 31;
  PairSetup ps = ps0;
  // the previous pair's reads of the staging buffers are over before the bulk copies refill them
  __syncwarp();
  fence_async_shared();
  uint32_t tx = 0;
  stage_hull(ps.s1, w->hull[0], &w->bar, &tx);
  stage_hull(ps.s2, w->hull[1], &w->bar, &tx);
  // the phase's one arrival, with the bytes the copies will complete (the phase cannot complete
  // before this arrival, so copies issued first are counted)
  if (lane == 0) mbar_arrive_expect_tx(&w->bar, tx);
  if (!mbar_wait_bounded(&w->bar, *phase, MBAR_WAIT_POLLS)) {
    if (lane == 0) atomicOr(err, ERR_TIMEOUT);
    mbar_wait_bounded(&w->bar, *phase, MBAR_WAIT_POLLS);  // the copies in flight, once more, before the warp leaves
    return false;
  }
  *phase ^= 1u;
  __syncwarp();  // the lanes' ragged stores are visible to the whole warp
  const ShapeDev& g1 = ps.s1;
  const ShapeDev& g2 = ps.s2;
  const Pose pos12 = ps.pos12;
  auto sup = [&](V3 d) {
    const V3 sp1 = warp_local_support(g1, d);
    const V3 sp2 = pose_point(pos12, warp_local_support(g2, pose_inv_rotate(pos12, -d)));
    return CSO{sp1 - sp2, sp1, sp2};
  };
  V3 dir;
  if (init_dirs) dir = v3(init_dirs[3 * k], init_dirs[3 * k + 1], init_dirs[3 * k + 2]);
  else if (!try_normalize(pos12.t, EPS, &dir)) dir = v3(1.f, 0.f, 0.f);
  Simplex s;
  simplex_reset(s, sup(dir));
  uint32_t gi = 0;
  const GjkOut g = gjk_closest_points_t(sup, prediction, s, &gi);
  ContactOut c;
  bool ok = false, done = true;
  V3 fd = g.dir;
  uint32_t ei = 0, calls = 0;
  if (g.kind == GJK_CLOSEST) {
    ok = true;
    finish_support_pair(pos12, g.p1, g.p2, g.dir, &c);
  } else if (g.kind == GJK_INTERSECTION) {
    EpaWsSmem ws{w->epa};
    V3 p1, p2, nn;
    const int r = epa_closest_points_t(ws, sup, s, &p1, &p2, &nn, &ei);
    if (r == EPA_OVERFLOW) {  // the per-thread EPA pass redoes this pair from GJK's simplex
      if (lane == 0) enqueue(queue, qcount, k, s);
      done = false;
      ei = 0;
    } else {
      calls = 1;
      if (r == EPA_OK) { ok = true; finish_support_pair(pos12, p1, p2, nn, &c); }
      fd = r == EPA_OK ? nn : v3(1.f, 0.f, 0.f);  // GJKResult::NoIntersection(x) when EPA fails
    }
  }
  if (lane == 0) {
    if (final_dirs && done) { final_dirs[3 * k] = fd.x; final_dirs[3 * k + 1] = fd.y; final_dirs[3 * k + 2] = fd.z; }
    if (done) write_out(out, has, k, ok, c, ps.pa, ps.pb);
    *gjk_iters += gi;
    *epa_iters += ei;
    *epa_calls += calls;
  }
  return true;
}

// Largest pair count n_large such that the last n_large pairs of the ascending cost order cost at
// least `threshold` (one thread, binary search over the sorted keys).
__global__ void k_count_costly(const uint32_t* __restrict__ sorted_keys, uint32_t n, uint32_t threshold, unsigned long long* __restrict__ out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  uint32_t lo = 0, hi = n;
  while (lo < hi) {
    const uint32_t mid = lo + (hi - lo) / 2;
    if (sorted_keys[mid] < threshold) lo = mid + 1; else hi = mid;
  }
  *out = n - lo;
}

// The persistent launch: item i < *n_large is the pair order[n - 1 - i] for one warp; the items after
// it are runs of 32 pairs of order[0 ..) (order = NULL: pairs in input order), one per lane.
// INLINE: per-thread pairs run EPA in their thread's own workspace slot of ws_pool right after GJK
// (else through the queue).
template <bool INLINE>
__global__ void __launch_bounds__(FUSED_THREADS, 3) k_contacts_fused(ShapeArrays sh, const uint32_t* __restrict__ pairs, uint64_t n,
                                                                  const uint32_t* __restrict__ order,
                                                                  const unsigned long long* __restrict__ n_large_ptr, float prediction,
                                                                  const float* __restrict__ init_dirs, float* __restrict__ out,
                                                                  uint8_t* __restrict__ has, uint32_t* __restrict__ queue,
                                                                  unsigned long long* __restrict__ qcount, unsigned long long* __restrict__ stats,
                                                                  uint32_t* __restrict__ err, float* __restrict__ final_dirs,
                                                                  unsigned long long* __restrict__ work, uint32_t* __restrict__ ws_pool,
                                                                  uint32_t* __restrict__ ovf, unsigned long long* __restrict__ ovf_count) {
  extern __shared__ __align__(16) unsigned char fused_smem[];
  WarpSmem* w = reinterpret_cast<WarpSmem*>(fused_smem) + (threadIdx.x >> 5);
  const uint32_t lane = threadIdx.x & 31;
  const EpaWs slot = epa_slot(ws_pool, blockIdx.x * blockDim.x + threadIdx.x);
  LaneEpa le{INLINE ? &slot : nullptr, ovf, ovf_count};
  const uint64_t n_large = order ? *n_large_ptr : 0;
  const uint64_t n_small = n - n_large;
  if (n_large && lane == 0) mbar_init(&w->bar, 1);
  __syncwarp();
  uint32_t phase = 0, gjk_iters = 0, epa_iters = 0, epa_calls = 0;
  for (;;) {
    unsigned long long item = 0;
    if (lane == 0) item = atomicAdd(work, 1ull);
    item = __shfl_sync(0xffffffffu, item, 0);
    if (item < n_large) {
      const uint64_t k = order[n - 1 - item];
      const uint32_t a = pairs[2 * k], b = pairs[2 * k + 1];
      bool warp_path = valid_pair(sh, a, b);
      PairSetup ps;
      if (warp_path) {
        setup_pair(sh, a, b, &ps);
        warp_path = ps.path == PATH_SUPPORT;
      }
      if (!warp_path) {  // a ball pair or an invalid one: the per-thread code on lane 0
        if (lane == 0) contact_pair_lane(sh, pairs, k, prediction, init_dirs, out, has, queue, qcount, err, final_dirs, &gjk_iters, le);
        __syncwarp();
        continue;
      }
      if (!contact_pair_warp(ps, k, prediction, init_dirs, out, has, queue, qcount, err, final_dirs, w, &phase, &gjk_iters,
                             &epa_iters, &epa_calls))
        break;
      continue;
    }
    const unsigned long long base = (item - n_large) * 32ull;
    if (base >= n_small) break;
    const uint64_t idx = base + lane;
    if (idx < n_small)
      contact_pair_lane(sh, pairs, order ? order[idx] : idx, prediction, init_dirs, out, has, queue, qcount, err, final_dirs, &gjk_iters,
                        le);
  }
  if (stats) {
    const uint32_t g = __reduce_add_sync(0xffffffffu, gjk_iters);
    const uint32_t e = __reduce_add_sync(0xffffffffu, epa_iters + le.iters);
    const uint32_t c = __reduce_add_sync(0xffffffffu, epa_calls + le.calls);
    if (lane == 0) {
      if (g) atomicAdd(&stats[0], (unsigned long long)g);
      if (e) atomicAdd(&stats[1], (unsigned long long)e);
      if (c) atomicAdd(&stats[2], (unsigned long long)c);
    }
  }
}

// EPA of the queued pairs. Regular pass (BIG = false): queue entries [*qstart, *qcount) (qstart
// NULL: from 0); a pair whose polytope outgrows the regular slot is appended to `ovf` (its result
// left to the second pass).
// Second pass (BIG = true): the entries listed in `ovf` [0, *qcount), on large slots; a pair that
// outgrows those raises the capacity error.
// MINB: resident blocks per SM the registers are budgeted for (8: the compiler's choice, about 126
// registers; 12 or 16: at most 85 or 64 registers, more warps to hide memory latency).
template <bool BIG, int MINB = 8>
__global__ void __launch_bounds__(EPA_THREADS, MINB) k_contacts_epa(ShapeArrays sh, const uint32_t* __restrict__ pairs, float prediction,
                                                              float* __restrict__ out, uint8_t* __restrict__ has,
                                                              const uint32_t* __restrict__ queue, const unsigned long long* __restrict__ qcount,
                                                              uint32_t* __restrict__ ws_pool, unsigned long long* __restrict__ stats,
                                                              uint32_t* __restrict__ err, float* __restrict__ final_dirs,
                                                              uint32_t* __restrict__ ovf, unsigned long long* __restrict__ ovf_count,
                                                              const unsigned long long* __restrict__ qstart) {
  const uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x;
  auto ws = [&]() { if constexpr (BIG) return epa_slot_big(ws_pool, slot); else return epa_slot(ws_pool, slot); }();
  const unsigned long long total = *qcount, start = qstart ? *qstart : 0ull;
  uint32_t iters = 0, calls = 0;
  for (unsigned long long i = start + slot; i < total; i += (unsigned long long)gridDim.x * blockDim.x) {
    const unsigned long long e = BIG ? ovf[i] : i;
    const uint32_t* q = queue + (size_t)e * QUEUE_WORDS;
    uint64_t k = q[0];
    Simplex s;
    simplex_reset(s, CSO{});
    s.dim = (int)q[1];
    for (int i = 0; i <= s.dim; ++i) {
      const float* f = reinterpret_cast<const float*>(q + 2 + 9 * i);
      s.v[i] = CSO{v3(f[0], f[1], f[2]), v3(f[3], f[4], f[5]), v3(f[6], f[7], f[8])};
    }
    PairSetup ps;
    setup_pair(sh, pairs[2 * k], pairs[2 * k + 1], &ps);
    const int r = epa_pair(ws, ps, k, s, prediction, out, has, final_dirs, &iters);
    if (r == EPA_OVERFLOW) {  // the second pass counts and writes this pair
      if (BIG) atomicOr(err, ERR_POLYTOPE_FULL);
      else ovf[atomicAdd(ovf_count, 1ull)] = (uint32_t)e;
      continue;
    }
    calls++;
  }
  if (stats) {
    uint32_t w = __reduce_add_sync(0xffffffffu, iters);
    uint32_t cw = __reduce_add_sync(0xffffffffu, calls);
    if ((threadIdx.x & 31) == 0) {
      if (w) atomicAdd(&stats[1], (unsigned long long)w);
      if (cw) atomicAdd(&stats[2], (unsigned long long)cw);
    }
  }
}

// Shape::compute_aabb(pos).loosened(margin)
__global__ void k_shape_aabbs(ShapeArrays sh, uint64_t n, float margin, float* __restrict__ out, uint32_t* __restrict__ err) {
  uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (!valid_pair(sh, (uint32_t)i, (uint32_t)i)) {
    atomicOr(err, ERR_CAPACITY);
    for (int j = 0; j < 6; ++j) out[6 * i + j] = 0.0f;
    return;
  }
  ShapeDev s = load_shape(sh.types, sh.params, sh.pool, (uint32_t)i);
  Pose p = load_pose(sh.poses, (uint32_t)i);
  V3 mn, mx;
  shape_world_aabb(s, p, &mn, &mx);
  if (margin > 0.0f) {
    mn = mn + v3(-margin, -margin, -margin);
    mx = mx + v3(margin, margin, margin);
  }
  float* o = out + 6 * i;
  o[0] = mn.x; o[1] = mn.y; o[2] = mn.z; o[3] = mx.x; o[4] = mx.y; o[5] = mx.z;
}

// Pairs cost at least this (vertices per support evaluation, two shapes) run one warp per pair
// unless the context's configuration says otherwise.
constexpr uint32_t DEFAULT_CONTACT_WARP_COST = 1024;

// k_contacts_fused on a persistent grid: as many blocks as fit on every SM with `smem` bytes of
// shared memory each.
// With inline EPA the context's EPA workspace pool is grown to one slot per thread of the grid.
parrygpu_status launch_fused(parrygpu_ctx* ctx, size_t smem, bool inline_epa, const ShapeArrays& sh, const uint32_t* pairs, uint64_t n,
                             const uint32_t* order, const unsigned long long* n_large, float prediction, const float* init_dirs, float* out,
                             uint8_t* has, uint32_t* queue, unsigned long long* qcount, unsigned long long* stats, float* final_dirs,
                             unsigned long long* work, uint32_t* ovf, unsigned long long* ovf_count) {
  auto kern = inline_epa ? k_contacts_fused<true> : k_contacts_fused<false>;
  if (smem > 48 * 1024) PG_CUDA(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  PG_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, FUSED_THREADS, smem));
  if (per_sm < 1) return set_error(ctx, PARRYGPU_CUDA_ERROR, "the fused contact kernel does not fit on an SM");
  const uint64_t sms = ctx->sm_count > 0 ? (uint64_t)ctx->sm_count : 152u;
  const uint64_t need = div_up(n, (uint64_t)FUSED_THREADS);
  const uint32_t blocks = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(sms * (uint64_t)per_sm, need));
  if (inline_epa) PG_CUDA(ctx, ctx->epa_ws.reserve((size_t)blocks * FUSED_THREADS * EPA_SLOT_BYTES));
  kern<<<blocks, FUSED_THREADS, smem, ctx->stream>>>(sh, pairs, n, order, n_large, prediction, init_dirs, out, has, queue, qcount, stats,
                                                     ctx->d_err, final_dirs, work, ctx->epa_ws.as<uint32_t>(), ovf, ovf_count);
  PG_LAUNCHED(ctx);
  return PARRYGPU_OK;
}

}  // namespace

parrygpu_status pg::stage_shapes(parrygpu_ctx* ctx, const parrygpu_shapes* s, ShapeArrays* out, bool defer_pool) {
  if (!s) return set_error(ctx, PARRYGPU_INVALID_ARG, "shapes is null");
  const void *t, *p, *q, *v;
  parrygpu_status st;
  if ((st = stage_input(ctx, ctx->stage_in[0], s->types, (size_t)s->n * 4, &t)) != PARRYGPU_OK) return st;
  if ((st = stage_input(ctx, ctx->stage_in[1], s->params, (size_t)s->n * 16, &p)) != PARRYGPU_OK) return st;
  if ((st = stage_input(ctx, ctx->stage_in[2], s->poses, (size_t)s->n * 28, &q)) != PARRYGPU_OK) return st;
  if (defer_pool && s->n_vertices && s->vertices && !is_device_ptr(s->vertices)) {
    if (on_other_device(s->vertices, ctx->device))
      return set_error(ctx, PARRYGPU_INVALID_ARG, "an input buffer lives on another GPU than the context's device %d", ctx->device);
    PG_CUDA(ctx, ctx->stage_in[3].reserve((size_t)s->n_vertices * 12));
    v = ctx->stage_in[3].ptr;
  } else if ((st = stage_input(ctx, ctx->stage_in[3], s->vertices, (size_t)s->n_vertices * 12, &v)) != PARRYGPU_OK) {
    return st;
  }
  if (((uintptr_t)p & 15) != 0) return set_error(ctx, PARRYGPU_INVALID_ARG, "shape params must be 16-byte aligned");
  *out = ShapeArrays{(const uint32_t*)t, (const float4*)p, (const float*)q, (const float*)v, s->n, s->n_vertices, PolyArrays{}};
  if (const parrygpu_polyhedra* ph = s->polyhedra) {
    PolyArrays& pa = out->poly;
    const void* d[9];
    const void* src[9] = {ph->hulls, ph->face_normals, ph->face_ranges, ph->face_vertices, ph->face_edges, ph->vertex_ranges,
                          ph->vertex_faces, ph->vertex_edges, ph->edge_dirs};
    size_t bytes[9] = {(size_t)ph->n_hulls * 32, (size_t)ph->n_faces * 12, (size_t)ph->n_faces * 8, (size_t)ph->n_face_entries * 4,
                       (size_t)ph->n_face_entries * 4, (size_t)s->n_vertices * 8, (size_t)ph->n_vertex_entries * 4,
                       (size_t)ph->n_vertex_entries * 4, (size_t)ph->n_edges * 12};
    for (int k = 0; k < 9; ++k)
      if ((st = stage_input(ctx, ctx->stage_poly[k], src[k], bytes[k], &d[k])) != PARRYGPU_OK) return st;
    pa.hulls = (const uint32_t*)d[0];
    pa.face_normals = (const float*)d[1];
    pa.face_ranges = (const uint32_t*)d[2];
    pa.face_vertices = (const uint32_t*)d[3];
    pa.face_edges = (const uint32_t*)d[4];
    pa.vertex_ranges = (const uint32_t*)d[5];
    pa.vertex_faces = (const uint32_t*)d[6];
    pa.vertex_edges = (const uint32_t*)d[7];
    pa.edge_dirs = (const float*)d[8];
    pa.n_hulls = ph->n_hulls;
    pa.n_faces = ph->n_faces;
    pa.n_face_entries = ph->n_face_entries;
    pa.n_vertex_entries = ph->n_vertex_entries;
    pa.n_edges = ph->n_edges;
  }
  return PARRYGPU_OK;
}

parrygpu_status pg::launch_shape_aabbs(parrygpu_ctx* ctx, const ShapeArrays& sh, uint64_t n, float margin, float* d_out) {
  if (n == 0) return PARRYGPU_OK;
  k_shape_aabbs<<<div_up(n, 256), 256, 0, ctx->stream>>>(sh, n, margin, d_out, ctx->d_err);
  PG_LAUNCHED(ctx);
  return PARRYGPU_OK;
}

parrygpu_status compound_part_aabbs(parrygpu_ctx* ctx, const parrygpu_compound* c, float* d_out) {
  ShapeArrays sh{c->types.as<uint32_t>(), c->params.as<float4>(), c->poses.as<float>(), c->pool.as<float>(), c->n, c->n_vertices};
  k_shape_aabbs<<<div_up(c->n, 256), 256, 0, ctx->stream>>>(sh, c->n, 0.0f, d_out, ctx->d_err);
  PG_LAUNCHED(ctx);
  return PARRYGPU_OK;
}

// Host shapes, pairs and outputs on a large batch: the vertex pool (most of the bytes) goes up in
// pieces on a copy stream while the context stream runs the pairs in chunks. A chunk's cost sort
// and GJK launch wait for the piece that completes the pool range its pairs reference (read back
// from a small kernel over the staged pairs before the chunks are queued). The EPA pass runs over
// the queue entries appended since the previous pass after the first chunk, after the third and
// after the last: the stream then alternates GJK chunks, whose pieces arrive about one chunk's
// GJK time apart, with EPA passes long enough to cover the next pieces' uploads, and each pass
// pays one tail (its last long polytopes). The large-slot pass and the output copies run once at
// the end. Every pair runs the kernels of the single-shot call on the same values, so the
// answers are the same.
constexpr uint64_t CT_PIPE_CHUNKS = 8;
constexpr uint64_t CT_PIPE_MIN = 131072;  // pairs per chunk at least
constexpr uint64_t CT_PIPE_PIECES = 16;

static parrygpu_status contacts_pipelined(parrygpu_ctx* ctx, const parrygpu_shapes* shapes, const ShapeArrays& sh, const uint32_t* dp,
                                   const float* di, uint64_t n_pairs, float prediction, float* d_out, uint8_t* d_has, float* d_dirs) {
  if (!ctx->up_stream) {
    PG_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->up_stream, cudaStreamNonBlocking));
    PG_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->down_stream, cudaStreamNonBlocking));
    for (cudaEvent_t& e : ctx->pipe_ev) PG_CUDA(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    if (!ctx->ev_fork) {
      PG_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming));
      PG_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming));
    }
  }
  if (!ctx->h_pipe) PG_CUDA(ctx, cudaMallocHost(&ctx->h_pipe, parrygpu_ctx::PIPE_EVENTS * sizeof(unsigned long long)));
  static_assert(CT_PIPE_CHUNKS <= parrygpu_ctx::PIPE_EVENTS && CT_PIPE_PIECES <= parrygpu_ctx::PIPE_EVENTS, "one event per piece");
  cudaStream_t main = ctx->stream;
  // the pool pieces, after the work already queued on the context stream (the staging buffer's last readers)
  const uint64_t nv = sh.n_vertices;
  const char* host_pool = static_cast<const char*>(static_cast<const void*>(shapes->vertices));
  char* dev_pool = ctx->stage_in[3].as<char>();
  uint64_t piece_end[CT_PIPE_PIECES];
  PG_CUDA(ctx, cudaEventRecord(ctx->ev_fork, main));
  PG_CUDA(ctx, cudaStreamWaitEvent(ctx->up_stream, ctx->ev_fork, 0));
  uint64_t prev = 0;
  for (uint64_t p = 0; p < CT_PIPE_PIECES; ++p) {
    const uint64_t end = nv * (p + 1) / CT_PIPE_PIECES;
    piece_end[p] = end;
    if (end > prev)
      PG_CUDA(ctx, cudaMemcpyAsync(dev_pool + 12 * prev, host_pool + 12 * prev, 12 * (end - prev), cudaMemcpyHostToDevice, ctx->up_stream));
    PG_CUDA(ctx, cudaEventRecord(ctx->pipe_ev[p], ctx->up_stream));
    prev = end;
  }
  // chunk sizes (multiples of 256) and the pool range each chunk references
  uint64_t chunks = CT_PIPE_CHUNKS;
  while (chunks > 2 && n_pairs / chunks < CT_PIPE_MIN) --chunks;
  const uint64_t chunk = div_up(div_up(n_pairs, chunks), (uint64_t)256) * 256;
  chunks = div_up(n_pairs, chunk);
  PG_CUDA(ctx, ctx->misc.reserve(parrygpu_ctx::PIPE_EVENTS * sizeof(unsigned long long)));
  unsigned long long* d_ends = ctx->misc.as<unsigned long long>();
  PG_CUDA(ctx, cudaMemsetAsync(d_ends, 0, chunks * sizeof(unsigned long long), main));
  k_chunk_vertex_ends<<<div_up(n_pairs, 256), 256, 0, main>>>(sh, dp, n_pairs, chunk, d_ends);
  PG_LAUNCHED(ctx);
  PG_CUDA(ctx, cudaMemcpyAsync(ctx->h_pipe, d_ends, chunks * sizeof(unsigned long long), cudaMemcpyDeviceToHost, main));
  PG_CUDA(ctx, cudaStreamSynchronize(main));
  // scratch: the EPA queue and overflow list hold the whole batch, the sort one chunk
  parrygpu_status s;
  PG_CUDA(ctx, ctx->ct_queue.reserve((size_t)n_pairs * QUEUE_WORDS * 4));
  PG_CUDA(ctx, ctx->ct_counters.reserve(128));
  PG_CUDA(ctx, ctx->ct_ovf.reserve((size_t)n_pairs * 4));
  uint32_t epa_per_sm = ctx->cfg.epa_blocks_per_sm ? ctx->cfg.epa_blocks_per_sm : 8;
  if (epa_per_sm > 32) epa_per_sm = 32;
  const uint32_t epa_blocks = (uint32_t)(ctx->sm_count > 0 ? ctx->sm_count : 152) * epa_per_sm;
  PG_CUDA(ctx, ctx->epa_ws.reserve((size_t)epa_blocks * EPA_THREADS * EPA_SLOT_BYTES));
  PG_CUDA(ctx, ctx->epa_ws_big.reserve((size_t)EPA_BIG_SLOTS * EPA_BIG_SLOT_BYTES));
  if ((s = radix_sort_reserve(ctx, (uint32_t)chunk)) != PARRYGPU_OK) return s;
  // [0] queue count, [1..3] stats, [4] overflow count, [5] work counter, [6] costly pairs, [8] EPA pass start
  unsigned long long* ctr = ctx->ct_counters.as<unsigned long long>();
  PG_CUDA(ctx, cudaMemsetAsync(ctr, 0, 128, main));
  const uint32_t warp_cost = ctx->cfg.contact_warp_cost ? ctx->cfg.contact_warp_cost : DEFAULT_CONTACT_WARP_COST;
  const bool warp_path = warp_cost < 1024;
  const size_t smem = warp_path ? sizeof(WarpSmem) * FUSED_WARPS : 0;
  auto epa = epa_per_sm <= 8 ? k_contacts_epa<false, 8> : (epa_per_sm <= 12 ? k_contacts_epa<false, 12> : k_contacts_epa<false, 16>);
  unsigned long long need = 0;
  for (uint64_t c = 0; c < chunks; ++c) {
    const uint64_t off = c * chunk, m = n_pairs - off < chunk ? n_pairs - off : chunk;
    need = ctx->h_pipe[c] > need ? ctx->h_pipe[c] : need;
    const uint64_t need_v = need < nv ? need : nv;
    if (need_v) {
      uint64_t p = 0;
      while (piece_end[p] < need_v) ++p;
      PG_CUDA(ctx, cudaStreamWaitEvent(main, ctx->pipe_ev[p], 0));
    }
    PG_CUDA(ctx, cudaMemsetAsync(ctr + 5, 0, 16, main));
    k_pair_cost_keys<<<div_up(m, (uint64_t)256), 256, 0, main>>>(sh, dp, (uint32_t)off, (uint32_t)m, ctx->sort_k[0].as<uint32_t>(),
                                                                 ctx->sort_v[0].as<uint32_t>());
    PG_LAUNCHED(ctx);
    int rb;
    if ((s = radix_sort_pairs(ctx, (uint32_t)m, 10, &rb)) != PARRYGPU_OK) return s;
    if (warp_path) {
      k_count_costly<<<1, 32, 0, main>>>(ctx->sort_k[rb].as<uint32_t>(), (uint32_t)m, warp_cost, ctr + 6);
      PG_LAUNCHED(ctx);
    }
    if ((s = launch_fused(ctx, smem, false, sh, dp, m, ctx->sort_v[rb].as<uint32_t>(), ctr + 6, prediction, di, d_out, d_has,
                          ctx->ct_queue.as<uint32_t>(), ctr, nullptr, d_dirs, ctr + 5, ctx->ct_ovf.as<uint32_t>(), ctr + 4)) != PARRYGPU_OK)
      return s;
    if (c == 0 || c == 2 || c + 1 == chunks) {
      epa<<<epa_blocks, EPA_THREADS, 0, main>>>(sh, dp, prediction, d_out, d_has, ctx->ct_queue.as<uint32_t>(), ctr,
                                                ctx->epa_ws.as<uint32_t>(), nullptr, ctx->d_err, d_dirs, ctx->ct_ovf.as<uint32_t>(), ctr + 4,
                                                ctr + 8);
      PG_LAUNCHED(ctx);
      PG_CUDA(ctx, cudaMemcpyAsync(ctr + 8, ctr, sizeof(unsigned long long), cudaMemcpyDeviceToDevice, main));
    }
  }
  k_contacts_epa<true><<<EPA_BIG_SLOTS / EPA_THREADS, EPA_THREADS, 0, main>>>(
      sh, dp, prediction, d_out, d_has, ctx->ct_queue.as<uint32_t>(), ctr + 4, ctx->epa_ws_big.as<uint32_t>(), nullptr, ctx->d_err, d_dirs,
      ctx->ct_ovf.as<uint32_t>(), nullptr, nullptr);
  PG_LAUNCHED(ctx);
  // every piece is in before the call returns (a tail of the pool that no pair references included)
  PG_CUDA(ctx, cudaEventRecord(ctx->ev_join, ctx->up_stream));
  PG_CUDA(ctx, cudaStreamWaitEvent(main, ctx->ev_join, 0));
  return PARRYGPU_OK;
}

extern "C" {

parrygpu_status parrygpu_shapes_aabbs(parrygpu_ctx* ctx, const parrygpu_shapes* shapes, float margin, float* aabbs) {
  if (!ctx || !shapes) return PARRYGPU_INVALID_ARG;
  if (shapes->n == 0) return PARRYGPU_OK;
  if (!aabbs) return set_error(ctx, PARRYGPU_INVALID_ARG, "aabbs is null");
  PG_CUDA(ctx, cudaSetDevice(ctx->device));
  ShapeArrays sh;
  parrygpu_status s = stage_shapes(ctx, shapes, &sh);
  if (s != PARRYGPU_OK) return s;
  void* d_out;
  bool copy;
  if ((s = stage_output(ctx, ctx->stage_out[0], aabbs, (size_t)shapes->n * 24, &d_out, &copy)) != PARRYGPU_OK) return s;
  KernelTimer kt(ctx, "shape_aabbs");
  k_shape_aabbs<<<div_up(shapes->n, 256), 256, 0, ctx->stream>>>(sh, shapes->n, margin, (float*)d_out, ctx->d_err);
  kt.stop();
  PG_LAUNCHED(ctx);
  if (copy) {
    PG_CUDA(ctx, cudaMemcpyAsync(aabbs, d_out, (size_t)shapes->n * 24, cudaMemcpyDeviceToHost, ctx->stream));
  }
  if (copy || sh.types != shapes->types || sh.poses != shapes->poses) return parrygpu_sync(ctx);
  return PARRYGPU_OK;
}

parrygpu_status parrygpu_contacts(parrygpu_ctx* ctx, const parrygpu_shapes* shapes, const uint32_t* pairs, uint64_t n_pairs,
                                  float prediction, const float* init_dirs, parrygpu_contact* out, uint8_t* has_contact,
                                  parrygpu_gjk_stats* stats) {
  return parrygpu_contacts_with_dirs(ctx, shapes, pairs, n_pairs, prediction, init_dirs, out, has_contact, stats, nullptr);
}

parrygpu_status parrygpu_contacts_with_dirs(parrygpu_ctx* ctx, const parrygpu_shapes* shapes, const uint32_t* pairs, uint64_t n_pairs,
                                            float prediction, const float* init_dirs, parrygpu_contact* out, uint8_t* has_contact,
                                            parrygpu_gjk_stats* stats, float* final_dirs) {
  if (!ctx || !shapes) return PARRYGPU_INVALID_ARG;
  if (stats) std::memset(stats, 0, sizeof(*stats));
  if (n_pairs == 0) return PARRYGPU_OK;
  if (!pairs || !out || !has_contact) return set_error(ctx, PARRYGPU_INVALID_ARG, "pairs, out and has_contact are required");
  PG_CUDA(ctx, cudaSetDevice(ctx->device));
  // a host vertex pool on a large batch: its upload overlapped with the kernels (no statistics or timing asked)
  const bool pipe = !stats && !ctx->timing && ctx->cfg.contact_epa_inline != 1 && n_pairs >= 2 * CT_PIPE_MIN && n_pairs < 0xffffffffull &&
                    shapes->n_vertices && shapes->vertices && !is_device_ptr(shapes->vertices);
  ShapeArrays sh;
  parrygpu_status s = stage_shapes(ctx, shapes, &sh, pipe);
  if (s != PARRYGPU_OK) return s;
  const void *dp, *di = nullptr;
  if ((s = stage_input(ctx, ctx->stage_in[4], pairs, (size_t)n_pairs * 8, &dp)) != PARRYGPU_OK) return s;
  if (init_dirs && (s = stage_input(ctx, ctx->stage_in[5], init_dirs, (size_t)n_pairs * 12, &di)) != PARRYGPU_OK) return s;
  void *d_out, *d_has;
  bool c_out, c_has;
  if ((s = stage_output(ctx, ctx->stage_out[0], out, (size_t)n_pairs * 52, &d_out, &c_out)) != PARRYGPU_OK) return s;
  if ((s = stage_output(ctx, ctx->stage_out[1], has_contact, (size_t)n_pairs, &d_has, &c_has)) != PARRYGPU_OK) return s;
  void* d_dirs = nullptr;
  bool c_dirs = false;
  if ((s = stage_output(ctx, ctx->stage_out[2], final_dirs, (size_t)n_pairs * 12, &d_dirs, &c_dirs)) != PARRYGPU_OK) return s;
  if (pipe) {
    if ((s = contacts_pipelined(ctx, shapes, sh, (const uint32_t*)dp, (const float*)di, n_pairs, prediction, (float*)d_out, (uint8_t*)d_has,
                                (float*)d_dirs)) != PARRYGPU_OK)
      return s;
    if (c_out) PG_CUDA(ctx, cudaMemcpyAsync(out, d_out, (size_t)n_pairs * 52, cudaMemcpyDeviceToHost, ctx->stream));
    if (c_has) PG_CUDA(ctx, cudaMemcpyAsync(has_contact, d_has, (size_t)n_pairs, cudaMemcpyDeviceToHost, ctx->stream));
    if (c_dirs) PG_CUDA(ctx, cudaMemcpyAsync(final_dirs, d_dirs, (size_t)n_pairs * 12, cudaMemcpyDeviceToHost, ctx->stream));
    return parrygpu_sync(ctx);
  }
  const bool inline_epa = ctx->cfg.contact_epa_inline == 1;
  PG_CUDA(ctx, ctx->ct_queue.reserve((size_t)n_pairs * QUEUE_WORDS * 4));
  PG_CUDA(ctx, ctx->ct_counters.reserve(64));
  uint32_t epa_per_sm = ctx->cfg.epa_blocks_per_sm ? ctx->cfg.epa_blocks_per_sm : 8;
  if (epa_per_sm > 32) epa_per_sm = 32;
  uint32_t epa_blocks = (uint32_t)(ctx->sm_count > 0 ? ctx->sm_count : 152) * epa_per_sm;
  uint32_t slots = epa_blocks * EPA_THREADS;
  PG_CUDA(ctx, ctx->epa_ws.reserve((size_t)slots * EPA_SLOT_BYTES));
  PG_CUDA(ctx, ctx->epa_ws_big.reserve((size_t)EPA_BIG_SLOTS * EPA_BIG_SLOT_BYTES));
  PG_CUDA(ctx, ctx->ct_ovf.reserve((size_t)n_pairs * 4));
  unsigned long long* ctr = ctx->ct_counters.as<unsigned long long>();  // [0] queue count, [1..3] stats, [4] overflow count
  PG_CUDA(ctx, cudaMemsetAsync(ctr, 0, 64, ctx->stream));
  // pairs binned by support-scan cost (a 10-bit key, two radix passes)
  const uint32_t* order = nullptr;
  int sorted_buf = 0;
  if (n_pairs > 4096 && n_pairs < 0xffffffffull) {
    uint32_t n = (uint32_t)n_pairs;
    if ((s = radix_sort_reserve(ctx, n)) != PARRYGPU_OK) return s;
    KernelTimer kt(ctx, "contacts_bin");
    k_pair_cost_keys<<<div_up(n, 256), 256, 0, ctx->stream>>>(sh, (const uint32_t*)dp, 0u, n, ctx->sort_k[0].as<uint32_t>(),
                                                                ctx->sort_v[0].as<uint32_t>());
    PG_LAUNCHED(ctx);
    int rb;
    if ((s = radix_sort_pairs(ctx, n, 10, &rb)) != PARRYGPU_OK) return s;
    kt.stop();
    order = ctx->sort_v[rb].as<uint32_t>();
    sorted_buf = rb;
  }
  {
    // warp-per-pair threshold: pairs of the sorted order whose cost reaches it (counted on the device)
    const uint32_t warp_cost = ctx->cfg.contact_warp_cost ? ctx->cfg.contact_warp_cost : DEFAULT_CONTACT_WARP_COST;
    const bool warp_path = order && warp_cost < 1024;
    KernelTimer kt(ctx, "contacts_gjk");
    if (warp_path) {
      k_count_costly<<<1, 32, 0, ctx->stream>>>(ctx->sort_k[sorted_buf].as<uint32_t>(), (uint32_t)n_pairs, warp_cost, ctr + 6);
      PG_LAUNCHED(ctx);
    }
    const size_t smem = warp_path ? sizeof(WarpSmem) * FUSED_WARPS : 0;
    if ((s = launch_fused(ctx, smem, inline_epa, sh, (const uint32_t*)dp, n_pairs, order, ctr + 6, prediction, (const float*)di,
                          (float*)d_out, (uint8_t*)d_has, ctx->ct_queue.as<uint32_t>(), ctr, ctr + 1, (float*)d_dirs, ctr + 5,
                          ctx->ct_ovf.as<uint32_t>(), ctr + 4)) != PARRYGPU_OK)
      return s;
    kt.stop();
  }
  {
    KernelTimer kt(ctx, "contacts_epa");
    if (!inline_epa) {
      auto kern = epa_per_sm <= 8 ? k_contacts_epa<false, 8> : (epa_per_sm <= 12 ? k_contacts_epa<false, 12> : k_contacts_epa<false, 16>);
      kern<<<epa_blocks, EPA_THREADS, 0, ctx->stream>>>(sh, (const uint32_t*)dp, prediction, (float*)d_out, (uint8_t*)d_has,
                                                        ctx->ct_queue.as<uint32_t>(), ctr, ctx->epa_ws.as<uint32_t>(), ctr + 1, ctx->d_err,
                                                        (float*)d_dirs, ctx->ct_ovf.as<uint32_t>(), ctr + 4, nullptr);
      PG_LAUNCHED(ctx);
    }
    // pairs whose polytope outgrew the regular slots, on the large slots (an empty list exits at once)
    k_contacts_epa<true><<<EPA_BIG_SLOTS / EPA_THREADS, EPA_THREADS, 0, ctx->stream>>>(
        sh, (const uint32_t*)dp, prediction, (float*)d_out, (uint8_t*)d_has, ctx->ct_queue.as<uint32_t>(), ctr + 4,
        ctx->epa_ws_big.as<uint32_t>(), ctr + 1, ctx->d_err, (float*)d_dirs, ctx->ct_ovf.as<uint32_t>(), nullptr, nullptr);
    kt.stop();
    PG_LAUNCHED(ctx);
  }
  if (c_out) PG_CUDA(ctx, cudaMemcpyAsync(out, d_out, (size_t)n_pairs * 52, cudaMemcpyDeviceToHost, ctx->stream));
  if (c_has) PG_CUDA(ctx, cudaMemcpyAsync(has_contact, d_has, (size_t)n_pairs, cudaMemcpyDeviceToHost, ctx->stream));
  if (c_dirs) PG_CUDA(ctx, cudaMemcpyAsync(final_dirs, d_dirs, (size_t)n_pairs * 12, cudaMemcpyDeviceToHost, ctx->stream));
  if (stats) {
    unsigned long long h[4];
    PG_CUDA(ctx, cudaMemcpyAsync(h, ctr, 32, cudaMemcpyDeviceToHost, ctx->stream));
    PG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    stats->gjk_iterations = h[1];
    stats->epa_iterations = h[2];
    stats->epa_calls = h[3];
  }
  bool staged_in = sh.types != shapes->types || sh.params != (const float4*)shapes->params || sh.poses != shapes->poses ||
                   dp != pairs || (init_dirs && di != init_dirs) || (shapes->n_vertices && sh.pool != shapes->vertices);
  if (c_out || c_has || c_dirs || stats || staged_in) return parrygpu_sync(ctx);
  return PARRYGPU_OK;
}

}  // extern "C"
