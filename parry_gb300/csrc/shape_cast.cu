// Batched linear shape casting: query::cast_shapes (time of impact of two shapes under
// translational motion) for ball and support-map pairs. Paths relative to the parry repository:
//   src/query/shape_cast/shape_cast.rs:230-286                 ShapeCastOptions, cast_shapes
//   src/query/default_query_dispatcher.rs:434-538              dispatch (ball-ball, support maps)
//   src/query/shape_cast/shape_cast_ball_ball.rs:10-69
//   src/query/shape_cast/shape_cast_support_map_support_map.rs:12-69
//   src/query/gjk/gjk.rs:632-657, 660-795                      directional_distance, minkowski_ray_cast
//   src/shape/round_shape.rs:330-349                           RoundShapeRef support (target_distance > 0)
//
// One thread per pair, persistent over the pair list so that each thread owns an EPA workspace
// slot: a pair found penetrating (toi below 1e-5) needs the contact geometry, whose EPA runs on that
// slot. Every expression keeps the reference's evaluation order (--fmad=false).
#include "internal.hpp"
#include "epa_device.cuh"
#include "contact_device.cuh"
#include "gjk_reg.cuh"

#include <cstring>

using namespace pg;

namespace {

constexpr int SC_THREADS = 64;
enum : uint32_t { CAST_OUT_OF_ITERATIONS = 0, CAST_CONVERGED = 1, CAST_FAILED = 2, CAST_PENETRATING = 3, CAST_NONE = 255 };

struct CastOptions {
  float max_toi, target;
  bool stop_at_penetration, geometry_on_penetration;
};

// SupportMap::local_support_point_toward for a unit direction (ball.rs:247-249, capsule.rs:412-418;
// the others forward to local_support_point, support_map.rs:302).
__device__ __forceinline__ V3 local_support_toward(const ShapeDev& s, V3 u) {
  if (s.type == SH_BALL) return u * s.a;
  if (s.type == SH_CAPSULE) {
    V3 a = v3(0.f, -s.a, 0.f), b = v3(0.f, s.a, 0.f);
    if (dot(u, a) > dot(u, b)) return a + u * s.b;
    return b + u * s.b;
  }
  return local_support(s, u);
}

// CSOPoint::from_shapes(pos12, g1, g2, dir) with g1 = RoundShapeRef(g1, border) when round.
__device__ __forceinline__ CSO cast_cso(const Pose& pos12, const ShapeDev& g1, bool round, float border, const ShapeDev& g2, V3 dir) {
  V3 sp1;
  if (round) {
    V3 u = normalize(dir);  // Unit::new_normalize
    sp1 = local_support_toward(g1, u) + u * border;
  } else {
    sp1 = local_support(g1, dir);
  }
  V3 sp2 = world_support(g2, pos12, -dir);
  return CSO{sp1 - sp2, sp1, sp2};
}

// ray_halfspace.rs: toi of the ray with the plane through `center` of normal `normal`, if >= 0.
__device__ __forceinline__ bool ray_toi_with_halfspace(V3 center, V3 normal, V3 o, V3 d, float* t) {
  V3 dpos = center - o;
  float denom = dot(normal, d);
  if (fabsf(denom) <= EPS) return false;
  float tt = dot(normal, dpos) / denom;
  if (tt >= 0.0f) { *t = tt; return true; }
  return false;
}

// gjk.rs:660-795 minkowski_ray_cast of the ray (origin, rd) with max_toi = f32::MAX on
// g1 - pos12 * g2; leaves the simplex as the reference does (directional_distance reads it). The
// simplex is a RegSimplex (gjk_reg.cuh) kept in registers: the loop is inlined into the kernel.
__device__ __forceinline__ bool minkowski_ray_cast(const Pose& pos12, const ShapeDev& g1, bool round, float border, const ShapeDev& g2,
                                                   V3 rd, RegSimplex<true>& s, float* toi_out, V3* n_out) {
  const float eps_tol = GJK_EPS_TOL;
  const float eps_rel = sqrtf(eps_tol);
  float ray_length = norm(rd);
  if (fabsf(ray_length) <= EPS) return false;
  float ltoi = 0.0f;
  V3 co = v3(0.f, 0.f, 0.f), cd = rd / ray_length;
  V3 dir = -cd;
  V3 ldir = dir;
  CSO sp = cast_cso(pos12, g1, round, border, g2, dir);
  rs_reset(s, CSO{sp.p - co, sp.o1, sp.o2});
  V3 proj = rs_project_origin_and_reduce(s);
  float max_bound = FLT_MAX;
  int niter = 0;
  bool last_chance = false;
  for (;;) {
    float old_max_bound = max_bound;
    float nb;
    V3 u;
    if (try_normalize(-proj, eps_tol, &u, &nb)) { dir = u; max_bound = nb; }
    else { *toi_out = ltoi / ray_length; *n_out = ldir; return true; }
    CSO support;
    if (max_bound >= old_max_bound) {
      last_chance = true;
      V3 p = proj + co;
      support = CSO{p, p, v3(0.f, 0.f, 0.f)};
    } else {
      support = cast_cso(pos12, g1, round, border, g2, dir);
    }
    if (last_chance && ltoi > 0.0f) { *toi_out = ltoi / ray_length; *n_out = ldir; return true; }
    float t;
    if (ray_toi_with_halfspace(support.p, dir, co, cd, &t)) {
      if (dot(dir, cd) < 0.0f && t > 0.0f) {
        ldir = dir;
        ltoi += t;
        if (ltoi / ray_length > FLT_MAX) return false;
        V3 shift = cd * t;
        co = co + shift;
        max_bound = FLT_MAX;
        rs_translate(s, -shift);
        last_chance = false;
      }
    } else {
      if (dot(dir, cd) > eps_tol) return false;
    }
    if (last_chance) return false;
    float min_bound = -dot(dir, support.p - co);
    if (max_bound - min_bound <= eps_rel * max_bound) return false;
    rs_add(s, CSO{support.p - co, support.o1, support.o2});
    proj = rs_project_origin_and_reduce(s);
    if (s.dim == 3) {
      if (min_bound >= eps_tol) return false;
      *toi_out = ltoi / ray_length; *n_out = ldir; return true;
    }
    niter += 1;
    if (niter == 100) return false;
  }
}

struct CastHit {
  float toi;
  V3 w1, w2, n1, n2;
  uint32_t status;
};

// shape_cast_ball_ball.rs:10-69
__device__ __forceinline__ bool cast_ball_ball(const Pose& pos12, V3 vel12, float r1, float r2, const CastOptions& opt, CastHit* h) {
  float rsum = (r1 + r2) + opt.target;
  float radius = rsum;
  V3 center = -pos12.t;
  // ray_toi_with_ball(center, radius, Ray(origin, vel12), solid = true): dcenter = origin - center
  V3 dcenter = pos12.t;
  float a = dot(vel12, vel12);
  float b = dot(dcenter, vel12);
  float c = dot(dcenter, dcenter) - radius * radius;
  bool inside;
  float toi;
  if (a == 0.0f) {
    if (c > 0.0f) return false;
    inside = true;
    toi = 0.0f;
  } else {
    if (c > 0.0f && b > 0.0f) return false;
    float delta = b * b - a * c;
    if (delta < 0.0f) return false;
    float t = (-b - sqrtf(delta)) / a;
    if (t <= 0.0f) { inside = true; toi = 0.0f; }
    else { inside = false; toi = t; }
  }
  if (toi > opt.max_toi) return false;
  V3 dpt = vel12 * toi - center;  // ray.point_at(toi) - center
  V3 n1, n2, w1 = v3(0.f, 0.f, 0.f), w2 = v3(0.f, 0.f, 0.f);
  if (radius == 0.0f) {
    n1 = v3(1.f, 0.f, 0.f);
    n2 = pose_inv_rotate(pos12, v3(-1.f, 0.f, 0.f));
  } else {
    n1 = dpt / radius;
    n2 = pose_inv_rotate(pos12, -n1);
    w1 = n1 * r1;
    w2 = n2 * r2;
  }
  if (!opt.stop_at_penetration && toi < 1.0e-5f && dot(n1, vel12) >= 0.0f) return false;
  uint32_t status = (inside && dot(center, center) < rsum * rsum) ? CAST_PENETRATING : CAST_CONVERGED;
  *h = CastHit{toi, w1, w2, n1, n2, status};
  return true;
}

// shape_cast_support_map_support_map.rs:12-69 (+ gjk::directional_distance, gjk.rs:632-657).
// Returns false for None; *epa_overflow when the penetration contact outgrew the workspace.
__device__ __forceinline__ bool cast_support_maps(const EpaWs& ws, const Pose& pos12, V3 vel12, const ShapeDev& g1, const ShapeDev& g2,
                                                  const CastOptions& opt, CastHit* h, uint32_t* gjk_iters, uint32_t* epa_iters,
                                                  uint32_t* epa_calls, bool* epa_overflow) {
  RegSimplex<true> s;
  float toi;
  V3 normal1;
  if (!minkowski_ray_cast(pos12, g1, opt.target > 0.0f, opt.target, g2, vel12, s, &toi, &normal1)) return false;
  V3 w1 = v3(0.f, 0.f, 0.f), w2 = v3(0.f, 0.f, 0.f);
  if (toi != 0.0f) rs_witness(s, s.dim == 3, &w1, &w2);
  if (toi > opt.max_toi) return false;
  if ((opt.geometry_on_penetration || !opt.stop_at_penetration) && toi < 1.0e-5f) {
    // contact_support_map_support_map(pos12, g1, g2, f32::MAX)
    V3 dir;
    if (!try_normalize(pos12.t, EPS, &dir)) dir = v3(1.f, 0.f, 0.f);
    Simplex cs;
    simplex_reset(cs, cso_from_shapes(pos12, g1, g2, dir));
    GjkOut g = gjk_closest_points(pos12, g1, g2, FLT_MAX, cs, gjk_iters);
    V3 p1, p2, n;
    if (g.kind == GJK_CLOSEST) {
      p1 = g.p1; p2 = g.p2; n = g.dir;
    } else if (g.kind == GJK_INTERSECTION) {
      (*epa_calls)++;
      int r = epa_closest_points(ws, pos12, g1, g2, cs, &p1, &p2, &n, epa_iters);
      if (r == EPA_OVERFLOW) { *epa_overflow = true; return false; }
      if (r != EPA_OK) return false;
    } else {
      return false;
    }
    // Contact: point1 = p1, point2 = pos12^-1 p2, normal1 = n, normal2 = pos12^-1 (-n)
    V3 c_n2 = pose_inv_rotate(pos12, -n);
    if (!opt.stop_at_penetration && dot(n, vel12) >= 0.0f) return false;
    *h = CastHit{toi, p1, pose_inv_point(pos12, p2), n, c_n2, CAST_PENETRATING};
    return true;
  }
  h->toi = toi;
  h->n1 = normal1;
  h->n2 = pose_inv_rotate(pos12, -normal1);
  h->w1 = w1 - normal1 * opt.target;
  h->w2 = pose_inv_point(pos12, w2);
  h->status = toi == 0.0f ? CAST_PENETRATING : CAST_CONVERGED;
  return true;
}

// MINB = resident blocks of SC_THREADS per SM the register budget is cut for: 4 leaves the inlined
// ray cast all the registers it wants, 6 caps it at 168 (a few spills, more warps per SM).
template <int MINB>
__global__ void __launch_bounds__(SC_THREADS, MINB) k_cast_shapes(ShapeArrays sh, const uint32_t* __restrict__ pairs, uint64_t n,
                                                            const float* __restrict__ vels, CastOptions opt, float* __restrict__ out,
                                                            uint8_t* __restrict__ status, uint32_t* __restrict__ ws_pool,
                                                            unsigned long long* __restrict__ stats, uint32_t* __restrict__ err) {
  const uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x;
  EpaWs ws = epa_slot(ws_pool, slot);
  uint32_t gi = 0, ei = 0, ec = 0;
  for (uint64_t k = slot; k < n; k += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t a = pairs[2 * k], b = pairs[2 * k + 1];
    float* o = out + 13 * k;
    CastHit h;
    bool ok = false;
    if (!valid_pair(sh, a, b)) {
      atomicOr(err, ERR_CAPACITY);
    } else {
      ShapeDev s1 = load_shape(sh.types, sh.params, sh.pool, a);
      ShapeDev s2 = load_shape(sh.types, sh.params, sh.pool, b);
      Pose p1 = load_pose(sh.poses, a), p2 = load_pose(sh.poses, b);
      Pose pos12 = pose_inv_mul(p1, p2);
      V3 v1 = v3(vels[3 * (size_t)a], vels[3 * (size_t)a + 1], vels[3 * (size_t)a + 2]);
      V3 v2 = v3(vels[3 * (size_t)b], vels[3 * (size_t)b + 1], vels[3 * (size_t)b + 2]);
      V3 vel12 = pose_inv_rotate(p1, v2 - v1);
      if (s1.type == SH_BALL && s2.type == SH_BALL) {
        ok = cast_ball_ball(pos12, vel12, s1.a, s2.a, opt, &h);
      } else {
        bool overflow = false;
        ok = cast_support_maps(ws, pos12, vel12, s1, s2, opt, &h, &gi, &ei, &ec, &overflow);
        if (overflow) atomicOr(err, ERR_POLYTOPE_FULL);
      }
    }
    if (ok) {
      o[0] = h.toi;
      o[1] = h.w1.x; o[2] = h.w1.y; o[3] = h.w1.z;
      o[4] = h.w2.x; o[5] = h.w2.y; o[6] = h.w2.z;
      o[7] = h.n1.x; o[8] = h.n1.y; o[9] = h.n1.z;
      o[10] = h.n2.x; o[11] = h.n2.y; o[12] = h.n2.z;
      status[k] = (uint8_t)h.status;
    } else {
#pragma unroll
      for (int j = 0; j < 13; ++j) o[j] = 0.0f;
      status[k] = (uint8_t)CAST_NONE;
    }
  }
  if (stats) {
    uint32_t w0 = __reduce_add_sync(0xffffffffu, gi), w1 = __reduce_add_sync(0xffffffffu, ei), w2 = __reduce_add_sync(0xffffffffu, ec);
    if ((threadIdx.x & 31) == 0) {
      if (w0) atomicAdd(&stats[0], (unsigned long long)w0);
      if (w1) atomicAdd(&stats[1], (unsigned long long)w1);
      if (w2) atomicAdd(&stats[2], (unsigned long long)w2);
    }
  }
}

}  // namespace

extern "C" parrygpu_status parrygpu_cast_shapes(parrygpu_ctx* ctx, const parrygpu_shapes* shapes, const uint32_t* pairs, uint64_t n_pairs,
                                                const float* velocities, const parrygpu_shape_cast_options* options,
                                                parrygpu_shape_cast_hit* out, uint8_t* status, parrygpu_gjk_stats* stats) {
  if (!ctx || !shapes || !options) return PARRYGPU_INVALID_ARG;
  if (stats) std::memset(stats, 0, sizeof(*stats));
  if (n_pairs == 0) return PARRYGPU_OK;
  if (!pairs || !velocities || !out || !status) return set_error(ctx, PARRYGPU_INVALID_ARG, "pairs, velocities, out and status are required");
  PG_CUDA(ctx, cudaSetDevice(ctx->device));
  ShapeArrays sh;
  parrygpu_status s = stage_shapes(ctx, shapes, &sh);
  if (s != PARRYGPU_OK) return s;
  const void *dp, *dv;
  if ((s = stage_input(ctx, ctx->stage_in[4], pairs, (size_t)n_pairs * 8, &dp)) != PARRYGPU_OK) return s;
  if ((s = stage_input(ctx, ctx->stage_in[5], velocities, (size_t)shapes->n * 12, &dv)) != PARRYGPU_OK) return s;
  void *d_out, *d_status;
  bool c_out, c_status;
  if ((s = stage_output(ctx, ctx->stage_out[0], out, (size_t)n_pairs * 52, &d_out, &c_out)) != PARRYGPU_OK) return s;
  if ((s = stage_output(ctx, ctx->stage_out[1], status, (size_t)n_pairs, &d_status, &c_status)) != PARRYGPU_OK) return s;
  uint32_t per_sm = ctx->cfg.epa_blocks_per_sm ? ctx->cfg.epa_blocks_per_sm : 8;
  uint32_t blocks = (uint32_t)(ctx->sm_count > 0 ? ctx->sm_count : 152) * per_sm;
  const uint64_t need = (n_pairs + SC_THREADS - 1) / SC_THREADS;
  if (blocks > need) blocks = (uint32_t)need;
  PG_CUDA(ctx, ctx->epa_ws.reserve((size_t)blocks * SC_THREADS * EPA_SLOT_BYTES));
  PG_CUDA(ctx, ctx->ct_counters.reserve(64));
  unsigned long long* ctr = ctx->ct_counters.as<unsigned long long>();
  PG_CUDA(ctx, cudaMemsetAsync(ctr, 0, 64, ctx->stream));
  CastOptions opt{options->max_time_of_impact, options->target_distance, options->stop_at_penetration != 0,
                  options->compute_impact_geometry_on_penetration != 0};
  {
    KernelTimer kt(ctx, "cast_shapes");
    // the persistent grid's residency decides the register budget
    if (per_sm <= 4)
      k_cast_shapes<4><<<blocks, SC_THREADS, 0, ctx->stream>>>(sh, (const uint32_t*)dp, n_pairs, (const float*)dv, opt, (float*)d_out,
                                                               (uint8_t*)d_status, ctx->epa_ws.as<uint32_t>(), ctr, ctx->d_err);
    else
      k_cast_shapes<6><<<blocks, SC_THREADS, 0, ctx->stream>>>(sh, (const uint32_t*)dp, n_pairs, (const float*)dv, opt, (float*)d_out,
                                                               (uint8_t*)d_status, ctx->epa_ws.as<uint32_t>(), ctr, ctx->d_err);
    kt.stop();
    PG_LAUNCHED(ctx);
  }
  if (c_out) PG_CUDA(ctx, cudaMemcpyAsync(out, d_out, (size_t)n_pairs * 52, cudaMemcpyDeviceToHost, ctx->stream));
  if (c_status) PG_CUDA(ctx, cudaMemcpyAsync(status, d_status, (size_t)n_pairs, cudaMemcpyDeviceToHost, ctx->stream));
  if (stats) {
    unsigned long long h[3];
    PG_CUDA(ctx, cudaMemcpyAsync(h, ctr, 24, cudaMemcpyDeviceToHost, ctx->stream));
    PG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    stats->gjk_iterations = h[0];
    stats->epa_iterations = h[1];
    stats->epa_calls = h[2];
  }
  if (c_out || c_status || stats || dp != pairs || dv != velocities) return parrygpu_sync(ctx);
  return PARRYGPU_OK;
}
