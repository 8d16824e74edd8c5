// Launch-configuration autotuner (no reference counterpart: parry runs on the CPU).
//
// The answers of every query are independent of the launch configuration (ray ordering, threads
// per block, EPA residency): those only change how the same per-ray / per-pair work maps onto the
// SMs. The best choice depends on the workload (ray coherence, mesh size against L2, how many
// pairs reach EPA), so the tuner times each candidate on the caller's own inputs with CUDA events
// on the context stream and keeps the fastest in the context's configuration.
#include "internal.hpp"

#include <cstring>

namespace {

// One untimed run, then `reps` runs between two events; *ms = mean milliseconds per run.
template <class F>
parrygpu_status time_runs(parrygpu_ctx* ctx, uint32_t reps, F run, float* ms) {
  parrygpu_status s = run();
  if (s != PARRYGPU_OK) return s;
  cudaEvent_t a = nullptr, b = nullptr;
  cudaError_t e = cudaEventCreate(&a);
  if (e == cudaSuccess) e = cudaEventCreate(&b);
  if (e == cudaSuccess) e = cudaEventRecord(a, ctx->stream);
  for (uint32_t r = 0; r < reps && e == cudaSuccess && s == PARRYGPU_OK; ++r) s = run();
  if (e == cudaSuccess) e = cudaEventRecord(b, ctx->stream);
  if (e == cudaSuccess) e = cudaEventSynchronize(b);
  float t = 0.0f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&t, a, b);
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  if (s != PARRYGPU_OK) return s;
  if (e != cudaSuccess) return check_cuda(ctx, e, "autotune timing");
  *ms = t / (float)(reps ? reps : 1);
  return PARRYGPU_OK;
}

struct RayCandidate {
  uint32_t sort_rays, ray_sort_key, ray_traversal, ray_block, ray_refill;
};

// Ray orderings: input order; 30-bit Morton code of the origin; direction octant above a 27-bit
// Morton code; top 16 bits of the Morton code. Each with one ray per thread and with postponed
// leaves, at 64 / 128 / 256 threads per block, and with the persistent dynamic-fetch traversal
// refilling at 8 / 16 / 24 idle lanes.
constexpr uint32_t SORTS[4][2] = {{0, 0}, {1, 0}, {1, 1}, {1, 2}};
constexpr uint32_t BLOCKS[3] = {64, 128, 256};
constexpr uint32_t REFILLS[3] = {8, 16, 24};

constexpr uint32_t EPA_CANDIDATES[] = {4, 6, 8, 12, 16};

}  // namespace

extern "C" {

parrygpu_status parrygpu_get_config(const parrygpu_ctx* ctx, parrygpu_config* out) {
  if (!ctx || !out) return PARRYGPU_INVALID_ARG;
  *out = ctx->cfg;
  return PARRYGPU_OK;
}

parrygpu_status parrygpu_autotune_trimesh_rays(parrygpu_ctx* ctx, const parrygpu_trimesh* mesh, const float* pose7, const float* rays,
                                               uint32_t n, float max_toi, uint32_t reps, parrygpu_config* chosen) {
  if (!ctx || !mesh || (n && !rays)) return PARRYGPU_INVALID_ARG;
  if (n == 0) {
    if (chosen) *chosen = ctx->cfg;
    return PARRYGPU_OK;
  }
  if (reps == 0) reps = 3;
  // Inputs copied once to the device, outputs kept on the device: the timed runs are the
  // device-resident call, the same for every candidate.
  DevBuf d_rays, d_feat, d_toi, d_nrm;
  auto release = [&]() { d_rays.release(); d_feat.release(); d_toi.release(); d_nrm.release(); };
  cudaError_t e = d_rays.reserve((size_t)n * 24);
  if (e == cudaSuccess) e = d_feat.reserve((size_t)n * 4);
  if (e == cudaSuccess) e = d_toi.reserve((size_t)n * 4);
  if (e == cudaSuccess) e = d_nrm.reserve((size_t)n * 12);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_rays.ptr, rays, (size_t)n * 24, cudaMemcpyDefault, ctx->stream);
  if (e != cudaSuccess) { release(); return check_cuda(ctx, e, "autotune ray buffers"); }
  const parrygpu_config saved = ctx->cfg;
  parrygpu_config best = saved;
  float best_ms = -1.0f;
  parrygpu_status s = PARRYGPU_OK;
  RayCandidate cands[4 * 9];
  int nc = 0;
  for (const auto& so : SORTS) {
    for (uint32_t b : BLOCKS) cands[nc++] = RayCandidate{so[0], so[1], 1u, b, 0u};
    for (uint32_t b : BLOCKS) cands[nc++] = RayCandidate{so[0], so[1], 3u, b, 0u};
    for (uint32_t f : REFILLS) cands[nc++] = RayCandidate{so[0], so[1], 2u, 0u, f};
  }
  for (int ci = 0; ci < nc; ++ci) {
    const RayCandidate& c = cands[ci];
    ctx->cfg.sort_rays = c.sort_rays;
    ctx->cfg.ray_sort_key = c.ray_sort_key;
    ctx->cfg.ray_traversal = c.ray_traversal;
    ctx->cfg.ray_block = c.ray_block;
    ctx->cfg.ray_refill = c.ray_refill;
    float ms = 0.0f;
    s = time_runs(ctx, reps, [&]() {
      return parrygpu_trimesh_cast_rays(ctx, mesh, pose7, d_rays.as<float>(), n, max_toi, 1, d_feat.as<uint32_t>(), d_toi.as<float>(),
                                        d_nrm.as<float>());
    }, &ms);
    if (s != PARRYGPU_OK) break;
    if (best_ms < 0.0f || ms < best_ms) { best_ms = ms; best = ctx->cfg; }
  }
  cudaError_t se = cudaStreamSynchronize(ctx->stream);
  release();
  if (s != PARRYGPU_OK) { ctx->cfg = saved; return s; }
  if (se != cudaSuccess) { ctx->cfg = saved; return check_cuda(ctx, se, "autotune"); }
  ctx->cfg = best;
  if (chosen) *chosen = best;
  return PARRYGPU_OK;
}

parrygpu_status parrygpu_autotune_contacts(parrygpu_ctx* ctx, const parrygpu_shapes* shapes, const uint32_t* pairs, uint64_t n_pairs,
                                           float prediction, uint32_t reps, parrygpu_config* chosen) {
  if (!ctx || !shapes || (n_pairs && !pairs)) return PARRYGPU_INVALID_ARG;
  if (n_pairs == 0) {
    if (chosen) *chosen = ctx->cfg;
    return PARRYGPU_OK;
  }
  if (reps == 0) reps = 2;
  DevBuf d_pairs, d_out, d_has;
  auto release = [&]() { d_pairs.release(); d_out.release(); d_has.release(); };
  cudaError_t e = d_pairs.reserve((size_t)n_pairs * 8);
  if (e == cudaSuccess) e = d_out.reserve((size_t)n_pairs * sizeof(parrygpu_contact));
  if (e == cudaSuccess) e = d_has.reserve((size_t)n_pairs);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_pairs.ptr, pairs, (size_t)n_pairs * 8, cudaMemcpyDefault, ctx->stream);
  if (e != cudaSuccess) { release(); return check_cuda(ctx, e, "autotune pair buffers"); }
  const parrygpu_config saved = ctx->cfg;
  parrygpu_config best = saved;
  float best_ms = -1.0f;
  parrygpu_status s = PARRYGPU_OK;
  auto trial = [&]() -> parrygpu_status {
    float ms = 0.0f;
    parrygpu_status st = time_runs(ctx, reps, [&]() {
      return parrygpu_contacts(ctx, shapes, d_pairs.as<uint32_t>(), n_pairs, prediction, nullptr, d_out.as<parrygpu_contact>(),
                               d_has.as<uint8_t>(), nullptr);
    }, &ms);
    if (st == PARRYGPU_OK && (best_ms < 0.0f || ms < best_ms)) { best_ms = ms; best = ctx->cfg; }
    return st;
  };
  // one thread per pair, EPA through the queue: each EPA residency
  ctx->cfg.contact_warp_cost = 1024;
  ctx->cfg.contact_epa_inline = 2;
  for (uint32_t blocks : EPA_CANDIDATES) {
    ctx->cfg.epa_blocks_per_sm = blocks;
    if ((s = trial()) != PARRYGPU_OK) break;
  }
  // then, at the best residency, the dearest pairs one warp each, and EPA right after GJK
  for (uint32_t variant = 0; variant < 3 && s == PARRYGPU_OK; ++variant) {
    ctx->cfg = best;
    if (variant < 2) ctx->cfg.contact_warp_cost = variant == 0 ? 512 : 256;
    else ctx->cfg.contact_epa_inline = 1;
    s = trial();
  }
  cudaError_t se = cudaStreamSynchronize(ctx->stream);
  release();
  if (s != PARRYGPU_OK) { ctx->cfg = saved; return s; }
  if (se != cudaSuccess) { ctx->cfg = saved; return check_cuda(ctx, se, "autotune"); }
  ctx->cfg = best;
  if (chosen) *chosen = best;
  return PARRYGPU_OK;
}

}  // extern "C"
