// Context, error reporting and host/device pointer staging for libparrygpu.
#include "internal.hpp"
#include <cstdarg>
#include <cstring>

parrygpu_status set_error(parrygpu_ctx* ctx, parrygpu_status s, const char* fmt, ...) {
  if (ctx) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    ctx->last_error = buf;
  }
  return s;
}

parrygpu_status check_cuda(parrygpu_ctx* ctx, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return PARRYGPU_OK;
  return set_error(ctx, PARRYGPU_CUDA_ERROR, "%s: %s", what, cudaGetErrorString(e));
}

bool is_device_ptr(const void* p) {
  if (!p) return false;
  cudaPointerAttributes a;
  cudaError_t e = cudaPointerGetAttributes(&a, p);
  if (e != cudaSuccess) { cudaGetLastError(); return false; }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

bool on_other_device(const void* p, int device) {
  if (!p) return false;
  cudaPointerAttributes a;
  cudaError_t e = cudaPointerGetAttributes(&a, p);
  if (e != cudaSuccess) { cudaGetLastError(); return false; }
  return a.type == cudaMemoryTypeDevice && a.device != device;
}

bool is_addressable(const void* p) {
  if (!p) return false;
  cudaPointerAttributes a;
  cudaError_t e = cudaPointerGetAttributes(&a, p);
  if (e != cudaSuccess) { cudaGetLastError(); return false; }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged || (a.type == cudaMemoryTypeHost && a.devicePointer);
}

void* device_view_ptr(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) { cudaGetLastError(); return const_cast<void*>(p); }
  return a.devicePointer ? a.devicePointer : const_cast<void*>(p);
}

parrygpu_status stage_input(parrygpu_ctx* ctx, DevBuf& buf, const void* src, size_t bytes, const void** dptr) {
  if (bytes == 0) { *dptr = src; return PARRYGPU_OK; }
  if (!src) return set_error(ctx, PARRYGPU_INVALID_ARG, "null input pointer");
  if (on_other_device(src, ctx->device))
    return set_error(ctx, PARRYGPU_INVALID_ARG, "an input buffer lives on another GPU than the context's device %d", ctx->device);
  if (is_device_ptr(src)) { *dptr = src; return PARRYGPU_OK; }
  PG_CUDA(ctx, buf.reserve(bytes));
  PG_CUDA(ctx, cudaMemcpyAsync(buf.ptr, src, bytes, cudaMemcpyHostToDevice, ctx->stream));
  *dptr = buf.ptr;
  return PARRYGPU_OK;
}

parrygpu_status stage_output(parrygpu_ctx* ctx, DevBuf& buf, void* dst, size_t bytes, void** dptr, bool* needs_copy) {
  *needs_copy = false;
  if (!dst) { *dptr = nullptr; return PARRYGPU_OK; }
  if (on_other_device(dst, ctx->device))
    return set_error(ctx, PARRYGPU_INVALID_ARG, "an output buffer lives on another GPU than the context's device %d", ctx->device);
  if (is_device_ptr(dst)) { *dptr = dst; return PARRYGPU_OK; }
  PG_CUDA(ctx, buf.reserve(bytes < 16 ? 16 : bytes));
  *dptr = buf.ptr;
  *needs_copy = true;
  return PARRYGPU_OK;
}

static void drop_pending(parrygpu_ctx* ctx) {
  for (auto& kv : ctx->pending)
    for (auto& ev : kv.second) { cudaEventDestroy(ev.first); cudaEventDestroy(ev.second); }
  ctx->pending.clear();
}

extern "C" {

void parrygpu_default_config(parrygpu_config* cfg) {
  if (!cfg) return;
  std::memset(cfg, 0, sizeof(*cfg));
  cfg->device = 0;
  cfg->ray_block = 0;
  cfg->sort_rays = 1;
}

parrygpu_status parrygpu_create(parrygpu_ctx** out, const parrygpu_config* cfg) {
  if (!out) return PARRYGPU_INVALID_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { cudaGetLastError(); return PARRYGPU_NO_DEVICE; }
  if (cfg && ((cfg->ray_block % 32) != 0 || cfg->ray_block > 1024 || cfg->ray_sort_key > 2 || cfg->epa_blocks_per_sm > 32 ||
              cfg->ray_traversal > 3 || cfg->ray_refill > 32 || cfg->ray_chunks > 64 || cfg->ray_host_access > 2 ||
              (cfg->contact_warp_cost != 0 && cfg->contact_warp_cost < 2) || cfg->contact_epa_inline > 2 || cfg->mlp_infer > 2 ||
              cfg->scene_ray_order > 3 ||
              cfg->scene_ray_grid > 2))
    return PARRYGPU_INVALID_ARG;
  parrygpu_ctx* ctx = new parrygpu_ctx();
  if (cfg) ctx->cfg = *cfg; else parrygpu_default_config(&ctx->cfg);
  ctx->device = ctx->cfg.device;
  if (ctx->device < 0 || ctx->device >= ndev) { delete ctx; return PARRYGPU_INVALID_ARG; }
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&ctx->d_err, sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMemset(ctx->d_err, 0, sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMallocHost(&ctx->h_err, sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, ctx->device);
  if (e == cudaSuccess) {
    int coherent = 0;
    e = cudaDeviceGetAttribute(&coherent, cudaDevAttrPageableMemoryAccessUsesHostPageTables, ctx->device);
    ctx->coherent_host = coherent != 0;
  }
  if (e != cudaSuccess) { delete ctx; return PARRYGPU_CUDA_ERROR; }
  ctx->stream = ctx->own_stream;
  *out = ctx;
  return PARRYGPU_OK;
}

void parrygpu_destroy(parrygpu_ctx* ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  for (auto* b : {&ctx->sort_k[0], &ctx->sort_k[1], &ctx->sort_v[0], &ctx->sort_v[1], &ctx->sort_hist, &ctx->misc,
                  &ctx->counters, &ctx->ray_keys, &ctx->ray_order})
    b->release();
  for (int i = 0; i < 8; ++i) ctx->stage_in[i].release();
  for (int i = 0; i < 4; ++i) ctx->stage_out[i].release();
  ctx->ct_queue.release();
  ctx->ct_counters.release();
  ctx->epa_ws.release();
  ctx->epa_ws_big.release();
  ctx->ct_ovf.release();
  for (DevBuf* d : {&ctx->mf.queue, &ctx->mf.counters, &ctx->mf.bins, &ctx->mf.epa_ws}) d->release();
  for (DevBuf* d : {&ctx->ray_wave.cands, &ctx->ray_wave.counter, &ctx->ray_wave.keys, &ctx->ray_wave.ovf}) d->release();
  if (ctx->d_err) cudaFree(ctx->d_err);
  if (ctx->h_err) cudaFreeHost(ctx->h_err);
  if (ctx->h_pipe) cudaFreeHost(ctx->h_pipe);
  drop_pending(ctx);
  if (ctx->aux_stream) { cudaStreamSynchronize(ctx->aux_stream); cudaStreamDestroy(ctx->aux_stream); }
  if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
  if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
  for (cudaStream_t s : {ctx->up_stream, ctx->down_stream})
    if (s) { cudaStreamSynchronize(s); cudaStreamDestroy(s); }
  for (cudaEvent_t e : ctx->pipe_ev)
    if (e) cudaEventDestroy(e);
  if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
  delete ctx;
}

parrygpu_status parrygpu_set_stream(parrygpu_ctx* ctx, void* stream) {
  if (!ctx) return PARRYGPU_INVALID_ARG;
  ctx->stream = stream ? (cudaStream_t)stream : ctx->own_stream;
  return PARRYGPU_OK;
}

parrygpu_status parrygpu_sync(parrygpu_ctx* ctx) {
  if (!ctx) return PARRYGPU_INVALID_ARG;
  PG_CUDA(ctx, cudaMemcpyAsync(ctx->h_err, ctx->d_err, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
  PG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  uint32_t err = *ctx->h_err;
  if (err) {
    PG_CUDA(ctx, cudaMemsetAsync(ctx->d_err, 0, sizeof(uint32_t), ctx->stream));
    PG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (err & ERR_TIMEOUT) return set_error(ctx, PARRYGPU_TIMEOUT, "a bounded device wait gave up");
    if (err & ERR_STACK_OVERFLOW) return set_error(ctx, PARRYGPU_STACK_OVERFLOW, "traversal stack overflow");
    if (err & ERR_CAPACITY) return set_error(ctx, PARRYGPU_CAPACITY_EXCEEDED, "output capacity exceeded");
    if (err & ERR_POLYTOPE_FULL) return set_error(ctx, PARRYGPU_CAPACITY_EXCEEDED, "EPA polytope capacity exceeded");
    if (err & ERR_BAD_INDEX) return set_error(ctx, PARRYGPU_INVALID_ARG, "a pair index or vertex range is out of bounds");
  }
  return PARRYGPU_OK;
}

const char* parrygpu_last_error(const parrygpu_ctx* ctx) { return ctx ? ctx->last_error.c_str() : "null context"; }

const char* parrygpu_status_string(parrygpu_status s) {
  switch (s) {
    case PARRYGPU_OK: return "ok";
    case PARRYGPU_INVALID_ARG: return "invalid argument";
    case PARRYGPU_UNSUPPORTED_PAIR: return "unsupported shape pair";
    case PARRYGPU_CAPACITY_EXCEEDED: return "capacity exceeded";
    case PARRYGPU_TIMEOUT: return "device wait timed out";
    case PARRYGPU_CUDA_ERROR: return "CUDA error";
    case PARRYGPU_STACK_OVERFLOW: return "traversal stack overflow";
    case PARRYGPU_NO_DEVICE: return "no CUDA device";
  }
  return "unknown status";
}

uint64_t parrygpu_kernel_launches(const parrygpu_ctx* ctx) { return ctx ? ctx->launches : 0; }

parrygpu_status parrygpu_enable_kernel_timing(parrygpu_ctx* ctx, int enable) {
  if (!ctx) return PARRYGPU_INVALID_ARG;
  ctx->timing = enable != 0;
  return PARRYGPU_OK;
}

parrygpu_status parrygpu_kernel_time(parrygpu_ctx* ctx, const char* kernel, double* total_ms, uint64_t* launches) {
  if (!ctx || !kernel) return PARRYGPU_INVALID_ARG;
  PG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  for (auto& kv : ctx->pending) {
    auto& acc = ctx->timed[kv.first];
    for (auto& ev : kv.second) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, ev.first, ev.second);
      acc.first += ms;
      acc.second += 1;
      cudaEventDestroy(ev.first);
      cudaEventDestroy(ev.second);
    }
  }
  ctx->pending.clear();
  auto it = ctx->timed.find(kernel);
  if (total_ms) *total_ms = it == ctx->timed.end() ? 0.0 : it->second.first;
  if (launches) *launches = it == ctx->timed.end() ? 0 : it->second.second;
  return PARRYGPU_OK;
}

parrygpu_status parrygpu_reset_kernel_timing(parrygpu_ctx* ctx) {
  if (!ctx) return PARRYGPU_INVALID_ARG;
  cudaStreamSynchronize(ctx->stream);
  drop_pending(ctx);
  ctx->timed.clear();
  return PARRYGPU_OK;
}

}  // extern "C"
