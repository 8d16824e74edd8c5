// Allocation-free variant of the batched TriMesh ray cast.
//
// Who needs it: callers that may not allocate device memory once they are running. A physics or
// rendering engine that owns the whole device-memory budget and hands out only its own buffers; a
// fixed-rate frame loop that must never block, where cudaMalloc can stall and cudaFree waits for the
// whole device to go idle; a host built on a custom allocator that forbids driver allocations after
// start-up. parrygpu_trimesh_cast_rays grows its ray-ordering scratch (Morton keys, sort ping-pong
// buffers, histograms) with cudaMalloc on first use and whenever a larger batch arrives; this entry
// point instead uses one fixed scratch array compiled into the library, so the only device memory it
// touches is the caller's inputs and outputs, the mesh and that array.
//
// The scratch is a file-scope __device__ array sized for PARRYGPU_NOALLOC_MAX_RAYS rays (about
// 4.3 MB). Every GPU that loads the library holds it until the process exits. All calls, from every
// context and stream of a device, share the same array, and it keeps the last call's contents:
// calls whose work overlaps on the GPU race on it, so issue them on one stream or synchronise
// between them.
#include "internal.hpp"
#include <mutex>

namespace {

constexpr uint32_t NA_MAX = PARRYGPU_NOALLOC_MAX_RAYS;
constexpr uint32_t NA_TILE = 2048;  // keys per radix-sort tile (sort.cu)
constexpr uint32_t NA_HIST = ((NA_MAX + NA_TILE - 1) / NA_TILE) * 256;
constexpr uint32_t NA_BOUNDS = 64;  // ray-origin bounds (words 0-5) and the traversal's ray counter (word 32), 256 bytes
constexpr size_t NA_WORDS = 4 * (size_t)NA_MAX + NA_HIST + NA_BOUNDS;

// keys0 | vals0 | keys1 | vals1 | histogram | bounds + ray counter
static __device__ __align__(256) uint32_t g_ray_scratch[NA_WORDS];

constexpr int NA_MAX_DEVICES = 64;
std::mutex g_setup_mutex;
uint32_t* g_scratch_addr[NA_MAX_DEVICES] = {};

// Device address of g_ray_scratch on `device` (which must be current). In host code the array's
// name is only a host-side stand-in, never a device address, so the address is looked up with
// cudaGetSymbolAddress. Outside stream capture it is looked up on every call (a lookup, no
// allocation, once the module is loaded), so an address made stale by cudaDeviceReset is never
// used; the cached value serves calls made while `stream` is being captured, which is why the first
// call on a device must come before any capture.
parrygpu_status scratch_for_device(parrygpu_ctx* ctx, int device, cudaStream_t stream, uint32_t** out) {
  if (device < 0 || device >= NA_MAX_DEVICES) return set_error(ctx, PARRYGPU_INVALID_ARG, "device ordinal %d out of range", device);
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  PG_CUDA(ctx, cudaStreamIsCapturing(stream, &cap));
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (cap == cudaStreamCaptureStatusNone) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_ray_scratch);
    if (e != cudaSuccess || !p) return check_cuda(ctx, e == cudaSuccess ? cudaErrorInvalidSymbol : e, "cudaGetSymbolAddress(ray scratch)");
    g_scratch_addr[device] = static_cast<uint32_t*>(p);
  } else if (!g_scratch_addr[device]) {
    return set_error(ctx, PARRYGPU_INVALID_ARG,
                     "parrygpu_trimesh_cast_rays_noalloc: the first call on device %d must come before any stream capture", device);
  }
  *out = g_scratch_addr[device];
  return PARRYGPU_OK;
}

// Device memory of the context's device, or managed memory.
bool on_ctx_device(const void* p, int device) { return is_device_ptr(p) && !on_other_device(p, device); }

}  // namespace

extern "C" parrygpu_status parrygpu_trimesh_cast_rays_noalloc(parrygpu_ctx* ctx, const parrygpu_trimesh* mesh, const float* pose7,
                                                               const float* rays, uint32_t n, float max_toi, int solid,
                                                               uint32_t* feature, float* toi, float* normal) {
  (void)solid;
  if (!ctx || !mesh) return PARRYGPU_INVALID_ARG;
  if (n > NA_MAX)
    return set_error(ctx, PARRYGPU_INVALID_ARG,
                     "parrygpu_trimesh_cast_rays_noalloc: %u rays exceed its fixed scratch of %u rays (PARRYGPU_NOALLOC_MAX_RAYS); "
                     "split the batch",
                     n, NA_MAX);
  if (n == 0) return PARRYGPU_OK;
  if (!rays || !feature || !toi) return set_error(ctx, PARRYGPU_INVALID_ARG, "rays, feature and toi are required");
  PG_CUDA(ctx, cudaSetDevice(ctx->device));
  const int dev = ctx->device;
  if (!on_ctx_device(rays, dev) || !on_ctx_device(feature, dev) || !on_ctx_device(toi, dev) || (normal && !on_ctx_device(normal, dev)))
    return set_error(ctx, PARRYGPU_INVALID_ARG,
                     "parrygpu_trimesh_cast_rays_noalloc needs rays and outputs in device memory of the context's GPU %d "
                     "(host buffers would need staging; another GPU's memory is not read in place)",
                     dev);
  if (pose7 && on_other_device(pose7, dev))
    return set_error(ctx, PARRYGPU_INVALID_ARG, "parrygpu_trimesh_cast_rays_noalloc: pose7 lives on another GPU than %d", dev);
  float pose_host[7];
  const float* pose_ptr = nullptr;
  if (pose7) {
    if (is_device_ptr(pose7)) {
      PG_CUDA(ctx, cudaMemcpyAsync(pose_host, pose7, sizeof(pose_host), cudaMemcpyDeviceToHost, ctx->stream));
      PG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    } else {
      for (int i = 0; i < 7; ++i) pose_host[i] = pose7[i];
    }
    pose_ptr = pose_host;
  }
  if (mesh->n_triangles == 0) {
    PG_CUDA(ctx, cudaMemsetAsync(feature, 0xff, (size_t)n * 4, ctx->stream));
    PG_CUDA(ctx, cudaMemsetAsync(toi, 0, (size_t)n * 4, ctx->stream));
    if (normal) PG_CUDA(ctx, cudaMemsetAsync(normal, 0, (size_t)n * 12, ctx->stream));
    return PARRYGPU_OK;
  }
  if (radix_sort_hist_entries(n) > NA_HIST) return set_error(ctx, PARRYGPU_INVALID_ARG, "sort histogram exceeds the fixed scratch");
  uint32_t* base = nullptr;
  parrygpu_status s = scratch_for_device(ctx, ctx->device, ctx->stream, &base);
  if (s != PARRYGPU_OK) return s;
  uint32_t* k0 = base;
  uint32_t* v0 = base + NA_MAX;
  uint32_t* k1 = base + 2 * (size_t)NA_MAX;
  uint32_t* v1 = base + 3 * (size_t)NA_MAX;
  uint32_t* hist = base + 4 * (size_t)NA_MAX;
  uint32_t* bounds = hist + NA_HIST;
  const uint32_t* order = nullptr;
  if (ctx->cfg.sort_rays && n > 1) {
    // launch_ray_keys clears the bounds words first; every histogram entry the sort reads is
    // rewritten by its histogram pass, and the keys/values are fully written before use.
    if ((s = launch_ray_keys(ctx, rays, n, bounds, k0, v0, ctx->cfg.ray_sort_key)) != PARRYGPU_OK) return s;
    int rb = 0;
    if ((s = radix_sort_pairs_in(ctx, n, ray_sort_bits(ctx), k0, v0, k1, v1, hist, &rb)) != PARRYGPU_OK) return s;
    order = rb ? v1 : v0;
  }
  return launch_trimesh_rays(ctx, mesh, pose_ptr, rays, order, n, max_toi, feature, toi, normal, bounds + 32);
}
