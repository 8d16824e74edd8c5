// Stable LSD radix sort of (u32 key, u32 value) pairs, written for the LBVH build (30-bit Morton
// keys) and for ray / pair ordering. 8-bit digits, 2048-key tiles:
//   1. per-tile digit histogram (shared-memory atomics), stored digit-major: hist[d * tiles + t]
//   2. one exclusive scan over the digit-major array -> global offset of (digit, tile)
//   3. per-tile stable scatter: each 256-key round ranks keys within a warp with __match_any_sync,
//      warps are ordered by a shared-memory prefix over per-warp digit counts.
#include "internal.hpp"

namespace {

constexpr int RS_BINS = 256;
constexpr int RS_THREADS = 256;
constexpr int RS_ITEMS = 8;
constexpr int RS_TILE = RS_THREADS * RS_ITEMS;
constexpr int RS_WARPS = RS_THREADS / 32;
constexpr int SCAN_THREADS = 1024;

__global__ void __launch_bounds__(RS_THREADS) k_rs_hist(const uint32_t* __restrict__ keys, uint32_t n, int shift,
                                                        uint32_t* __restrict__ hist, uint32_t tiles) {
  __shared__ uint32_t h[RS_BINS];
  h[threadIdx.x] = 0;
  __syncthreads();
  uint32_t base = blockIdx.x * (uint32_t)RS_TILE;
#pragma unroll 4
  for (int r = 0; r < RS_ITEMS; ++r) {
    uint32_t i = base + r * RS_THREADS + threadIdx.x;
    if (i < n) atomicAdd(&h[(keys[i] >> shift) & 0xffu], 1u);
  }
  __syncthreads();
  hist[threadIdx.x * tiles + blockIdx.x] = h[threadIdx.x];
}

// Exclusive scan of the digit-major histogram (m = tiles * 256 entries, a multiple of 4) in one
// block: 4096-entry chunks, 4 consecutive entries per thread (one 16-byte load), warp-shuffle scans,
// a running carry between chunks.
__global__ void __launch_bounds__(SCAN_THREADS) k_rs_scan(uint32_t* __restrict__ data, uint32_t m) {
  __shared__ uint32_t warp_sums[SCAN_THREADS / 32];
  __shared__ uint32_t carry;
  const uint32_t tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  if (tid == 0) carry = 0;
  __syncthreads();
  for (uint32_t base = 0; base < m; base += SCAN_THREADS * 4) {
    uint32_t idx = base + tid * 4;
    uint4 v = make_uint4(0, 0, 0, 0);
    if (idx < m) v = *reinterpret_cast<const uint4*>(data + idx);
    uint32_t t = v.x + v.y + v.z + v.w;
    uint32_t incl = t;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= (uint32_t)o) incl += y;
    }
    if (lane == 31) warp_sums[w] = incl;
    __syncthreads();
    if (w == 0) {
      uint32_t ws = warp_sums[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, ws, o);
        if (lane >= (uint32_t)o) ws += y;
      }
      warp_sums[lane] = ws;  // inclusive over warps
    }
    __syncthreads();
    uint32_t excl = carry + (w ? warp_sums[w - 1] : 0u) + (incl - t);
    if (idx < m) {
      uint4 o;
      o.x = excl;
      o.y = excl + v.x;
      o.z = o.y + v.y;
      o.w = o.z + v.z;
      *reinterpret_cast<uint4*>(data + idx) = o;
    }
    __syncthreads();
    if (tid == 0) carry += warp_sums[SCAN_THREADS / 32 - 1];
    __syncthreads();
  }
}

__global__ void __launch_bounds__(RS_THREADS) k_rs_scatter(const uint32_t* __restrict__ kin, const uint32_t* __restrict__ vin,
                                                           uint32_t* __restrict__ kout, uint32_t* __restrict__ vout, uint32_t n,
                                                           int shift, const uint32_t* __restrict__ hist, uint32_t tiles) {
  __shared__ uint32_t digit_base[RS_BINS];
  __shared__ uint32_t round_total[RS_BINS];
  __shared__ uint32_t warp_cnt[RS_WARPS][RS_BINS];
  __shared__ uint32_t warp_off[RS_WARPS][RS_BINS];
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  digit_base[tid] = hist[tid * tiles + blockIdx.x];
#pragma unroll
  for (int ww = 0; ww < RS_WARPS; ++ww) warp_cnt[ww][tid] = 0;
  __syncthreads();
  const uint32_t base = blockIdx.x * (uint32_t)RS_TILE;
  const unsigned lt_mask = (1u << lane) - 1u;
  for (int r = 0; r < RS_ITEMS; ++r) {
    if (base + r * RS_THREADS >= n) break;  // uniform across the block
    uint32_t i = base + r * RS_THREADS + tid;
    bool valid = i < n;
    uint32_t k = valid ? kin[i] : 0u;
    uint32_t v = valid ? vin[i] : 0u;
    uint32_t d = valid ? ((k >> shift) & 0xffu) : (256u + lane);
    unsigned peers = __match_any_sync(0xffffffffu, d);
    uint32_t rank = __popc(peers & lt_mask);
    if (valid && rank == 0) warp_cnt[w][d] = __popc(peers);
    __syncthreads();
    {
      uint32_t off = 0;
#pragma unroll
      for (int ww = 0; ww < RS_WARPS; ++ww) {
        uint32_t c = warp_cnt[ww][tid];
        warp_off[ww][tid] = off;
        off += c;
      }
      round_total[tid] = off;
    }
    __syncthreads();
    if (valid) {
      uint32_t pos = digit_base[d] + warp_off[w][d] + rank;
      kout[pos] = k;
      vout[pos] = v;
    }
    __syncthreads();
    digit_base[tid] += round_total[tid];
#pragma unroll
    for (int ww = 0; ww < RS_WARPS; ++ww) warp_cnt[ww][tid] = 0;
    __syncthreads();
  }
}

}  // namespace

parrygpu_status radix_sort_reserve(parrygpu_ctx* ctx, uint32_t n) {
  size_t bytes = (size_t)(n ? n : 1) * 4;
  for (int i = 0; i < 2; ++i) {
    PG_CUDA(ctx, ctx->sort_k[i].reserve(bytes));
    PG_CUDA(ctx, ctx->sort_v[i].reserve(bytes));
  }
  uint32_t tiles = div_up(n ? n : 1, RS_TILE);
  PG_CUDA(ctx, ctx->sort_hist.reserve((size_t)tiles * RS_BINS * 4));
  return PARRYGPU_OK;
}

parrygpu_status radix_sort_pairs(parrygpu_ctx* ctx, uint32_t n, int key_bits, int* result_buf) {
  *result_buf = 0;
  if (n <= 1) return PARRYGPU_OK;
  parrygpu_status s = radix_sort_reserve(ctx, n);
  if (s != PARRYGPU_OK) return s;
  uint32_t tiles = div_up(n, RS_TILE);
  uint32_t* hist = ctx->sort_hist.as<uint32_t>();
  int cur = 0;
  for (int shift = 0; shift < key_bits; shift += 8) {
    const uint32_t* kin = ctx->sort_k[cur].as<uint32_t>();
    const uint32_t* vin = ctx->sort_v[cur].as<uint32_t>();
    uint32_t* kout = ctx->sort_k[cur ^ 1].as<uint32_t>();
    uint32_t* vout = ctx->sort_v[cur ^ 1].as<uint32_t>();
    k_rs_hist<<<tiles, RS_THREADS, 0, ctx->stream>>>(kin, n, shift, hist, tiles);
    PG_LAUNCHED(ctx);
    k_rs_scan<<<1, SCAN_THREADS, 0, ctx->stream>>>(hist, tiles * RS_BINS);
    PG_LAUNCHED(ctx);
    k_rs_scatter<<<tiles, RS_THREADS, 0, ctx->stream>>>(kin, vin, kout, vout, n, shift, hist, tiles);
    PG_LAUNCHED(ctx);
    cur ^= 1;
  }
  *result_buf = cur;
  return PARRYGPU_OK;
}

// Same sort on caller-provided buffers (k0/v0 hold the input; k1/v1 and hist are scratch of at least
// n and 256 * ceil(n / 2048) entries). Allocates nothing.
parrygpu_status radix_sort_pairs_in(parrygpu_ctx* ctx, uint32_t n, int key_bits, uint32_t* k0, uint32_t* v0, uint32_t* k1,
                                    uint32_t* v1, uint32_t* hist, int* result_buf) {
  *result_buf = 0;
  if (n <= 1) return PARRYGPU_OK;
  uint32_t tiles = div_up(n, RS_TILE);
  uint32_t* ks[2] = {k0, k1};
  uint32_t* vs[2] = {v0, v1};
  int cur = 0;
  for (int shift = 0; shift < key_bits; shift += 8) {
    k_rs_hist<<<tiles, RS_THREADS, 0, ctx->stream>>>(ks[cur], n, shift, hist, tiles);
    PG_LAUNCHED(ctx);
    k_rs_scan<<<1, SCAN_THREADS, 0, ctx->stream>>>(hist, tiles * RS_BINS);
    PG_LAUNCHED(ctx);
    k_rs_scatter<<<tiles, RS_THREADS, 0, ctx->stream>>>(ks[cur], vs[cur], ks[cur ^ 1], vs[cur ^ 1], n, shift, hist, tiles);
    PG_LAUNCHED(ctx);
    cur ^= 1;
  }
  *result_buf = cur;
  return PARRYGPU_OK;
}

uint32_t radix_sort_hist_entries(uint32_t n) { return div_up(n ? n : 1, RS_TILE) * RS_BINS; }

// In-place exclusive prefix sum of `m` words in one block (the buffer holds m rounded up to a
// multiple of 4 words, the padding zeroed).
namespace {

constexpr uint32_t MSCAN_THREADS = 256;
constexpr uint32_t MSCAN_TILE = MSCAN_THREADS * 16;  // words per block

// Sum of each tile of `data` (m words, a multiple of 4) into sums[tile].
__global__ void __launch_bounds__(MSCAN_THREADS) k_mscan_reduce(const uint32_t* __restrict__ data, uint32_t m, uint32_t* __restrict__ sums) {
  __shared__ uint32_t ws[MSCAN_THREADS / 32];
  const uint32_t base = blockIdx.x * MSCAN_TILE, tid = threadIdx.x;
  uint32_t t = 0;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const uint32_t idx = base + (j * MSCAN_THREADS + tid) * 4;
    if (idx < m) {
      const uint4 v = *reinterpret_cast<const uint4*>(data + idx);
      t += v.x + v.y + v.z + v.w;
    }
  }
  t = __reduce_add_sync(0xffffffffu, t);
  if ((tid & 31) == 0) ws[tid >> 5] = t;
  __syncthreads();
  if (tid < 32) {
    uint32_t v = tid < MSCAN_THREADS / 32 ? ws[tid] : 0u;
    v = __reduce_add_sync(0xffffffffu, v);
    if (tid == 0) sums[blockIdx.x] = v;
  }
}

// Exclusive scan of each tile in place, offset by the tile's scanned sum: 4 consecutive words per
// thread per step, warp-shuffle scans, a running carry over the tile's 4 steps.
__global__ void __launch_bounds__(MSCAN_THREADS) k_mscan_tiles(uint32_t* __restrict__ data, uint32_t m, const uint32_t* __restrict__ offs) {
  __shared__ uint32_t ws[MSCAN_THREADS / 32];
  __shared__ uint32_t carry;
  const uint32_t tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  if (tid == 0) carry = offs[blockIdx.x];
  __syncthreads();
  for (int j = 0; j < 4; ++j) {
    const uint32_t idx = blockIdx.x * MSCAN_TILE + (j * MSCAN_THREADS + tid) * 4;
    uint4 v = make_uint4(0u, 0u, 0u, 0u);
    if (idx < m) v = *reinterpret_cast<const uint4*>(data + idx);
    const uint32_t t = v.x + v.y + v.z + v.w;
    uint32_t incl = t;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= (uint32_t)o) incl += y;
    }
    if (lane == 31) ws[w] = incl;
    __syncthreads();
    if (w == 0) {
      uint32_t x = lane < MSCAN_THREADS / 32 ? ws[lane] : 0u;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (uint32_t)o) x += y;
      }
      if (lane < MSCAN_THREADS / 32) ws[lane] = x;
    }
    __syncthreads();
    const uint32_t excl = carry + (w ? ws[w - 1] : 0u) + (incl - t);
    if (idx < m) {
      uint4 o;
      o.x = excl;
      o.y = excl + v.x;
      o.z = o.y + v.y;
      o.w = o.z + v.z;
      *reinterpret_cast<uint4*>(data + idx) = o;
    }
    __syncthreads();
    if (tid == 0) carry += ws[MSCAN_THREADS / 32 - 1];
    __syncthreads();
  }
}

}  // namespace

uint32_t exclusive_scan_u32_sums(uint32_t m) { return (m + MSCAN_TILE - 1) / MSCAN_TILE + 4; }

parrygpu_status exclusive_scan_u32_wide(parrygpu_ctx* ctx, uint32_t* data, uint32_t m, uint32_t* sums) {
  if (m == 0) return PARRYGPU_OK;
  m = (m + 3u) & ~3u;
  const uint32_t tiles = (m + MSCAN_TILE - 1) / MSCAN_TILE;
  k_mscan_reduce<<<tiles, MSCAN_THREADS, 0, ctx->stream>>>(data, m, sums);
  PG_LAUNCHED(ctx);
  PG_CUDA(ctx, cudaMemsetAsync(sums + tiles, 0, ((tiles + 3u) & ~3u) * 4 - tiles * 4 + 4, ctx->stream));
  k_rs_scan<<<1, SCAN_THREADS, 0, ctx->stream>>>(sums, (tiles + 3u) & ~3u);
  PG_LAUNCHED(ctx);
  k_mscan_tiles<<<tiles, MSCAN_THREADS, 0, ctx->stream>>>(data, m, sums);
  PG_LAUNCHED(ctx);
  return PARRYGPU_OK;
}

parrygpu_status exclusive_scan_u32(parrygpu_ctx* ctx, uint32_t* data, uint32_t m) {
  if (m == 0) return PARRYGPU_OK;
  k_rs_scan<<<1, SCAN_THREADS, 0, ctx->stream>>>(data, (m + 3u) & ~3u);
  PG_LAUNCHED(ctx);
  return PARRYGPU_OK;
}
