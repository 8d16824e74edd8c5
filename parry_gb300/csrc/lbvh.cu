// LBVH build, refit and pair traversal (partitioning::Bvh replacement).
//
// Build pipeline (one CUDA stream, no host round trip):
//   k_centroid_bounds  centroid bounds of the leaf AABBs (warp-reduced, order-preserving atomics)
//   k_morton           30-bit Morton code of each centroid on a cubic grid over the centroid bounds, value = leaf index
//   radix_sort_pairs   stable device radix sort (sort.cu); equal codes keep leaf-index order
//   k_karras           Karras (2012) hierarchy: internal node i owns wide node i, root = wide 0,
//                      exactly the reference's "root is BvhNodeWide 0" convention
//   k_fit              bottom-up AABB fit: one thread per leaf climbs; the second thread to reach
//                      a node (atomic arrival counter) merges both children and continues
// The tree is stored in the reference's BvhNodeWide layout (2 x 32-byte BvhNode: mins, children,
// maxs, data; src/partitioning/bvh/bvh_tree.rs:263-266, 456-467), read with float4 loads.
#include "internal.hpp"
#include "common.cuh"
#include "lbvh_device.cuh"

using namespace pg;

namespace {

constexpr int FIT_THREADS = 256;

__global__ void k_centroid_bounds(const float* __restrict__ aabbs, uint32_t n, uint32_t* __restrict__ bounds) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  float mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, mx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
  if (i < n) {
    const float* a = aabbs + 6 * (size_t)i;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      float c = (a[d] + a[3 + d]) * 0.5f;
      mn[d] = c; mx[d] = c;
    }
  }
#pragma unroll
  for (int d = 0; d < 3; ++d) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      mn[d] = fminf(mn[d], __shfl_xor_sync(0xffffffffu, mn[d], o));
      mx[d] = fmaxf(mx[d], __shfl_xor_sync(0xffffffffu, mx[d], o));
    }
  }
  if ((threadIdx.x & 31) == 0) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      atomicMin(&bounds[d], float_flip(mn[d]));
      atomicMax(&bounds[3 + d], float_flip(mx[d]));
    }
  }
}

__global__ void k_morton(const float* __restrict__ aabbs, uint32_t n, const uint32_t* __restrict__ bounds,
                         uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float* a = aabbs + 6 * (size_t)i;
  // One scale for all axes (the longest centroid extent): the Morton grid cells are cubes, so a
  // flat set (a height field, a floor) is split along its long axes first instead of spending a
  // third of the hierarchy on its thin one.
  float ext = 0.0f;
#pragma unroll
  for (int d = 0; d < 3; ++d) ext = fmaxf(ext, float_unflip(bounds[3 + d]) - float_unflip(bounds[d]));
  float u[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    float c = (a[d] + a[3 + d]) * 0.5f;
    u[d] = ext > 0.0f ? (c - float_unflip(bounds[d])) / ext : 0.5f;
  }
  keys[i] = morton30(u[0], u[1], u[2]);
  vals[i] = i;
}

// Longest common prefix of sorted keys i and j (index-augmented for duplicates), -1 out of range.
__device__ __forceinline__ int lcp(const uint32_t* __restrict__ keys, int n, int i, int j) {
  if (j < 0 || j >= n) return -1;
  uint32_t a = keys[i], b = keys[j];
  if (a != b) return __clz(a ^ b);
  return 32 + __clz((uint32_t)i ^ (uint32_t)j);
}

// Leaf data of sorted position i: the input index, or ids[input index] when the caller names its
// leaves (Bvh::insert with arbitrary leaf indices).
__device__ __forceinline__ uint32_t leaf_id(const uint32_t* __restrict__ sorted_vals, const uint32_t* __restrict__ ids, int i) {
  const uint32_t v = sorted_vals[i];
  return ids ? ids[v] : v;
}

__global__ void k_karras(const uint32_t* __restrict__ keys, const uint32_t* __restrict__ sorted_vals, int n,
                         WideNode* __restrict__ wide, uint32_t* __restrict__ leaf_parent, uint32_t* __restrict__ node_parent,
                         uint32_t* __restrict__ leaf_index, uint2* __restrict__ info, int leaf_data_is_position,
                         const uint32_t* __restrict__ ids) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) leaf_index[i] = leaf_id(sorted_vals, ids, i);
  if (i >= n - 1) return;
  int d = (lcp(keys, n, i, i + 1) - lcp(keys, n, i, i - 1)) >= 0 ? 1 : -1;
  int dmin = lcp(keys, n, i, i - d);
  int lmax = 2;
  while (lcp(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
  int l = 0;
  for (int t = lmax >> 1; t >= 1; t >>= 1)
    if (lcp(keys, n, i, i + (l + t) * d) > dmin) l += t;
  int j = i + l * d;
  int dnode = lcp(keys, n, i, j);
  int s = 0, step = l;
  do {
    step = (step + 1) >> 1;
    if (lcp(keys, n, i, i + (s + step) * d) > dnode) s += step;
  } while (step > 1);
  int gamma = i + s * d + (d < 0 ? -1 : 0);
  int first = i < j ? i : j, last = i < j ? j : i;
  info[i] = make_uint2((uint32_t)gamma, (uint32_t)last);
  uint32_t lchild, lcount, rchild, rcount;
  if (first == gamma) {
    lchild = leaf_data_is_position ? (uint32_t)gamma : leaf_id(sorted_vals, ids, gamma);
    lcount = 1;
    leaf_parent[gamma] = ((uint32_t)i << 1) | 0u;
  } else {
    lchild = (uint32_t)gamma;
    lcount = (uint32_t)(gamma - first + 1);
    node_parent[gamma] = ((uint32_t)i << 1) | 0u;
  }
  if (last == gamma + 1) {
    rchild = leaf_data_is_position ? (uint32_t)(gamma + 1) : leaf_id(sorted_vals, ids, gamma + 1);
    rcount = 1;
    leaf_parent[gamma + 1] = ((uint32_t)i << 1) | 1u;
  } else {
    rchild = (uint32_t)(gamma + 1);
    rcount = (uint32_t)(last - gamma);
    node_parent[gamma + 1] = ((uint32_t)i << 1) | 1u;
  }
  if (i == 0) node_parent[0] = 0xffffffffu;
  // Leaves carry the reference's pending-change flags (with_leaf_count_and_pending_change).
  wide[i].l.children = lchild;
  wide[i].l.data = lcount == 1 ? (1u | (3u << 30)) : lcount;
  wide[i].r.children = rchild;
  wide[i].r.data = rcount == 1 ? (1u | (3u << 30)) : rcount;
}

__device__ __forceinline__ void store_node_aabb(BvhNodeDev* nd, float3 mn, float3 mx) {
  float* f = reinterpret_cast<float*>(nd);
  __stcg(f + 0, mn.x); __stcg(f + 1, mn.y); __stcg(f + 2, mn.z);
  __stcg(f + 4, mx.x); __stcg(f + 5, mx.y); __stcg(f + 6, mx.z);
}

// rows (may be null): the AABB row of each sorted leaf when it is not the leaf data (a build over a
// compact list of named leaves).
__global__ void __launch_bounds__(FIT_THREADS) k_fit(const float* __restrict__ aabbs, uint32_t n, const uint32_t* __restrict__ leaf_index,
                                                     const uint32_t* __restrict__ leaf_parent, const uint32_t* __restrict__ node_parent,
                                                     WideNode* wide, uint32_t* flags, float* root_aabb, const uint32_t* __restrict__ rows) {
  uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const float* a = aabbs + 6 * (size_t)(rows ? rows[p] : leaf_index[p]);
  float3 mn = make_float3(a[0], a[1], a[2]);
  float3 mx = make_float3(a[3], a[4], a[5]);
  uint32_t lp = leaf_parent[p];
  uint32_t node = lp >> 1;
  store_node_aabb((lp & 1) ? &wide[node].r : &wide[node].l, mn, mx);
  __threadfence();
  // At most n - 1 internal nodes lie on the path to the root.
  for (uint32_t guard = 0; guard < n; ++guard) {
    uint32_t old = atomicAdd(&flags[node], 1u);
    if (old == 0) return;  // the sibling subtree is not finished; its last thread continues
    __threadfence();
    const float* w = reinterpret_cast<const float*>(&wide[node]);
    float3 lmn = make_float3(__ldcg(w + 0), __ldcg(w + 1), __ldcg(w + 2));
    float3 lmx = make_float3(__ldcg(w + 4), __ldcg(w + 5), __ldcg(w + 6));
    float3 rmn = make_float3(__ldcg(w + 8), __ldcg(w + 9), __ldcg(w + 10));
    float3 rmx = make_float3(__ldcg(w + 12), __ldcg(w + 13), __ldcg(w + 14));
    mn = make_float3(fminf(lmn.x, rmn.x), fminf(lmn.y, rmn.y), fminf(lmn.z, rmn.z));
    mx = make_float3(fmaxf(lmx.x, rmx.x), fmaxf(lmx.y, rmx.y), fmaxf(lmx.z, rmx.z));
    uint32_t np = node_parent[node];
    if (np == 0xffffffffu) {
      root_aabb[0] = mn.x; root_aabb[1] = mn.y; root_aabb[2] = mn.z;
      root_aabb[3] = mx.x; root_aabb[4] = mx.y; root_aabb[5] = mx.z;
      return;
    }
    node = np >> 1;
    store_node_aabb((np & 1) ? &wide[node].r : &wide[node].l, mn, mx);
    __threadfence();
  }
}

// Single-leaf tree: the reference's "partial root" (right child zeroed, bvh_tree.rs:1921-1929).
__global__ void k_single_leaf(const float* __restrict__ aabbs, WideNode* wide, uint32_t* leaf_index, uint32_t* leaf_parent,
                              float* root_aabb, int leaf_data_is_position, const uint32_t* __restrict__ ids) {
  if (threadIdx.x != 0) return;
  WideNode w;
  float* f = reinterpret_cast<float*>(&w);
  for (int k = 0; k < 16; ++k) f[k] = 0.0f;
  w.l.mins = make_float3(aabbs[0], aabbs[1], aabbs[2]);
  w.l.maxs = make_float3(aabbs[3], aabbs[4], aabbs[5]);
  const uint32_t id = (ids && !leaf_data_is_position) ? ids[0] : 0u;
  w.l.children = id;
  w.l.data = 1u | (3u << 30);
  w.r.children = 0;
  w.r.data = 0;
  wide[0] = w;
  leaf_index[0] = id;
  leaf_parent[0] = 0;
  for (int k = 0; k < 6; ++k) root_aabb[k] = aabbs[k];
  (void)leaf_data_is_position;
}

__global__ void k_single_leaf_refit(const float* __restrict__ aabbs, const uint32_t* __restrict__ leaf_index, int leaf_data_is_position,
                                    WideNode* wide, float* root_aabb) {
  if (threadIdx.x != 0) return;
  aabbs += leaf_data_is_position ? 0 : 6 * (size_t)leaf_index[0];
  wide[0].l.mins = make_float3(aabbs[0], aabbs[1], aabbs[2]);
  wide[0].l.maxs = make_float3(aabbs[3], aabbs[4], aabbs[5]);
  for (int k = 0; k < 6; ++k) root_aabb[k] = aabbs[k];
}

// ---------------- pair traversal ----------------

constexpr int PAIR_THREADS = 128;
constexpr int PAIR_STACK = 64;

__device__ __forceinline__ bool aabb_overlap(float3 amn, float3 amx, float3 bmn, float3 bmx) {
  return amn.x <= bmx.x && amn.y <= bmx.y && amn.z <= bmx.z && amx.x >= bmn.x && amx.y >= bmn.y && amx.z >= bmn.z;
}

__device__ __forceinline__ void emit_pair(uint32_t a, uint32_t b, uint32_t* pairs, unsigned long long cap,
                                          unsigned long long* count) {
  unsigned long long slot = atomicAdd(count, 1ull);
  if (slot < cap) { pairs[2 * slot] = a; pairs[2 * slot + 1] = b; }
}

// One thread per sorted leaf p: walks the tree with p's AABB and reports leaves q > p whose AABB
// intersects it. Subtrees whose sorted range lies entirely at or left of p are pruned (ranges
// from `info`), so every unordered pair is produced exactly once.
__global__ void __launch_bounds__(PAIR_THREADS) k_self_pairs(const WideNode* __restrict__ wide, const uint2* __restrict__ info,
                                                             const uint32_t* __restrict__ leaf_parent,
                                                             const uint32_t* __restrict__ leaf_index, uint32_t n,
                                                             uint32_t* __restrict__ pairs, unsigned long long cap,
                                                             unsigned long long* __restrict__ count, uint32_t* __restrict__ err) {
  uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  uint32_t lp = leaf_parent[p];
  const BvhNodeDev& me = (lp & 1) ? wide[lp >> 1].r : wide[lp >> 1].l;
  float3 qmn = me.mins, qmx = me.maxs;
  uint32_t myid = leaf_index[p];
  uint32_t stack[PAIR_STACK];
  int sp = 0;
  uint32_t cur = 0;
  for (;;) {
    uint2 inf = info[cur];
    uint32_t gamma = inf.x, last = inf.y;
    WideNode w;
    load_wide(wide, cur, &w);
    bool goL = false, goR = false;
    if (gamma > p && aabb_overlap(qmn, qmx, w.l.mins, w.l.maxs)) {
      if ((w.l.data & 0x3fffffffu) == 1u) {
        uint32_t o = leaf_index[gamma];
        emit_pair(min(myid, o), max(myid, o), pairs, cap, count);
      } else goL = true;
    }
    if (last > p && aabb_overlap(qmn, qmx, w.r.mins, w.r.maxs)) {
      if ((w.r.data & 0x3fffffffu) == 1u) {
        uint32_t o = leaf_index[gamma + 1];
        emit_pair(min(myid, o), max(myid, o), pairs, cap, count);
      } else goR = true;
    }
    if (goL && goR) {
      if (sp >= PAIR_STACK) { atomicOr(err, ERR_STACK_OVERFLOW); return; }
      stack[sp++] = w.r.children;
      cur = w.l.children;
    } else if (goL) {
      cur = w.l.children;
    } else if (goR) {
      cur = w.r.children;
    } else {
      if (sp == 0) return;
      cur = stack[--sp];
    }
  }
}

// One thread per sorted leaf of tree A: walks tree B. Leaves that are direct children of both
// roots are paired without an AABB check, as the reference iterator seeds them unchecked.
__global__ void __launch_bounds__(PAIR_THREADS) k_leaf_pairs(const WideNode* __restrict__ wa, const uint32_t* __restrict__ a_leaf_parent,
                                                             const uint32_t* __restrict__ a_leaf_index, uint32_t na,
                                                             const WideNode* __restrict__ wb, uint32_t nb,
                                                             uint32_t* __restrict__ pairs, unsigned long long cap,
                                                             unsigned long long* __restrict__ count, uint32_t* __restrict__ err) {
  uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= na) return;
  uint32_t lp = a_leaf_parent[p];
  const BvhNodeDev& me = (lp & 1) ? wa[lp >> 1].r : wa[lp >> 1].l;
  float3 qmn = me.mins, qmx = me.maxs;
  uint32_t myid = a_leaf_index[p];
  bool a_root_leaf = (lp >> 1) == 0;
  uint32_t stack[PAIR_STACK];
  int sp = 0;
  uint32_t cur = 0;
  for (;;) {
    WideNode w;
    load_wide(wb, cur, &w);
    bool goL = false, goR = false;
    bool at_root = cur == 0;
    const BvhNodeDev* ch[2] = {&w.l, &w.r};
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      uint32_t cnt = ch[s]->data & 0x3fffffffu;
      if (cnt == 0) continue;  // partial root
      bool leaf = cnt == 1u;
      bool unchecked = at_root && leaf && a_root_leaf;
      if (unchecked || aabb_overlap(qmn, qmx, ch[s]->mins, ch[s]->maxs)) {
        if (leaf) emit_pair(myid, ch[s]->children, pairs, cap, count);
        else if (s == 0) goL = true;
        else goR = true;
      }
    }
    if (goL && goR) {
      if (sp >= PAIR_STACK) { atomicOr(err, ERR_STACK_OVERFLOW); return; }
      stack[sp++] = w.r.children;
      cur = w.l.children;
    } else if (goL) {
      cur = w.l.children;
    } else if (goR) {
      cur = w.r.children;
    } else {
      if (sp == 0) return;
      cur = stack[--sp];
    }
  }
}

__global__ void k_split_pairs(const uint32_t* __restrict__ pairs, uint64_t n, uint32_t* __restrict__ first,
                              uint32_t* __restrict__ second) {
  uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint2 pr = reinterpret_cast<const uint2*>(pairs)[i];
  first[i] = pr.x;
  second[i] = pr.y;
}

__global__ void k_join_pairs(const uint32_t* __restrict__ first, const uint32_t* __restrict__ second, uint64_t n,
                             uint32_t* __restrict__ pairs) {
  uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  reinterpret_cast<uint2*>(pairs)[i] = make_uint2(first[i], second[i]);
}

int bits_for(uint32_t maxval) {
  int b = 1;
  while (b < 32 && (maxval >> b) != 0) ++b;
  return b;
}

// Sorts n (a, b) pairs in place lexicographically: stable sort by b, then stable sort by a.
parrygpu_status sort_pairs_inplace(parrygpu_ctx* ctx, uint32_t* d_pairs, uint64_t n, uint32_t max_a, uint32_t max_b) {
  if (n <= 1) return PARRYGPU_OK;
  if (n > 0xffffffffull) return set_error(ctx, PARRYGPU_INVALID_ARG, "too many pairs to sort");
  uint32_t nn = (uint32_t)n;
  parrygpu_status s = radix_sort_reserve(ctx, nn);
  if (s != PARRYGPU_OK) return s;
  // key = b, value = a
  k_split_pairs<<<div_up(n, 256), 256, 0, ctx->stream>>>(d_pairs, n, ctx->sort_v[0].as<uint32_t>(), ctx->sort_k[0].as<uint32_t>());
  PG_LAUNCHED(ctx);
  int rb;
  s = radix_sort_pairs(ctx, nn, bits_for(max_b), &rb);
  if (s != PARRYGPU_OK) return s;
  // Now key = a, value = b: swap roles by copying into buffer 0 in the swapped slots.
  if (rb != 0) {
    PG_CUDA(ctx, cudaMemcpyAsync(ctx->sort_k[0].ptr, ctx->sort_v[1].ptr, (size_t)n * 4, cudaMemcpyDeviceToDevice, ctx->stream));
    PG_CUDA(ctx, cudaMemcpyAsync(ctx->sort_v[0].ptr, ctx->sort_k[1].ptr, (size_t)n * 4, cudaMemcpyDeviceToDevice, ctx->stream));
  } else {
    std::swap(ctx->sort_k[0], ctx->sort_v[0]);
  }
  s = radix_sort_pairs(ctx, nn, bits_for(max_a), &rb);
  if (s != PARRYGPU_OK) return s;
  k_join_pairs<<<div_up(n, 256), 256, 0, ctx->stream>>>(ctx->sort_k[rb].as<uint32_t>(), ctx->sort_v[rb].as<uint32_t>(), n, d_pairs);
  PG_LAUNCHED(ctx);
  return PARRYGPU_OK;
}

}  // namespace

static parrygpu_status lbvh_fit(parrygpu_ctx* ctx, parrygpu_bvh* bvh, const float* d_aabbs, const uint32_t* rows);

parrygpu_status lbvh_build(parrygpu_ctx* ctx, parrygpu_bvh* bvh, const float* d_aabbs, uint32_t n, bool leaf_data_is_position,
                           const uint32_t* d_ids, uint32_t id_bound) {
  bvh->n_leaves = n;
  bvh->id_bound = d_ids ? id_bound : n;
  bvh->leaf_data_is_position = leaf_data_is_position;
  bvh->n_wide = n == 0 ? 0 : (n == 1 ? 1 : n - 1);
  if (n == 0) return PARRYGPU_OK;
  PG_CUDA(ctx, bvh->wide.reserve((size_t)bvh->n_wide * sizeof(WideNode)));
  PG_CUDA(ctx, bvh->leaf_parent.reserve((size_t)n * 4));
  PG_CUDA(ctx, bvh->leaf_index.reserve((size_t)n * 4));
  PG_CUDA(ctx, bvh->node_parent.reserve((size_t)bvh->n_wide * 4));
  PG_CUDA(ctx, bvh->flags.reserve((size_t)bvh->n_wide * 4));
  PG_CUDA(ctx, bvh->info.reserve((size_t)bvh->n_wide * 8));
  PG_CUDA(ctx, bvh->root_aabb.reserve(6 * 4));
  if (n == 1) {
    k_single_leaf<<<1, 32, 0, ctx->stream>>>(d_aabbs, bvh->wide.as<WideNode>(), bvh->leaf_index.as<uint32_t>(),
                                             bvh->leaf_parent.as<uint32_t>(), bvh->root_aabb.as<float>(), leaf_data_is_position, d_ids);
    PG_LAUNCHED(ctx);
    PG_CUDA(ctx, cudaMemsetAsync(bvh->info.ptr, 0, 8, ctx->stream));
    return PARRYGPU_OK;
  }
  parrygpu_status s = radix_sort_reserve(ctx, n);
  if (s != PARRYGPU_OK) return s;
  PG_CUDA(ctx, ctx->misc.reserve(64));
  uint32_t* bounds = ctx->misc.as<uint32_t>();
  PG_CUDA(ctx, cudaMemsetAsync(bounds, 0xff, 12, ctx->stream));
  PG_CUDA(ctx, cudaMemsetAsync(bounds + 3, 0x00, 12, ctx->stream));
  k_centroid_bounds<<<div_up(n, 256), 256, 0, ctx->stream>>>(d_aabbs, n, bounds);
  PG_LAUNCHED(ctx);
  k_morton<<<div_up(n, 256), 256, 0, ctx->stream>>>(d_aabbs, n, bounds, ctx->sort_k[0].as<uint32_t>(), ctx->sort_v[0].as<uint32_t>());
  PG_LAUNCHED(ctx);
  int rb;
  s = radix_sort_pairs(ctx, n, 30, &rb);
  if (s != PARRYGPU_OK) return s;
  k_karras<<<div_up(n, 256), 256, 0, ctx->stream>>>(ctx->sort_k[rb].as<uint32_t>(), ctx->sort_v[rb].as<uint32_t>(), (int)n,
                                                    bvh->wide.as<WideNode>(), bvh->leaf_parent.as<uint32_t>(),
                                                    bvh->node_parent.as<uint32_t>(), bvh->leaf_index.as<uint32_t>(),
                                                    bvh->info.as<uint2>(), leaf_data_is_position ? 1 : 0, d_ids);
  PG_LAUNCHED(ctx);
  return lbvh_fit(ctx, bvh, d_aabbs, d_ids ? ctx->sort_v[rb].as<uint32_t>() : nullptr);
}

parrygpu_status lbvh_refit(parrygpu_ctx* ctx, parrygpu_bvh* bvh, const float* d_aabbs) { return lbvh_fit(ctx, bvh, d_aabbs, nullptr); }

static parrygpu_status lbvh_fit(parrygpu_ctx* ctx, parrygpu_bvh* bvh, const float* d_aabbs, const uint32_t* rows) {
  uint32_t n = bvh->n_leaves;
  if (n == 0) return PARRYGPU_OK;
  if (n == 1) {
    k_single_leaf_refit<<<1, 32, 0, ctx->stream>>>(d_aabbs, bvh->leaf_index.as<uint32_t>(), bvh->leaf_data_is_position ? 1 : 0,
                                                   bvh->wide.as<WideNode>(), bvh->root_aabb.as<float>());
    PG_LAUNCHED(ctx);
    return PARRYGPU_OK;
  }
  PG_CUDA(ctx, cudaMemsetAsync(bvh->flags.ptr, 0, (size_t)bvh->n_wide * 4, ctx->stream));
  k_fit<<<div_up(n, FIT_THREADS), FIT_THREADS, 0, ctx->stream>>>(d_aabbs, n, bvh->leaf_index.as<uint32_t>(), bvh->leaf_parent.as<uint32_t>(),
                                                                 bvh->node_parent.as<uint32_t>(), bvh->wide.as<WideNode>(),
                                                                 bvh->flags.as<uint32_t>(), bvh->root_aabb.as<float>(), rows);
  PG_LAUNCHED(ctx);
  return PARRYGPU_OK;
}

// Runs a pair kernel into the caller's buffer (device or host), then optionally sorts.
template <class Launch>
static parrygpu_status run_pairs(parrygpu_ctx* ctx, uint32_t* pairs, uint64_t cap, uint64_t* n_out, int sorted, uint32_t max_a,
                                 uint32_t max_b, Launch launch) {
  if (!n_out) return set_error(ctx, PARRYGPU_INVALID_ARG, "n_out is null");
  if (cap > 0 && !pairs) return set_error(ctx, PARRYGPU_INVALID_ARG, "pairs is null");
  void* dpairs = nullptr;
  bool copy_back = false;
  parrygpu_status s = stage_output(ctx, ctx->stage_out[0], pairs, (size_t)cap * 8, &dpairs, &copy_back);
  if (s != PARRYGPU_OK) return s;
  PG_CUDA(ctx, ctx->counters.reserve(64));
  unsigned long long* d_count = ctx->counters.as<unsigned long long>();
  PG_CUDA(ctx, cudaMemsetAsync(d_count, 0, 8, ctx->stream));
  s = launch((uint32_t*)dpairs, (unsigned long long)cap, d_count);
  if (s != PARRYGPU_OK) return s;
  unsigned long long total = 0;
  PG_CUDA(ctx, cudaMemcpyAsync(&total, d_count, 8, cudaMemcpyDeviceToHost, ctx->stream));
  PG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  *n_out = total;
  uint64_t written = total < cap ? total : cap;
  if (sorted && total <= cap) {
    s = sort_pairs_inplace(ctx, (uint32_t*)dpairs, written, max_a, max_b);
    if (s != PARRYGPU_OK) return s;
  }
  if (copy_back && written) {
    PG_CUDA(ctx, cudaMemcpyAsync(pairs, dpairs, (size_t)written * 8, cudaMemcpyDeviceToHost, ctx->stream));
    PG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  }
  parrygpu_status es = parrygpu_sync(ctx);
  if (es != PARRYGPU_OK) return es;
  if (total > cap) return set_error(ctx, PARRYGPU_CAPACITY_EXCEEDED, "pair buffer holds %llu pairs, %llu found",
                                    (unsigned long long)cap, total);
  return PARRYGPU_OK;
}

parrygpu_status launch_self_pairs(parrygpu_ctx* ctx, const parrygpu_bvh* bvh, uint32_t* d_pairs, unsigned long long cap,
                                  unsigned long long* d_count) {
  uint32_t n = bvh->n_leaves;
  if (n < 2) return PARRYGPU_OK;
  k_self_pairs<<<div_up(n, PAIR_THREADS), PAIR_THREADS, 0, ctx->stream>>>(bvh->wide.as<WideNode>(), bvh->info.as<uint2>(),
                                                                          bvh->leaf_parent.as<uint32_t>(), bvh->leaf_index.as<uint32_t>(), n,
                                                                          d_pairs, cap, d_count, ctx->d_err);
  PG_LAUNCHED(ctx);
  return PARRYGPU_OK;
}

extern "C" {

parrygpu_status parrygpu_bvh_build(parrygpu_ctx* ctx, const float* aabbs, uint32_t n, parrygpu_bvh** out) {
  if (!ctx || !out) return PARRYGPU_INVALID_ARG;
  *out = nullptr;
  PG_CUDA(ctx, cudaSetDevice(ctx->device));
  const void* d_aabbs = nullptr;
  parrygpu_status s = stage_input(ctx, ctx->stage_in[0], aabbs, (size_t)n * 24, &d_aabbs);
  if (s != PARRYGPU_OK) return s;
  parrygpu_bvh* b = new parrygpu_bvh();
  s = lbvh_build(ctx, b, (const float*)d_aabbs, n, false);
  if (s != PARRYGPU_OK) { parrygpu_bvh_destroy(b); return s; }
  // The staged input may be reused by the next call: finish the build first when it was staged.
  if (d_aabbs != aabbs) PG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  *out = b;
  return PARRYGPU_OK;
}

parrygpu_status parrygpu_bvh_rebuild(parrygpu_ctx* ctx, parrygpu_bvh* bvh, const float* aabbs, uint32_t n) {
  if (!ctx || !bvh) return PARRYGPU_INVALID_ARG;
  PG_CUDA(ctx, cudaSetDevice(ctx->device));
  const void* d_aabbs = nullptr;
  parrygpu_status s = stage_input(ctx, ctx->stage_in[0], aabbs, (size_t)n * 24, &d_aabbs);
  if (s != PARRYGPU_OK) return s;
  if ((s = lbvh_build(ctx, bvh, (const float*)d_aabbs, n, false)) != PARRYGPU_OK) return s;
  if (d_aabbs != aabbs) PG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return PARRYGPU_OK;
}

void parrygpu_bvh_destroy(parrygpu_bvh* b) {
  if (!b) return;
  for (DevBuf* d : {&b->wide, &b->leaf_parent, &b->node_parent, &b->leaf_index, &b->flags, &b->root_aabb, &b->info}) d->release();
  delete b;
}

parrygpu_status parrygpu_bvh_refit(parrygpu_ctx* ctx, parrygpu_bvh* bvh, const float* aabbs) {
  if (!ctx || !bvh) return PARRYGPU_INVALID_ARG;
  PG_CUDA(ctx, cudaSetDevice(ctx->device));
  const void* d_aabbs = nullptr;
  parrygpu_status s = stage_input(ctx, ctx->stage_in[0], aabbs, (size_t)bvh->id_bound * 24, &d_aabbs);
  if (s != PARRYGPU_OK) return s;
  s = lbvh_refit(ctx, bvh, (const float*)d_aabbs);
  if (s != PARRYGPU_OK) return s;
  if (d_aabbs != aabbs) PG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return PARRYGPU_OK;
}

parrygpu_status parrygpu_bvh_self_pairs(parrygpu_ctx* ctx, const parrygpu_bvh* bvh, uint32_t* pairs, uint64_t cap,
                                        uint64_t* n_out, int sorted) {
  if (!ctx || !bvh) return PARRYGPU_INVALID_ARG;
  PG_CUDA(ctx, cudaSetDevice(ctx->device));
  if (bvh->n_leaves < 2) { if (n_out) *n_out = 0; return n_out ? PARRYGPU_OK : PARRYGPU_INVALID_ARG; }
  uint32_t n = bvh->n_leaves;
  return run_pairs(ctx, pairs, cap, n_out, sorted, bvh->id_bound - 1, bvh->id_bound - 1, [&](uint32_t* dp, unsigned long long c, unsigned long long* cnt) {
    k_self_pairs<<<div_up(n, PAIR_THREADS), PAIR_THREADS, 0, ctx->stream>>>(bvh->wide.as<WideNode>(), bvh->info.as<uint2>(),
                                                                            bvh->leaf_parent.as<uint32_t>(), bvh->leaf_index.as<uint32_t>(),
                                                                            n, dp, c, cnt, ctx->d_err);
    PG_LAUNCHED(ctx);
    return PARRYGPU_OK;
  });
}

parrygpu_status parrygpu_bvh_leaf_pairs(parrygpu_ctx* ctx, const parrygpu_bvh* a, const parrygpu_bvh* b, uint32_t* pairs,
                                        uint64_t cap, uint64_t* n_out, int sorted) {
  if (!ctx || !a || !b) return PARRYGPU_INVALID_ARG;
  PG_CUDA(ctx, cudaSetDevice(ctx->device));
  if (a->n_leaves == 0 || b->n_leaves == 0) { if (n_out) *n_out = 0; return n_out ? PARRYGPU_OK : PARRYGPU_INVALID_ARG; }
  uint32_t na = a->n_leaves, nb = b->n_leaves;
  return run_pairs(ctx, pairs, cap, n_out, sorted, a->id_bound - 1, b->id_bound - 1, [&](uint32_t* dp, unsigned long long c, unsigned long long* cnt) {
    k_leaf_pairs<<<div_up(na, PAIR_THREADS), PAIR_THREADS, 0, ctx->stream>>>(a->wide.as<WideNode>(), a->leaf_parent.as<uint32_t>(),
                                                                             a->leaf_index.as<uint32_t>(), na, b->wide.as<WideNode>(), nb,
                                                                             dp, c, cnt, ctx->d_err);
    PG_LAUNCHED(ctx);
    return PARRYGPU_OK;
  });
}

parrygpu_status parrygpu_bvh_info(const parrygpu_bvh* bvh, uint32_t* leaf_count, uint32_t* wide_node_count) {
  if (!bvh) return PARRYGPU_INVALID_ARG;
  if (leaf_count) *leaf_count = bvh->n_leaves;
  if (wide_node_count) *wide_node_count = bvh->n_wide;
  return PARRYGPU_OK;
}

parrygpu_status parrygpu_bvh_copy_nodes(parrygpu_ctx* ctx, const parrygpu_bvh* bvh, void* out) {
  if (!ctx || !bvh || (!out && bvh->n_wide)) return PARRYGPU_INVALID_ARG;
  if (bvh->n_wide == 0) return PARRYGPU_OK;
  PG_CUDA(ctx, cudaSetDevice(ctx->device));
  PG_CUDA(ctx, cudaMemcpyAsync(out, bvh->wide.ptr, (size_t)bvh->n_wide * sizeof(WideNode), cudaMemcpyDefault, ctx->stream));
  PG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return PARRYGPU_OK;
}

}  // extern "C"
