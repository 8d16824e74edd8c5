// The reference's serialised Bvh and its leaf edits on a parrygpu_bvh. Paths relative to the parry
// repository:
//   src/partitioning/bvh/bvh_tree.rs:1748-1761   Bvh { nodes, parents, leaf_node_indices } (serde / rkyv)
//   src/partitioning/bvh/bvh_tree.rs:1244-1290   BvhNodeIndex = (wide node << 1) | is_right
//   src/partitioning/bvh/bvh_insert.rs:126-370   Bvh::insert / insert_or_update_partially
//   src/partitioning/bvh/bvh_tree.rs:2360-2428   Bvh::remove
//
// Export hands the tree over in the reference's arrays; import takes any tree in that layout (one
// built and serialised by parry, say) and derives what the GPU traversals need: the parent links,
// the leaves in depth-first order (every subtree then covers a contiguous range of leaf positions,
// which the self-pair traversal prunes on) and each node's range. Insert and remove do not edit the
// tree node by node as the reference does: they rebuild the LBVH over the new leaf set, which costs
// about as much as one refit on the GPU. The tree layout therefore differs from the reference's after
// an edit (decision D-9); pairs, ray hits (lowest index on exact ties) and AABB queries do not depend
// on it.
#include "internal.hpp"
#include "common.cuh"
#include "lbvh_device.cuh"

using namespace pg;

namespace {

constexpr int IO_THREADS = 256;
constexpr uint32_t COUNT_MASK = 0x3fffffffu;
constexpr uint32_t NO_PARENT = 0xffffffffu;

__device__ __forceinline__ uint32_t count_of(const BvhNodeDev& n) { return n.data & COUNT_MASK; }
__device__ __forceinline__ const BvhNodeDev& side_of(const WideNode& w, uint32_t s) { return s ? w.r : w.l; }

// ---- export ----

__global__ void k_export_parents(uint32_t n_wide, const uint32_t* __restrict__ node_parent, unsigned long long* __restrict__ parents) {
  const uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= n_wide) return;
  const uint32_t p = node_parent[w];
  parents[w] = (w == 0 || p == NO_PARENT) ? 0ull : (unsigned long long)p;  // the root's entry is BvhNodeIndex::default()
}

__global__ void k_export_leaves(uint32_t n, const uint32_t* __restrict__ leaf_index, const uint32_t* __restrict__ leaf_parent,
                                unsigned long long* __restrict__ out, uint64_t cap, uint32_t* __restrict__ err) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const uint32_t id = leaf_index[p];
  if (id >= cap) { atomicOr(err, ERR_CAPACITY); return; }
  out[id] = leaf_parent[p];
}

// ---- import ----

// Parent links, leaf slots and the structural checks of every wide node.
__global__ void k_import_links(const WideNode* __restrict__ wide, uint32_t n_wide, uint32_t* __restrict__ parent_of,
                               uint32_t* __restrict__ pcount, uint32_t* __restrict__ leaf_slots, uint32_t* __restrict__ n_slots,
                               uint32_t* __restrict__ err) {
  const uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= n_wide) return;
  const WideNode node = wide[w];
#pragma unroll
  for (uint32_t s = 0; s < 2; ++s) {
    const BvhNodeDev& c = side_of(node, s);
    const uint32_t cnt = count_of(c);
    if (cnt == 0) {
      if (!(w == 0 && s == 1)) atomicOr(err, ERR_BAD_INDEX);  // only the partial root has an empty child
    } else if (cnt == 1) {
      const uint32_t k = atomicAdd(n_slots, 1u);
      leaf_slots[k] = (w << 1) | s;
    } else {
      const uint32_t ch = c.children;
      if (ch == 0 || ch >= n_wide) { atomicOr(err, ERR_BAD_INDEX); continue; }
      const WideNode& cw = wide[ch];
      if (count_of(cw.l) + count_of(cw.r) != cnt) atomicOr(err, ERR_BAD_INDEX);
      parent_of[ch] = (w << 1) | s;
      atomicAdd(&pcount[ch], 1u);
    }
  }
}

// Leaves before a node in depth-first order: the left subtrees passed on the way down from the root.
__device__ __forceinline__ bool dfs_start(const WideNode* __restrict__ wide, const uint32_t* __restrict__ parent_of, uint32_t n_wide,
                                          uint32_t w, uint32_t* start) {
  uint32_t pos = 0;
  for (uint32_t steps = 0; w != 0; ++steps) {
    if (steps >= n_wide) return false;
    const uint32_t p = parent_of[w];
    if (p == NO_PARENT) return false;
    if (p & 1u) pos += count_of(wide[p >> 1].l);
    w = p >> 1;
  }
  *start = pos;
  return true;
}

__global__ void k_import_nodes(const WideNode* __restrict__ wide, uint32_t n_wide, const uint32_t* __restrict__ parent_of,
                               const uint32_t* __restrict__ pcount, uint32_t* __restrict__ node_parent, uint2* __restrict__ info,
                               uint32_t* __restrict__ err) {
  const uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= n_wide) return;
  if (pcount[w] != (w == 0 ? 0u : 1u)) { atomicOr(err, ERR_BAD_INDEX); return; }
  uint32_t start = 0;
  if (!dfs_start(wide, parent_of, n_wide, w, &start)) { atomicOr(err, ERR_BAD_INDEX); return; }
  const uint32_t cl = count_of(wide[w].l), cr = count_of(wide[w].r);
  const uint32_t gamma = start + cl - 1u;
  info[w] = make_uint2(gamma, gamma + cr);
  node_parent[w] = w == 0 ? NO_PARENT : parent_of[w];
}

__global__ void k_import_leaves(const WideNode* __restrict__ wide, uint32_t n_wide, const uint32_t* __restrict__ parent_of,
                                const uint32_t* __restrict__ leaf_slots, uint32_t n, uint32_t* __restrict__ leaf_parent,
                                uint32_t* __restrict__ leaf_index, uint32_t* __restrict__ seen, uint32_t* __restrict__ max_id,
                                uint32_t* __restrict__ err) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const uint32_t slot = leaf_slots[k], w = slot >> 1, s = slot & 1u;
  uint32_t start = 0;
  if (!dfs_start(wide, parent_of, n_wide, w, &start)) { atomicOr(err, ERR_BAD_INDEX); return; }
  const uint32_t pos = start + (s ? count_of(wide[w].l) : 0u);
  if (pos >= n || atomicExch(&seen[pos], 1u) != 0u) { atomicOr(err, ERR_BAD_INDEX); return; }
  const uint32_t id = side_of(wide[w], s).children;
  if (id > PARRYGPU_MAX_LEAF_INDEX) { atomicOr(err, ERR_BAD_INDEX); return; }
  leaf_parent[pos] = slot;
  leaf_index[pos] = id;
  atomicMax(max_id, id);
}

__global__ void k_import_root(const WideNode* __restrict__ wide, float* __restrict__ root_aabb) {
  if (threadIdx.x != 0) return;
  const WideNode r = wide[0];
  float3 mn = r.l.mins, mx = r.l.maxs;
  if (count_of(r.r) != 0) {
    mn = make_float3(fminf(mn.x, r.r.mins.x), fminf(mn.y, r.r.mins.y), fminf(mn.z, r.r.mins.z));
    mx = make_float3(fmaxf(mx.x, r.r.maxs.x), fmaxf(mx.y, r.r.maxs.y), fmaxf(mx.z, r.r.maxs.z));
  }
  root_aabb[0] = mn.x; root_aabb[1] = mn.y; root_aabb[2] = mn.z;
  root_aabb[3] = mx.x; root_aabb[4] = mx.y; root_aabb[5] = mx.z;
}

// ---- edits ----

// The current leaves as (id, AABB) rows, in leaf-position order.
__global__ void k_gather_leaves(uint32_t n, const uint32_t* __restrict__ leaf_index, const uint32_t* __restrict__ leaf_parent,
                                const WideNode* __restrict__ wide, uint32_t* __restrict__ ids, float* __restrict__ aabbs) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const uint32_t lp = leaf_parent[p];
  const BvhNodeDev& c = side_of(wide[lp >> 1], lp & 1u);
  ids[p] = leaf_index[p];
  float* a = aabbs + 6 * (size_t)p;
  a[0] = c.mins.x; a[1] = c.mins.y; a[2] = c.mins.z;
  a[3] = c.maxs.x; a[4] = c.maxs.y; a[5] = c.maxs.z;
}

__global__ void k_iota_keys(uint32_t n, const uint32_t* __restrict__ src, uint32_t* __restrict__ keys, uint32_t* __restrict__ vals,
                            uint32_t* __restrict__ max_id) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  keys[i] = src[i];
  vals[i] = i;
  atomicMax(max_id, src[i]);
}

// Insert / update: in id order, the last row of each id wins (a new row comes after the current one).
__global__ void k_keep_last(uint32_t n, const uint32_t* __restrict__ keys, uint32_t* __restrict__ keep) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  keep[i] = (i + 1 == n || keys[i + 1] != keys[i]) ? 1u : 0u;
}

// Remove: a current leaf stays unless its id is in the sorted removal list.
__global__ void k_keep_unremoved(uint32_t n, const uint32_t* __restrict__ ids, const uint32_t* __restrict__ removed, uint32_t k,
                                 uint32_t* __restrict__ keep) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const uint32_t id = ids[p];
  uint32_t lo = 0, hi = k;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (removed[mid] < id) lo = mid + 1; else hi = mid;
  }
  keep[p] = (lo < k && removed[lo] == id) ? 0u : 1u;
}

// Rows i (through `order`, identity when null) with keep[i] set, packed by the exclusive scan.
__global__ void k_compact(uint32_t n, const uint32_t* __restrict__ order, const uint32_t* __restrict__ keep,
                          const uint32_t* __restrict__ scan, const uint32_t* __restrict__ ids, const float* __restrict__ aabbs,
                          uint32_t* __restrict__ ids_out, float* __restrict__ aabbs_out, uint32_t* __restrict__ max_id) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || !keep[i]) return;
  const uint32_t src = order ? order[i] : i, dst = scan[i];
  ids_out[dst] = ids[src];
  for (int k = 0; k < 6; ++k) aabbs_out[6 * (size_t)dst + k] = aabbs[6 * (size_t)src + k];
  atomicMax(max_id, ids[src]);
}

int bits_for(uint32_t v) {
  int b = 0;
  while (b < 32 && (v >> b) != 0u) ++b;
  return b < 8 ? 8 : b;
}

// Scratch of one edit, released on every exit path.
struct EditScratch {
  DevBuf ids, aabbs, keys[2], vals[2], hist, keep, scan, ids_out, aabbs_out, misc;
  void release() {
    for (DevBuf* d : {&ids, &aabbs, &keys[0], &keys[1], &vals[0], &vals[1], &hist, &keep, &scan, &ids_out, &aabbs_out, &misc}) d->release();
  }
  ~EditScratch() { release(); }
};

// Import state: the tree under construction and its scratch, both released unless the import
// succeeds (then `tree` is handed over).
struct ImportScratch {
  parrygpu_bvh* tree = nullptr;
  DevBuf parent_of, pcount, slots, seen, misc;
  ~ImportScratch() {
    for (DevBuf* d : {&parent_of, &pcount, &slots, &seen, &misc}) d->release();
    if (tree) parrygpu_bvh_destroy(tree);
  }
};

// Packs the kept rows (keep / scan over n rows, read through `order`) and rebuilds the tree over them.
parrygpu_status compact_and_rebuild(parrygpu_ctx* ctx, parrygpu_bvh* bvh, EditScratch& sc, uint32_t n, const uint32_t* order) {
  uint32_t* keep = sc.keep.as<uint32_t>();
  uint32_t* scan = sc.scan.as<uint32_t>();
  uint32_t* max_id = sc.misc.as<uint32_t>();
  PG_CUDA(ctx, cudaMemsetAsync(scan, 0, ((size_t)n + 4) * 4, ctx->stream));
  PG_CUDA(ctx, cudaMemcpyAsync(scan, keep, (size_t)n * 4, cudaMemcpyDeviceToDevice, ctx->stream));
  parrygpu_status s = exclusive_scan_u32(ctx, scan, n);
  if (s != PARRYGPU_OK) return s;
  PG_CUDA(ctx, cudaMemsetAsync(max_id, 0, 4, ctx->stream));
  k_compact<<<div_up(n, IO_THREADS), IO_THREADS, 0, ctx->stream>>>(n, order, keep, scan, sc.ids.as<uint32_t>(), sc.aabbs.as<float>(),
                                                                   sc.ids_out.as<uint32_t>(), sc.aabbs_out.as<float>(), max_id);
  PG_LAUNCHED(ctx);
  uint32_t h[3] = {0, 0, 0};
  PG_CUDA(ctx, cudaMemcpyAsync(&h[0], scan + (n - 1), 4, cudaMemcpyDeviceToHost, ctx->stream));
  PG_CUDA(ctx, cudaMemcpyAsync(&h[1], keep + (n - 1), 4, cudaMemcpyDeviceToHost, ctx->stream));
  PG_CUDA(ctx, cudaMemcpyAsync(&h[2], max_id, 4, cudaMemcpyDeviceToHost, ctx->stream));
  PG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  const uint32_t count = h[0] + h[1];
  const uint64_t id_bound = count ? (uint64_t)h[2] + 1u : 0u;
  if (id_bound > (uint64_t)PARRYGPU_MAX_LEAF_INDEX + 1u)
    return set_error(ctx, PARRYGPU_INVALID_ARG, "leaf index %u above PARRYGPU_MAX_LEAF_INDEX", h[2]);
  s = lbvh_build(ctx, bvh, sc.aabbs_out.as<float>(), count, false, sc.ids_out.as<uint32_t>(), (uint32_t)id_bound);
  if (s != PARRYGPU_OK) return s;
  PG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return parrygpu_sync(ctx);
}

}  // namespace

extern "C" {

parrygpu_status parrygpu_bvh_export(parrygpu_ctx* ctx, const parrygpu_bvh* bvh, void* nodes, uint64_t* parents, uint64_t* leaf_nodes,
                                    uint64_t leaf_capacity) {
  if (!ctx || !bvh) return PARRYGPU_INVALID_ARG;
  if (bvh->leaf_data_is_position) return set_error(ctx, PARRYGPU_INVALID_ARG, "a TriMesh tree keeps sorted positions as leaf data");
  PG_CUDA(ctx, cudaSetDevice(ctx->device));
  const uint32_t nw = bvh->n_wide, n = bvh->n_leaves;
  if (nodes && nw) PG_CUDA(ctx, cudaMemcpyAsync(nodes, bvh->wide.ptr, (size_t)nw * sizeof(WideNode), cudaMemcpyDefault, ctx->stream));
  if (parents && nw) {
    void* dp = nullptr;
    bool copy = false;
    parrygpu_status s = stage_output(ctx, ctx->stage_out[0], parents, (size_t)nw * 8, &dp, &copy);
    if (s != PARRYGPU_OK) return s;
    k_export_parents<<<div_up(nw, IO_THREADS), IO_THREADS, 0, ctx->stream>>>(nw, bvh->node_parent.as<uint32_t>(),
                                                                             (unsigned long long*)dp);
    PG_LAUNCHED(ctx);
    if (copy) PG_CUDA(ctx, cudaMemcpyAsync(parents, dp, (size_t)nw * 8, cudaMemcpyDeviceToHost, ctx->stream));
  }
  if (leaf_nodes && leaf_capacity) {
    void* dl = nullptr;
    bool copy = false;
    parrygpu_status s = stage_output(ctx, ctx->stage_out[1], leaf_nodes, (size_t)leaf_capacity * 8, &dl, &copy);
    if (s != PARRYGPU_OK) return s;
    PG_CUDA(ctx, cudaMemsetAsync(dl, 0xff, (size_t)leaf_capacity * 8, ctx->stream));  // holes of the VecMap
    if (n) {
      k_export_leaves<<<div_up(n, IO_THREADS), IO_THREADS, 0, ctx->stream>>>(n, bvh->leaf_index.as<uint32_t>(), bvh->leaf_parent.as<uint32_t>(),
                                                                             (unsigned long long*)dl, leaf_capacity, ctx->d_err);
      PG_LAUNCHED(ctx);
    }
    if (copy) PG_CUDA(ctx, cudaMemcpyAsync(leaf_nodes, dl, (size_t)leaf_capacity * 8, cudaMemcpyDeviceToHost, ctx->stream));
  }
  PG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return parrygpu_sync(ctx);
}

parrygpu_status parrygpu_bvh_import(parrygpu_ctx* ctx, const void* nodes, uint32_t n_wide, parrygpu_bvh** out) {
  if (!ctx || !out || (n_wide && !nodes)) return PARRYGPU_INVALID_ARG;
  *out = nullptr;
  PG_CUDA(ctx, cudaSetDevice(ctx->device));
  ImportScratch sc;
  sc.tree = new parrygpu_bvh();
  parrygpu_bvh* b = sc.tree;
  if (n_wide == 0) {
    *out = b;
    sc.tree = nullptr;
    return PARRYGPU_OK;
  }
  const size_t nw = n_wide;
  PG_CUDA(ctx, b->wide.reserve(nw * sizeof(WideNode)));
  PG_CUDA(ctx, b->node_parent.reserve(nw * 4));
  PG_CUDA(ctx, b->info.reserve(nw * 8));
  PG_CUDA(ctx, b->flags.reserve(nw * 4));
  PG_CUDA(ctx, b->root_aabb.reserve(24));
  PG_CUDA(ctx, sc.parent_of.reserve(nw * 4));
  PG_CUDA(ctx, sc.pcount.reserve(nw * 4));
  PG_CUDA(ctx, sc.slots.reserve(2 * nw * 4));
  PG_CUDA(ctx, sc.misc.reserve(16));
  PG_CUDA(ctx, cudaMemcpyAsync(b->wide.ptr, nodes, nw * sizeof(WideNode), cudaMemcpyDefault, ctx->stream));
  PG_CUDA(ctx, cudaMemsetAsync(sc.parent_of.ptr, 0xff, nw * 4, ctx->stream));
  PG_CUDA(ctx, cudaMemsetAsync(sc.pcount.ptr, 0, nw * 4, ctx->stream));
  PG_CUDA(ctx, cudaMemsetAsync(sc.misc.ptr, 0, 16, ctx->stream));
  uint32_t* d_n = sc.misc.as<uint32_t>();  // [0] leaf slots, [1] largest leaf index
  k_import_links<<<div_up(n_wide, IO_THREADS), IO_THREADS, 0, ctx->stream>>>(b->wide.as<WideNode>(), n_wide, sc.parent_of.as<uint32_t>(),
                                                                             sc.pcount.as<uint32_t>(), sc.slots.as<uint32_t>(), d_n, ctx->d_err);
  PG_LAUNCHED(ctx);
  uint32_t h[2] = {0, 0};
  WideNode root;
  PG_CUDA(ctx, cudaMemcpyAsync(&h[0], d_n, 4, cudaMemcpyDeviceToHost, ctx->stream));
  PG_CUDA(ctx, cudaMemcpyAsync(&root, b->wide.ptr, sizeof(WideNode), cudaMemcpyDeviceToHost, ctx->stream));
  PG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (parrygpu_sync(ctx) != PARRYGPU_OK)
    return set_error(ctx, PARRYGPU_INVALID_ARG, "not a BvhNodeWide tree (child index or leaf count)");
  const uint32_t n = h[0];
  if (n == 0 || (root.l.data & COUNT_MASK) + (root.r.data & COUNT_MASK) != n)
    return set_error(ctx, PARRYGPU_INVALID_ARG, "the root's leaf counts do not match the %u leaves of the tree", n);
  PG_CUDA(ctx, b->leaf_parent.reserve((size_t)n * 4));
  PG_CUDA(ctx, b->leaf_index.reserve((size_t)n * 4));
  PG_CUDA(ctx, sc.seen.reserve((size_t)n * 4));
  PG_CUDA(ctx, cudaMemsetAsync(sc.seen.ptr, 0, (size_t)n * 4, ctx->stream));
  k_import_nodes<<<div_up(n_wide, IO_THREADS), IO_THREADS, 0, ctx->stream>>>(b->wide.as<WideNode>(), n_wide, sc.parent_of.as<uint32_t>(),
                                                                             sc.pcount.as<uint32_t>(), b->node_parent.as<uint32_t>(),
                                                                             b->info.as<uint2>(), ctx->d_err);
  PG_LAUNCHED(ctx);
  k_import_leaves<<<div_up(n, IO_THREADS), IO_THREADS, 0, ctx->stream>>>(b->wide.as<WideNode>(), n_wide, sc.parent_of.as<uint32_t>(),
                                                                         sc.slots.as<uint32_t>(), n, b->leaf_parent.as<uint32_t>(),
                                                                         b->leaf_index.as<uint32_t>(), sc.seen.as<uint32_t>(), d_n + 1,
                                                                         ctx->d_err);
  PG_LAUNCHED(ctx);
  k_import_root<<<1, 32, 0, ctx->stream>>>(b->wide.as<WideNode>(), b->root_aabb.as<float>());
  PG_LAUNCHED(ctx);
  PG_CUDA(ctx, cudaMemcpyAsync(&h[1], d_n + 1, 4, cudaMemcpyDeviceToHost, ctx->stream));
  PG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (parrygpu_sync(ctx) != PARRYGPU_OK)
    return set_error(ctx, PARRYGPU_INVALID_ARG, "not a BvhNodeWide tree (parent links or leaf counts)");
  b->n_wide = n_wide;
  b->n_leaves = n;
  if (h[1] > PARRYGPU_MAX_LEAF_INDEX)  // unreachable after the kernel's check; kept for the row count below
    return set_error(ctx, PARRYGPU_INVALID_ARG, "leaf index %u above PARRYGPU_MAX_LEAF_INDEX", h[1]);
  b->id_bound = h[1] + 1u;
  b->leaf_data_is_position = false;
  *out = b;
  sc.tree = nullptr;
  return PARRYGPU_OK;
}

parrygpu_status parrygpu_bvh_insert(parrygpu_ctx* ctx, parrygpu_bvh* bvh, const float* aabbs, const uint32_t* leaf_ids, uint32_t k) {
  if (!ctx || !bvh || (k && (!aabbs || !leaf_ids))) return PARRYGPU_INVALID_ARG;
  if (bvh->leaf_data_is_position) return set_error(ctx, PARRYGPU_INVALID_ARG, "a TriMesh tree cannot take new leaves");
  if (k == 0) return PARRYGPU_OK;
  PG_CUDA(ctx, cudaSetDevice(ctx->device));
  const uint32_t n = bvh->n_leaves;
  const uint64_t m64 = (uint64_t)n + k;
  if (m64 >= 0x7fffffffull) return set_error(ctx, PARRYGPU_INVALID_ARG, "too many leaves");
  const uint32_t m = (uint32_t)m64;
  EditScratch sc;
  PG_CUDA(ctx, sc.ids.reserve((size_t)m * 4));
  PG_CUDA(ctx, sc.aabbs.reserve((size_t)m * 24));
  for (int i = 0; i < 2; ++i) {
    PG_CUDA(ctx, sc.keys[i].reserve((size_t)m * 4));
    PG_CUDA(ctx, sc.vals[i].reserve((size_t)m * 4));
  }
  PG_CUDA(ctx, sc.hist.reserve((size_t)radix_sort_hist_entries(m) * 4));
  PG_CUDA(ctx, sc.keep.reserve((size_t)m * 4));
  PG_CUDA(ctx, sc.scan.reserve(((size_t)m + 4) * 4));
  PG_CUDA(ctx, sc.ids_out.reserve((size_t)m * 4));
  PG_CUDA(ctx, sc.aabbs_out.reserve((size_t)m * 24));
  PG_CUDA(ctx, sc.misc.reserve(16));
  if (n) {
    k_gather_leaves<<<div_up(n, IO_THREADS), IO_THREADS, 0, ctx->stream>>>(n, bvh->leaf_index.as<uint32_t>(), bvh->leaf_parent.as<uint32_t>(),
                                                                           bvh->wide.as<WideNode>(), sc.ids.as<uint32_t>(), sc.aabbs.as<float>());
    PG_LAUNCHED(ctx);
  }
  // the new rows after the current ones: in id order they come last and win
  PG_CUDA(ctx, cudaMemcpyAsync(sc.ids.as<uint32_t>() + n, leaf_ids, (size_t)k * 4, cudaMemcpyDefault, ctx->stream));
  PG_CUDA(ctx, cudaMemcpyAsync(sc.aabbs.as<float>() + 6 * (size_t)n, aabbs, (size_t)k * 24, cudaMemcpyDefault, ctx->stream));
  PG_CUDA(ctx, cudaMemsetAsync(sc.misc.ptr, 0, 16, ctx->stream));
  uint32_t* max_id = sc.misc.as<uint32_t>();
  k_iota_keys<<<div_up(m, IO_THREADS), IO_THREADS, 0, ctx->stream>>>(m, sc.ids.as<uint32_t>(), sc.keys[0].as<uint32_t>(),
                                                                     sc.vals[0].as<uint32_t>(), max_id);
  PG_LAUNCHED(ctx);
  uint32_t hmax = 0;
  PG_CUDA(ctx, cudaMemcpyAsync(&hmax, max_id, 4, cudaMemcpyDeviceToHost, ctx->stream));
  PG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (hmax > PARRYGPU_MAX_LEAF_INDEX)  // nothing was changed yet: the tree stays as it was
    return set_error(ctx, PARRYGPU_INVALID_ARG, "leaf index %u above PARRYGPU_MAX_LEAF_INDEX", hmax);
  int rb = 0;
  parrygpu_status s = radix_sort_pairs_in(ctx, m, bits_for(hmax), sc.keys[0].as<uint32_t>(), sc.vals[0].as<uint32_t>(),
                                          sc.keys[1].as<uint32_t>(), sc.vals[1].as<uint32_t>(), sc.hist.as<uint32_t>(), &rb);
  if (s != PARRYGPU_OK) return s;
  k_keep_last<<<div_up(m, IO_THREADS), IO_THREADS, 0, ctx->stream>>>(m, sc.keys[rb].as<uint32_t>(), sc.keep.as<uint32_t>());
  PG_LAUNCHED(ctx);
  return compact_and_rebuild(ctx, bvh, sc, m, sc.vals[rb].as<uint32_t>());
}

parrygpu_status parrygpu_bvh_remove(parrygpu_ctx* ctx, parrygpu_bvh* bvh, const uint32_t* leaf_ids, uint32_t k) {
  if (!ctx || !bvh || (k && !leaf_ids)) return PARRYGPU_INVALID_ARG;
  if (bvh->leaf_data_is_position) return set_error(ctx, PARRYGPU_INVALID_ARG, "a TriMesh tree cannot drop leaves");
  const uint32_t n = bvh->n_leaves;
  if (k == 0 || n == 0) return PARRYGPU_OK;
  PG_CUDA(ctx, cudaSetDevice(ctx->device));
  EditScratch sc;
  PG_CUDA(ctx, sc.ids.reserve((size_t)n * 4));
  PG_CUDA(ctx, sc.aabbs.reserve((size_t)n * 24));
  for (int i = 0; i < 2; ++i) {
    PG_CUDA(ctx, sc.keys[i].reserve((size_t)k * 4));
    PG_CUDA(ctx, sc.vals[i].reserve((size_t)k * 4));
  }
  PG_CUDA(ctx, sc.hist.reserve((size_t)radix_sort_hist_entries(k) * 4));
  PG_CUDA(ctx, sc.keep.reserve((size_t)n * 4));
  PG_CUDA(ctx, sc.scan.reserve(((size_t)n + 4) * 4));
  PG_CUDA(ctx, sc.ids_out.reserve((size_t)n * 4));
  PG_CUDA(ctx, sc.aabbs_out.reserve((size_t)n * 24));
  PG_CUDA(ctx, sc.misc.reserve(16));
  // the removal list, sorted (ids that name no leaf are ignored, as Bvh::remove does)
  PG_CUDA(ctx, cudaMemcpyAsync(sc.keys[0].ptr, leaf_ids, (size_t)k * 4, cudaMemcpyDefault, ctx->stream));
  PG_CUDA(ctx, cudaMemsetAsync(sc.vals[0].ptr, 0, (size_t)k * 4, ctx->stream));
  k_gather_leaves<<<div_up(n, IO_THREADS), IO_THREADS, 0, ctx->stream>>>(n, bvh->leaf_index.as<uint32_t>(), bvh->leaf_parent.as<uint32_t>(),
                                                                         bvh->wide.as<WideNode>(), sc.ids.as<uint32_t>(), sc.aabbs.as<float>());
  PG_LAUNCHED(ctx);
  int rb = 0;
  parrygpu_status s = radix_sort_pairs_in(ctx, k, 32, sc.keys[0].as<uint32_t>(), sc.vals[0].as<uint32_t>(), sc.keys[1].as<uint32_t>(),
                                          sc.vals[1].as<uint32_t>(), sc.hist.as<uint32_t>(), &rb);
  if (s != PARRYGPU_OK) return s;
  k_keep_unremoved<<<div_up(n, IO_THREADS), IO_THREADS, 0, ctx->stream>>>(n, sc.ids.as<uint32_t>(), sc.keys[rb].as<uint32_t>(), k,
                                                                          sc.keep.as<uint32_t>());
  PG_LAUNCHED(ctx);
  return compact_and_rebuild(ctx, bvh, sc, n, nullptr);
}

}  // extern "C"
