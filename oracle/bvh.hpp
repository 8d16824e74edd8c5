// Oracle (test infrastructure only): CPU restatement of parry3d's `partitioning::Bvh`.
// Used by tests/, the smoke check and the bench's CPU-baseline leg as the checker; the product
// path never calls it.
//
// Follows (paths relative to the parry repository):
//   src/partitioning/bvh/bvh_tree.rs      BvhNode / BvhNodeWide layout (:263-266, :456-467),
//                                         leaf (:520-527), merged (:610-618), intersects (:955-957),
//                                         BvhNode::cast_ray (:1177-1181), from_iter (:1891-1955)
//   src/partitioning/bvh/bvh_binned_build.rs  rebuild_range_binned (:39-176)
//   src/partitioning/bvh/bvh_traverse.rs  find_best (:335-417)
//   src/partitioning/bvh/bvh_traverse_bvtt.rs traverse_bvtt_single_tree (:19-204), leaf_pairs (:210-316)
//   src/partitioning/bvh/bvh_refit.rs     refit (bottom-up AABB recompute, :170-320)
//   src/bounding_volume/aabb.rs           center (:392), extents (:480), merge (:961), intersects (:951)
//   src/query/ray/ray_aabb.rs             Aabb::cast_local_ray (:11-49)
#pragma once
#include "math.hpp"
#include <vector>
#include <cstdint>
#include <cstring>

namespace oracle {

template <class R> struct Aabb {
  Vec3<R> mins, maxs;
  Aabb() {}
  Aabb(const Vec3<R>& a, const Vec3<R>& b) : mins(a), maxs(b) {}
  static Aabb invalid() {
    R m = std::numeric_limits<R>::max();
    return Aabb(Vec3<R>::repeat(m), Vec3<R>::repeat(-m));
  }
  // nalgebra::center(a, b) = (a + b) * 0.5
  Vec3<R> center() const { return (mins + maxs) * R(0.5); }
  Vec3<R> extents() const { return maxs - mins; }
  Vec3<R> half_extents() const { return (maxs - mins) * R(0.5); }
  R volume() const { Vec3<R> e = extents(); return e.x * e.y * e.z; }
  void merge(const Aabb& o) { mins = vinf(mins, o.mins); maxs = vsup(maxs, o.maxs); }
  Aabb merged(const Aabb& o) const { return Aabb(vinf(mins, o.mins), vsup(maxs, o.maxs)); }
  // na::partial_le(mins, o.maxs) && na::partial_ge(maxs, o.mins): inclusive on every axis.
  bool intersects(const Aabb& o) const {
    return mins.x <= o.maxs.x && mins.y <= o.maxs.y && mins.z <= o.maxs.z &&
           maxs.x >= o.mins.x && maxs.y >= o.mins.y && maxs.z >= o.mins.z;
  }
  Aabb loosened(R amount) const {
    return Aabb(mins + Vec3<R>::repeat(-amount), maxs + Vec3<R>::repeat(amount));
  }
};

template <class R> struct Ray {
  Vec3<R> origin, dir;
};

// ray_aabb.rs:12-49  Aabb::cast_local_ray. Returns false on a miss.
template <class R>
inline bool aabb_cast_local_ray(const Aabb<R>& b, const Ray<R>& ray, R max_toi, bool solid, R* out) {
  R tmin = R(0);
  R tmax = max_toi;
  for (int i = 0; i < 3; ++i) {
    if (ray.dir[i] == R(0)) {
      if (ray.origin[i] < b.mins[i] || ray.origin[i] > b.maxs[i]) return false;
    } else {
      R denom = R(1) / ray.dir[i];
      R n = (b.mins[i] - ray.origin[i]) * denom;
      R f = (b.maxs[i] - ray.origin[i]) * denom;
      if (n > f) std::swap(n, f);
      tmin = rmax(tmin, n);
      tmax = rmin(tmax, f);
      if (tmin > tmax) return false;
    }
  }
  *out = (tmin == R(0) && !solid) ? tmax : tmin;
  return true;
}

// bvh_tree.rs:456-467 — 32-byte node: mins, children, maxs, data (leaf count in the low 30 bits).
template <class R> struct BvhNode {
  Vec3<R> mins;
  uint32_t children = 0;
  Vec3<R> maxs;
  uint32_t data = 0;
  static BvhNode leaf(const Aabb<R>& a, uint32_t leaf_data) {
    BvhNode n;
    n.mins = a.mins; n.maxs = a.maxs; n.children = leaf_data;
    n.data = 1u | (3u << 30);  // with_leaf_count_and_pending_change(1)
    return n;
  }
  uint32_t leaf_count() const { return data & 0x3fffffffu; }
  bool is_leaf() const { return leaf_count() == 1; }
  Aabb<R> aabb() const { return Aabb<R>(mins, maxs); }
  Vec3<R> center() const { return (mins + maxs) * R(0.5); }
  BvhNode merged(const BvhNode& o, uint32_t children_id) const {
    BvhNode n;
    n.mins = vinf(mins, o.mins); n.maxs = vsup(maxs, o.maxs); n.children = children_id;
    uint32_t lc = leaf_count() + o.leaf_count();
    uint32_t ch = (data >> 30) | (o.data >> 30);
    n.data = lc | (ch << 30);
    return n;
  }
  bool intersects(const BvhNode& o) const { return aabb().intersects(o.aabb()); }
  // bvh_tree.rs:1177-1181: solid slab cast, Real::MAX on a miss.
  R cast_ray(const Ray<R>& ray, R max_toi) const {
    R t;
    if (aabb_cast_local_ray(aabb(), ray, max_toi, true, &t)) return t;
    return std::numeric_limits<R>::max();
  }
};

template <class R> struct BvhNodeWide {
  BvhNode<R> left, right;
};

// Per-query traversal counters (used for the algorithmic-bytes figure of the ray roofline).
struct VisitStats {
  uint64_t wide_visits = 0;  // BvhNodeWide records loaded
  uint64_t leaf_tests = 0;   // leaf-cost evaluations (triangle / part tests)
};

template <class R> struct Bvh {
  std::vector<BvhNodeWide<R>> nodes;

  uint32_t leaf_count() const {
    if (nodes.empty()) return 0;
    return nodes[0].left.leaf_count() + nodes[0].right.leaf_count();
  }

  // bvh_tree.rs:1891-1955 from_iter with BvhBuildStrategy::Binned.
  static Bvh from_leaves(const std::vector<Aabb<R>>& aabbs) {
    Bvh b;
    std::vector<BvhNode<R>> leaves;
    leaves.reserve(aabbs.size());
    for (size_t i = 0; i < aabbs.size(); ++i) leaves.push_back(BvhNode<R>::leaf(aabbs[i], (uint32_t)i));
    if (leaves.empty()) return b;
    if (leaves.size() == 1) { b.nodes.push_back({leaves[0], BvhNode<R>()}); return b; }
    if (leaves.size() == 2) { b.nodes.push_back({leaves[0], leaves[1]}); return b; }
    b.nodes.reserve(leaves.size());
    b.nodes.push_back(BvhNodeWide<R>());
    b.rebuild_range_binned(0, leaves.data(), leaves.size());
    return b;
  }

  // bvh_binned_build.rs:39-176
  void rebuild_range_binned(uint32_t target, BvhNode<R>* leaves, size_t len) {
    const int NUM_BINS = 8;
    const R BIN_EPSILON = R(1.0e-5);
    struct Bin { Aabb<R> aabb = Aabb<R>::invalid(); uint32_t leaf_count = 0; };
    Bin bins[NUM_BINS];
    // Aabb::from_points(centers)
    Vec3<R> c0 = leaves[0].center();
    Aabb<R> caabb(c0, c0);
    for (size_t i = 1; i < len; ++i) {
      Vec3<R> c = leaves[i].center();
      caabb.mins = vinf(caabb.mins, c);
      caabb.maxs = vsup(caabb.maxs, c);
    }
    int axis = imax(caabb.extents());
    R r0 = caabb.mins[axis], r1 = caabb.maxs[axis];
    R k1 = R(NUM_BINS) * (R(1) - BIN_EPSILON) / (r1 - r0);
    R k0 = r0;
    auto bin_of = [&](const BvhNode<R>& n) -> size_t {
      R v = k1 * (n.center()[axis] - k0);
      // Rust `as usize` saturates: NaN -> 0, negative -> 0.
      if (!(v > R(0))) return 0;
      return (size_t)v;
    };
    for (size_t i = 0; i < len; ++i) {
      size_t id = bin_of(leaves[i]);
      bins[id].aabb.merge(leaves[i].aabb());
      bins[id].leaf_count += 1;
    }
    Bin right_merges[NUM_BINS];
    for (int i = 0; i < NUM_BINS; ++i) right_merges[i] = bins[i];
    Bin right_acc = bins[NUM_BINS - 1];
    for (int i = 1; i < NUM_BINS - 1; ++i) {
      right_acc.aabb.merge(right_merges[NUM_BINS - 1 - i].aabb);
      right_acc.leaf_count += right_merges[NUM_BINS - 1 - i].leaf_count;
      right_merges[NUM_BINS - 1 - i] = right_acc;
    }
    R best_cost = std::numeric_limits<R>::max();
    size_t best_plane = 0;
    Bin left_merge = bins[0];
    uint32_t best_leaf_count = bins[0].leaf_count;
    for (int i = 0; i < NUM_BINS - 1; ++i) {
      const Bin& right = right_merges[i + 1];
      R cost = left_merge.aabb.volume() * R(left_merge.leaf_count) + right.aabb.volume() * R(right.leaf_count);
      if (cost < best_cost) { best_cost = cost; best_plane = i; best_leaf_count = left_merge.leaf_count; }
      left_merge.aabb.merge(bins[i + 1].aabb);
      left_merge.leaf_count += bins[i + 1].leaf_count;
    }
    size_t mid = best_leaf_count;
    if (mid == 0 || mid == len) {
      mid = len / 2;
    } else {
      size_t left_id = 0, right_id = mid;
      while (left_id != mid && right_id != len) {
        bool brk = false;
        while (bin_of(leaves[left_id]) <= best_plane) {
          left_id += 1;
          if (left_id == mid) { brk = true; break; }
        }
        if (brk) break;
        while (bin_of(leaves[right_id]) > best_plane) {
          right_id += 1;
          if (right_id == len) { brk = true; break; }
        }
        if (brk) break;
        std::swap(leaves[left_id], leaves[right_id]);
        left_id += 1; right_id += 1;
      }
    }
    BvhNode<R>* ll = leaves; size_t ln = mid;
    BvhNode<R>* rl = leaves + mid; size_t rn = len - mid;
    if (ln == 1) {
      nodes[target].left = ll[0];
    } else {
      uint32_t lid = (uint32_t)nodes.size();
      nodes.push_back(BvhNodeWide<R>());
      rebuild_range_binned(lid, ll, ln);
      nodes[target].left = nodes[lid].left.merged(nodes[lid].right, lid);
    }
    if (rn == 1) {
      nodes[target].right = rl[0];
    } else {
      uint32_t rid = (uint32_t)nodes.size();
      nodes.push_back(BvhNodeWide<R>());
      rebuild_range_binned(rid, rl, rn);
      nodes[target].right = nodes[rid].left.merged(nodes[rid].right, rid);
    }
  }

  // Refit: replace every leaf's AABB with `aabbs[leaf_data]` and recompute internal AABBs
  // bottom-up (bvh_refit.rs:259-320 recurse; the topology is unchanged).
  void refit(const std::vector<Aabb<R>>& aabbs) {
    if (nodes.empty()) return;
    if (nodes[0].right.leaf_count() == 0) {
      nodes[0].left.mins = aabbs[nodes[0].left.children].mins;
      nodes[0].left.maxs = aabbs[nodes[0].left.children].maxs;
      return;
    }
    refit_rec(0, aabbs);
  }
  void refit_rec(uint32_t id, const std::vector<Aabb<R>>& aabbs) {
    BvhNode<R>* sides[2] = {&nodes[id].left, &nodes[id].right};
    for (BvhNode<R>* n : sides) {
      if (n->is_leaf()) {
        n->mins = aabbs[n->children].mins; n->maxs = aabbs[n->children].maxs;
      } else {
        refit_rec(n->children, aabbs);
        const BvhNodeWide<R>& c = nodes[n->children];
        n->mins = vinf(c.left.mins, c.right.mins);
        n->maxs = vsup(c.left.maxs, c.right.maxs);
      }
    }
  }

  // bvh_traverse.rs:335-417 find_best, restated exactly (strict `<`; ties keep the first found).
  // `leaf_cost(leaf, best) -> bool` writes the leaf cost into *cost on success.
  template <class AabbCost, class LeafCost>
  bool find_best(R max_cost, AabbCost aabb_cost, LeafCost leaf_cost, uint32_t* out_id, VisitStats* st = nullptr) const {
    if (nodes.empty()) return false;
    if (nodes[0].right.leaf_count() == 0) {
      const BvhNode<R>& leaf = nodes[0].left;
      if (st) st->wide_visits++;
      if (aabb_cost(leaf, max_cost) < max_cost) {
        R c;
        if (st) st->leaf_tests++;
        if (!leaf_cost(leaf.children, max_cost, &c)) return false;
        if (c < max_cost) { *out_id = leaf.children; return true; }
      }
      return false;
    }
    std::vector<uint32_t> stack;
    stack.reserve(32);
    R best_cost = max_cost;
    uint32_t best_id = UINT32_MAX;
    bool have = false;
    uint32_t curr = 0;
    const R RMAX = std::numeric_limits<R>::max();
    for (;;) {
      if (st) st->wide_visits++;
      const BvhNode<R>* left = &nodes[curr].left;
      const BvhNode<R>* right = &nodes[curr].right;
      R ls = aabb_cost(*left, best_cost);
      R rs = aabb_cost(*right, best_cost);
      if (ls > rs) { std::swap(ls, rs); std::swap(left, right); }
      bool found_next = false;
      if (ls < best_cost && ls != RMAX) {
        if (left->is_leaf()) {
          R c;
          if (st) st->leaf_tests++;
          if (leaf_cost(left->children, best_cost, &c) && c < best_cost) {
            best_cost = c; best_id = left->children; have = true;
          }
        } else { curr = left->children; found_next = true; }
      }
      if (rs < best_cost && rs != RMAX) {
        if (right->is_leaf()) {
          R c;
          if (st) st->leaf_tests++;
          if (leaf_cost(right->children, best_cost, &c) && c < best_cost) {
            best_cost = c; best_id = right->children; have = true;
          }
        } else if (found_next) {
          stack.push_back(right->children);
        } else { curr = right->children; found_next = true; }
      }
      if (!found_next) {
        if (stack.empty()) { if (have) *out_id = best_id; return have; }
        curr = stack.back(); stack.pop_back();
      }
    }
  }

  // Same traversal with the lowest-leaf-index rule on exact cost ties: a node is visited when
  // its cost is <= the best cost (once a hit exists) and a leaf replaces the best on a smaller
  // cost, or an equal cost with a smaller leaf index. Before the first hit the strict `< max_cost`
  // bound of find_best is kept.
  template <class AabbCost, class LeafCost>
  bool find_best_lowest_index(R max_cost, AabbCost aabb_cost, LeafCost leaf_cost, uint32_t* out_id, VisitStats* st = nullptr) const {
    if (nodes.empty()) return false;
    if (nodes[0].right.leaf_count() == 0) return find_best(max_cost, aabb_cost, leaf_cost, out_id, st);
    std::vector<uint32_t> stack;
    stack.reserve(32);
    R best_cost = max_cost;
    uint32_t best_id = UINT32_MAX;
    bool have = false;
    uint32_t curr = 0;
    const R RMAX = std::numeric_limits<R>::max();
    auto visit_ok = [&](R s) { return s != RMAX && (s < best_cost || (have && s == best_cost)); };
    auto try_leaf = [&](uint32_t leaf) {
      R c;
      if (st) st->leaf_tests++;
      if (!leaf_cost(leaf, best_cost, &c)) return;
      if (c < best_cost || (have && c == best_cost && leaf < best_id)) { best_cost = c; best_id = leaf; have = true; }
    };
    for (;;) {
      if (st) st->wide_visits++;
      const BvhNode<R>* left = &nodes[curr].left;
      const BvhNode<R>* right = &nodes[curr].right;
      R ls = aabb_cost(*left, best_cost);
      R rs = aabb_cost(*right, best_cost);
      if (ls > rs) { std::swap(ls, rs); std::swap(left, right); }
      bool found_next = false;
      if (visit_ok(ls)) {
        if (left->is_leaf()) try_leaf(left->children);
        else { curr = left->children; found_next = true; }
      }
      if (visit_ok(rs)) {
        if (right->is_leaf()) try_leaf(right->children);
        else if (found_next) stack.push_back(right->children);
        else { curr = right->children; found_next = true; }
      }
      if (!found_next) {
        if (stack.empty()) { if (have) *out_id = best_id; return have; }
        curr = stack.back(); stack.pop_back();
      }
    }
  }

  // bvh_traverse_bvtt.rs:19-204 with CHANGE_DETECTION = false.
  template <class F> void traverse_bvtt_single_tree(F&& f) const {
    if (nodes.empty() || nodes[0].right.leaf_count() == 0) return;
    std::vector<uint32_t> stack;
    self_intersect_node(0, f, stack);
  }
  template <class F> void self_intersect_node(uint32_t id, F& f, std::vector<uint32_t>& stack) const {
    const BvhNodeWide<R>& node = nodes[id];
    bool lr = node.left.intersects(node.right);
    if (!node.left.is_leaf()) self_intersect_node(node.left.children, f, stack);
    if (!node.right.is_leaf()) self_intersect_node(node.right.children, f, stack);
    if (lr) {
      bool ll = node.left.is_leaf(), rl = node.right.is_leaf();
      if (ll && rl) f(node.left.children, node.right.children);
      else if (ll && !rl) traverse_single_subtree(node.left, node.right.children, f, stack);
      else if (!ll && rl) traverse_single_subtree(node.right, node.left.children, f, stack);
      else traverse_two_branches(node.left.children, node.right.children, f, stack);
    }
  }
  template <class F> void traverse_two_branches(uint32_t a, uint32_t b, F& f, std::vector<uint32_t>& stack) const {
    const BvhNodeWide<R>& n1 = nodes[a];
    const BvhNodeWide<R>& n2 = nodes[b];
    const BvhNode<R>* ca[4] = {&n1.left, &n1.left, &n1.right, &n1.right};
    const BvhNode<R>* cb[4] = {&n2.left, &n2.right, &n2.left, &n2.right};
    bool chk[4];
    for (int k = 0; k < 4; ++k) chk[k] = ca[k]->intersects(*cb[k]);
    for (int k = 0; k < 4; ++k) {
      if (!chk[k]) continue;
      bool la = ca[k]->is_leaf(), lb = cb[k]->is_leaf();
      if (la && lb) f(ca[k]->children, cb[k]->children);
      else if (la && !lb) traverse_single_subtree(*ca[k], cb[k]->children, f, stack);
      else if (!la && lb) traverse_single_subtree(*cb[k], ca[k]->children, f, stack);
      else traverse_two_branches(ca[k]->children, cb[k]->children, f, stack);
    }
  }
  template <class F> void traverse_single_subtree(const BvhNode<R>& node, uint32_t subtree, F& f, std::vector<uint32_t>& stack) const {
    uint32_t curr = subtree;
    for (;;) {
      const BvhNode<R>& left = nodes[curr].left;
      const BvhNode<R>& right = nodes[curr].right;
      bool lc = node.intersects(left), rc = node.intersects(right);
      bool found_next = false;
      if (lc) {
        if (left.is_leaf()) f(node.children, left.children);
        else { curr = left.children; found_next = true; }
      }
      if (rc) {
        if (right.is_leaf()) f(node.children, right.children);
        else if (!found_next) { curr = right.children; found_next = true; }
        else stack.push_back(right.children);
      }
      if (!found_next) {
        if (stack.empty()) return;
        curr = stack.back(); stack.pop_back();
      }
    }
  }

  // bvh_traverse_bvtt.rs:210-316 leaf_pairs with check = AABB intersection. The root-level pairs
  // are seeded without a check, exactly as the reference iterator does.
  template <class F> void leaf_pairs(const Bvh& other, F&& f) const {
    if (nodes.empty() || other.nodes.empty()) return;
    typedef std::pair<const BvhNode<R>*, const BvhNode<R>*> P;
    std::vector<P> stack;
    const BvhNodeWide<R>& r1 = nodes[0];
    const BvhNodeWide<R>& r2 = other.nodes[0];
    if (r1.left.leaf_count() > 0 && r2.right.leaf_count() > 0) stack.push_back(P(&r1.left, &r2.right));
    if (r1.right.leaf_count() > 0) {
      if (r2.right.leaf_count() > 0) stack.push_back(P(&r1.right, &r2.right));
      stack.push_back(P(&r1.right, &r2.left));
    }
    bool has_next = true;
    P next(&r1.left, &r2.left);
    for (;;) {
      if (!has_next) {
        if (stack.empty()) return;
        next = stack.back(); stack.pop_back(); has_next = true;
      }
      P cur = next; has_next = false;
      const BvhNode<R>* a = cur.first; const BvhNode<R>* b = cur.second;
      bool la = a->is_leaf(), lb = b->is_leaf();
      if (la && lb) { f(a->children, b->children); continue; }
      if (la && !lb) {
        const BvhNodeWide<R>& c2 = other.nodes[b->children];
        if (a->intersects(c2.left)) { next = P(a, &c2.left); has_next = true; }
        if (a->intersects(c2.right)) {
          if (!has_next) { next = P(a, &c2.right); has_next = true; } else stack.push_back(P(a, &c2.right));
        }
      } else if (!la && lb) {
        const BvhNodeWide<R>& c1 = nodes[a->children];
        if (c1.left.intersects(*b)) { next = P(&c1.left, b); has_next = true; }
        if (c1.right.intersects(*b)) {
          if (!has_next) { next = P(&c1.right, b); has_next = true; } else stack.push_back(P(&c1.right, b));
        }
      } else {
        const BvhNodeWide<R>& c1 = nodes[a->children];
        const BvhNodeWide<R>& c2 = other.nodes[b->children];
        if (c1.left.intersects(c2.left)) stack.push_back(P(&c1.left, &c2.left));
        if (c1.right.intersects(c2.left)) stack.push_back(P(&c1.right, &c2.left));
        if (c1.left.intersects(c2.right)) stack.push_back(P(&c1.left, &c2.right));
        if (c1.right.intersects(c2.right)) stack.push_back(P(&c1.right, &c2.right));
      }
    }
  }
};

}  // namespace oracle
