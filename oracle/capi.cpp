// Oracle (test infrastructure only): flat C entry points over the C++ restatement of parry3d,
// loaded with ctypes by tests/, the smoke check and the bench's CPU-baseline leg. Never linked
// into the product library.
//
// Each function comes in an f32 flavour (parry3d) and an f64 flavour (parry3d-f64); f64 inputs
// are the f32 inputs widened, so the f64 result measures the f32 path's rounding error.
#include "ray.hpp"
#include "query.hpp"
#include <thread>
#include <vector>
#include <algorithm>
#include <cstring>

using namespace oracle;

namespace {

template <class F> void parallel_for(uint64_t n, int threads, F&& f) {
  if (threads <= 1 || n < 2048) { for (uint64_t i = 0; i < n; ++i) f(i); return; }
  std::vector<std::thread> ts;
  uint64_t chunk = 1024;
  std::atomic<uint64_t> next{0};
  for (int t = 0; t < threads; ++t) {
    ts.emplace_back([&]() {
      for (;;) {
        uint64_t s = next.fetch_add(chunk);
        if (s >= n) break;
        uint64_t e = std::min(n, s + chunk);
        for (uint64_t i = s; i < e; ++i) f(i);
      }
    });
  }
  for (auto& t : ts) t.join();
}

template <class R> TriMesh<R>* make_mesh(const float* v, uint32_t nv, const uint32_t* idx, uint32_t nt) {
  TriMesh<R>* m = new TriMesh<R>();
  m->vertices.resize(nv);
  for (uint32_t i = 0; i < nv; ++i) m->vertices[i] = Vec3<R>(R(v[3 * i]), R(v[3 * i + 1]), R(v[3 * i + 2]));
  m->indices.assign(idx, idx + 3 * (size_t)nt);
  m->build();
  return m;
}

template <class R, class O>
void cast_rays(const TriMesh<R>* m, const float* pose7, const float* rays, uint64_t n, float max_toi, int lowest_index,
               int threads, uint32_t* feat, O* toi, O* normal, uint64_t* stats) {
  Iso<R> iso = pose7 ? Iso<R>::from_pose7(pose7) : Iso<R>::identity();
  std::vector<VisitStats> per(n > 0 ? 1 : 0);
  std::atomic<uint64_t> wide{0}, leaves{0};
  parallel_for(n, threads, [&](uint64_t i) {
    Ray<R> r;
    r.origin = Vec3<R>(R(rays[6 * i]), R(rays[6 * i + 1]), R(rays[6 * i + 2]));
    r.dir = Vec3<R>(R(rays[6 * i + 3]), R(rays[6 * i + 4]), R(rays[6 * i + 5]));
    RayHit<R> h;
    uint32_t f;
    VisitStats st;
    bool ok = pose7 ? m->cast_ray_and_get_normal(iso, r, R(max_toi), lowest_index != 0, &h, &f, stats ? &st : nullptr)
                    : m->cast_local_ray_and_get_normal(r, R(max_toi), lowest_index != 0, &h, &f, stats ? &st : nullptr);
    if (stats) { wide += st.wide_visits; leaves += st.leaf_tests; }
    if (ok) {
      feat[i] = f;
      if (toi) toi[i] = O(h.toi);
      if (normal) { normal[3 * i] = O(h.normal.x); normal[3 * i + 1] = O(h.normal.y); normal[3 * i + 2] = O(h.normal.z); }
    } else {
      feat[i] = UINT32_MAX;
      if (toi) toi[i] = O(0);
      if (normal) { normal[3 * i] = 0; normal[3 * i + 1] = 0; normal[3 * i + 2] = 0; }
    }
  });
  if (stats) { stats[0] = wide.load(); stats[1] = leaves.load(); }
}

template <class R> Bvh<R>* make_bvh(const float* aabbs, uint32_t n) {
  std::vector<Aabb<R>> v(n);
  for (uint32_t i = 0; i < n; ++i)
    v[i] = Aabb<R>(Vec3<R>(R(aabbs[6 * i]), R(aabbs[6 * i + 1]), R(aabbs[6 * i + 2])),
                   Vec3<R>(R(aabbs[6 * i + 3]), R(aabbs[6 * i + 4]), R(aabbs[6 * i + 5])));
  return new Bvh<R>(Bvh<R>::from_leaves(v));
}

struct PairBuf {
  std::vector<uint32_t> v;
};

}  // namespace

extern "C" {

// ---------------- TriMesh ray casts ----------------
void* oracle_trimesh_new_f32(const float* v, uint32_t nv, const uint32_t* idx, uint32_t nt) { return make_mesh<float>(v, nv, idx, nt); }
void* oracle_trimesh_new_f64(const float* v, uint32_t nv, const uint32_t* idx, uint32_t nt) { return make_mesh<double>(v, nv, idx, nt); }
void oracle_trimesh_free_f32(void* m) { delete (TriMesh<float>*)m; }
void oracle_trimesh_free_f64(void* m) { delete (TriMesh<double>*)m; }

void oracle_trimesh_cast_rays_f32(void* m, const float* pose7, const float* rays, uint64_t n, float max_toi, int lowest_index,
                                  int threads, uint32_t* feat, float* toi, float* normal, uint64_t* stats) {
  cast_rays<float, float>((TriMesh<float>*)m, pose7, rays, n, max_toi, lowest_index, threads, feat, toi, normal, stats);
}
void oracle_trimesh_cast_rays_f64(void* m, const float* pose7, const float* rays, uint64_t n, float max_toi, int lowest_index,
                                  int threads, uint32_t* feat, double* toi, double* normal, uint64_t* stats) {
  cast_rays<double, double>((TriMesh<double>*)m, pose7, rays, n, max_toi, lowest_index, threads, feat, toi, normal, stats);
}

// Downloads the mesh BVH in the reference's 64-byte wide-node layout (for structure checks).
uint32_t oracle_trimesh_bvh_nodes_f32(void* m, void* out, uint32_t cap) {
  TriMesh<float>* mm = (TriMesh<float>*)m;
  uint32_t n = (uint32_t)mm->bvh.nodes.size();
  if (out && cap >= n) std::memcpy(out, mm->bvh.nodes.data(), sizeof(BvhNodeWide<float>) * n);
  return n;
}

// ---------------- Bvh ----------------
void* oracle_bvh_new_f32(const float* aabbs, uint32_t n) { return make_bvh<float>(aabbs, n); }
void oracle_bvh_free_f32(void* b) { delete (Bvh<float>*)b; }
uint32_t oracle_bvh_nodes_f32(void* b, void* out, uint32_t cap) {
  Bvh<float>* bb = (Bvh<float>*)b;
  uint32_t n = (uint32_t)bb->nodes.size();
  if (out && cap >= n) std::memcpy(out, bb->nodes.data(), sizeof(BvhNodeWide<float>) * n);
  return n;
}
void oracle_bvh_refit_f32(void* b, const float* aabbs, uint32_t n) {
  std::vector<Aabb<float>> v(n);
  for (uint32_t i = 0; i < n; ++i)
    v[i] = Aabb<float>(Vec3<float>(aabbs[6 * i], aabbs[6 * i + 1], aabbs[6 * i + 2]),
                       Vec3<float>(aabbs[6 * i + 3], aabbs[6 * i + 4], aabbs[6 * i + 5]));
  ((Bvh<float>*)b)->refit(v);
}
// Self pairs: returns an opaque buffer; read with oracle_pairs_count / oracle_pairs_copy.
void* oracle_bvh_self_pairs_f32(void* b) {
  PairBuf* pb = new PairBuf();
  ((Bvh<float>*)b)->traverse_bvtt_single_tree([&](uint32_t x, uint32_t y) { pb->v.push_back(x); pb->v.push_back(y); });
  return pb;
}
void* oracle_bvh_leaf_pairs_f32(void* a, void* b) {
  PairBuf* pb = new PairBuf();
  ((Bvh<float>*)a)->leaf_pairs(*(Bvh<float>*)b, [&](uint32_t x, uint32_t y) { pb->v.push_back(x); pb->v.push_back(y); });
  return pb;
}
uint64_t oracle_pairs_count(void* p) { return ((PairBuf*)p)->v.size() / 2; }
void oracle_pairs_copy(void* p, uint32_t* out) { std::memcpy(out, ((PairBuf*)p)->v.data(), ((PairBuf*)p)->v.size() * 4); }
void oracle_pairs_free(void* p) { delete (PairBuf*)p; }

}  // extern "C"
