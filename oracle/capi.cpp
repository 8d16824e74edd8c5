// Oracle (test infrastructure only): flat C entry points over the C++ restatement of parry3d,
// loaded with ctypes by tests/, the smoke check and the bench's CPU-baseline leg. Never linked
// into the product library.
//
// Each function comes in an f32 flavour (parry3d) and an f64 flavour (parry3d-f64); f64 inputs
// are the f32 inputs widened, so the f64 result measures the f32 path's rounding error.
#include "ray.hpp"
#include "contact.hpp"
#include "shape_ray.hpp"
#include "manifold.hpp"
#include "shape_cast.hpp"
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

// A shape set in the C-ABI layout: types[n], params[n x 4], poses[n x 7], convex vertex pool.
// Same field layout as parrygpu_polyhedra (the library's C ABI for ConvexPolyhedron topology).
struct PolyIn {
  uint64_t n_hulls;
  const uint32_t* hulls;
  uint64_t n_faces;
  const float* face_normals;
  const uint32_t* face_ranges;
  uint64_t n_face_entries;
  const uint32_t* face_vertices;
  const uint32_t* face_edges;
  const uint32_t* vertex_ranges;
  uint64_t n_vertex_entries;
  const uint32_t* vertex_faces;
  const uint32_t* vertex_edges;
  uint64_t n_edges;
  const float* edge_dirs;
};

template <class R> struct ShapeSet {
  std::vector<Shape<R>> shapes;
  std::vector<Iso<R>> poses;
  std::vector<Vec3<R>> pool;
  std::vector<HullTopo> topos;
  // Attaches hull topology to convex shapes whose params[2] (u32 bits) holds hull index + 1.
  void attach(const float* params, const PolyIn* ph) {
    if (!ph) return;
    topos.resize(ph->n_hulls);
    for (uint64_t h = 0; h < ph->n_hulls; ++h) {
      const uint32_t* r = ph->hulls + 8 * h;
      HullTopo& t = topos[h];
      t.n_faces = r[3];
      t.n_edges = r[5];
      t.face_normals = ph->face_normals + 3 * (size_t)r[2];
      t.face_ranges = ph->face_ranges + 2 * (size_t)r[2];
      t.face_vertices = ph->face_vertices;
      t.face_edges = ph->face_edges;
      t.vertex_ranges = ph->vertex_ranges + 2 * (size_t)r[0];
      t.vertex_faces = ph->vertex_faces;
      t.vertex_edges = ph->vertex_edges;
      t.edge_dirs = ph->edge_dirs + 3 * (size_t)r[4];
    }
    for (size_t i = 0; i < shapes.size(); ++i) {
      if (shapes[i].type != SHAPE_CONVEX) continue;
      uint32_t h1;
      std::memcpy(&h1, params + 4 * i + 2, 4);
      if (h1 && h1 - 1 < ph->n_hulls && topos[h1 - 1].n_faces) shapes[i].topo = &topos[h1 - 1];
    }
  }
  ShapeSet(const uint32_t* types, const float* params, const float* poses7, const float* hullv, uint32_t nhv, uint64_t n) {
    pool.resize(nhv);
    for (uint32_t i = 0; i < nhv; ++i) pool[i] = Vec3<R>(R(hullv[3 * i]), R(hullv[3 * i + 1]), R(hullv[3 * i + 2]));
    shapes.resize(n);
    poses.resize(n);
    for (uint64_t i = 0; i < n; ++i) {
      Shape<R>& s = shapes[i];
      const float* p = params + 4 * i;
      s.type = types[i];
      if (s.type == SHAPE_BALL) s.radius = R(p[0]);
      else if (s.type == SHAPE_CUBOID) s.half = Vec3<R>(R(p[0]), R(p[1]), R(p[2]));
      else if (s.type == SHAPE_CAPSULE) { s.half_height = R(p[0]); s.radius = R(p[1]); }
      else {
        uint32_t first, count;
        std::memcpy(&first, p, 4);
        std::memcpy(&count, p + 1, 4);
        s.pts = pool.data() + first;
        s.npts = count;
      }
      poses[i] = Iso<R>::from_pose7(poses7 + 7 * i);
    }
  }
};

template <class R, class O>
void contacts(const uint32_t* types, const float* params, const float* poses, const float* hullv, uint32_t nhv, uint64_t nshapes,
              const uint32_t* pairs, uint64_t npairs, float prediction, const float* init_dirs, int threads, O* out, uint8_t* has,
              uint64_t* stats) {
  ShapeSet<R> set(types, params, poses, hullv, nhv, nshapes);
  std::atomic<uint64_t> gi{0}, ei{0}, ec{0}, mf{0}, mv{0}, ms{0}, sv{0};
  auto amax = [](std::atomic<uint64_t>& a, uint64_t v) {
    uint64_t cur = a.load();
    while (v > cur && !a.compare_exchange_weak(cur, v)) {}
  };
  parallel_for(npairs, threads, [&](uint64_t k) {
    uint32_t a = pairs[2 * k], b = pairs[2 * k + 1];
    Contact<R> c;
    GjkStats st;
    Vec3<R> idir;
    const Vec3<R>* ip = nullptr;
    if (init_dirs) {
      idir = Vec3<R>(R(init_dirs[3 * k]), R(init_dirs[3 * k + 1]), R(init_dirs[3 * k + 2]));
      ip = &idir;
    }
    g_support_vertices = 0;
    bool ok = contact_world(set.poses[a], set.shapes[a], set.poses[b], set.shapes[b], R(prediction), &c, &st, ip);
    sv += g_support_vertices;
    gi += st.gjk_iters; ei += st.epa_iters; ec += st.epa_calls;
    amax(mf, st.epa_max_faces); amax(mv, st.epa_max_verts); amax(ms, st.epa_max_sil);
    has[k] = ok ? 1 : 0;
    O* o = out + 13 * k;
    if (ok) {
      const Vec3<R>* v[4] = {&c.point1, &c.point2, &c.normal1, &c.normal2};
      for (int j = 0; j < 4; ++j) { o[3 * j] = O(v[j]->x); o[3 * j + 1] = O(v[j]->y); o[3 * j + 2] = O(v[j]->z); }
      o[12] = O(c.dist);
    } else {
      for (int j = 0; j < 13; ++j) o[j] = O(0);
    }
  });
  if (stats) {
    stats[0] = gi.load(); stats[1] = ei.load(); stats[2] = ec.load();
    stats[3] = mf.load(); stats[4] = mv.load(); stats[5] = ms.load(); stats[6] = sv.load();
  }
}

// query::cast_shapes per (a, b) pair; vels = per-shape linear velocities (n x 3). opts = max toi,
// target distance, stop_at_penetration, compute_impact_geometry_on_penetration. out per pair:
// toi, witness1, witness2, normal1, normal2 (13 values); status[k] = ShapeCastStatus or 0xff (None).
template <class R, class O>
void cast_shapes_batch(const uint32_t* types, const float* params, const float* poses, const float* hullv, uint32_t nhv, uint64_t nshapes,
                       const uint32_t* pairs, uint64_t npairs, const float* vels, const float* opts, int threads, O* out, uint8_t* status,
                       uint64_t* stats) {
  ShapeSet<R> set(types, params, poses, hullv, nhv, nshapes);
  ShapeCastOptions<R> opt;
  opt.max_time_of_impact = R(opts[0]);
  opt.target_distance = R(opts[1]);
  opt.stop_at_penetration = opts[2] != 0.0f;
  opt.compute_impact_geometry_on_penetration = opts[3] != 0.0f;
  std::atomic<uint64_t> gi{0}, ei{0}, ec{0};
  parallel_for(npairs, threads, [&](uint64_t k) {
    uint32_t a = pairs[2 * k], b = pairs[2 * k + 1];
    Vec3<R> v1(R(vels[3 * a]), R(vels[3 * a + 1]), R(vels[3 * a + 2])), v2(R(vels[3 * b]), R(vels[3 * b + 1]), R(vels[3 * b + 2]));
    ShapeCastHit<R> h;
    GjkStats st;
    bool ok = cast_shapes(set.poses[a], v1, set.shapes[a], set.poses[b], v2, set.shapes[b], opt, &h, &st);
    gi += st.gjk_iters; ei += st.epa_iters; ec += st.epa_calls;
    O* o = out + 13 * k;
    if (ok) {
      o[0] = O(h.toi);
      const Vec3<R>* v[4] = {&h.witness1, &h.witness2, &h.normal1, &h.normal2};
      for (int j = 0; j < 4; ++j) { o[1 + 3 * j] = O(v[j]->x); o[2 + 3 * j] = O(v[j]->y); o[3 + 3 * j] = O(v[j]->z); }
      status[k] = (uint8_t)h.status;
    } else {
      for (int j = 0; j < 13; ++j) o[j] = O(0);
      status[k] = 0xff;
    }
  });
  if (stats) { stats[0] = gi.load(); stats[1] = ei.load(); stats[2] = ec.load(); }
}

template <class R> Compound<R>* make_compound(const uint32_t* types, const float* params, const float* poses, const float* hullv,
                                              uint32_t nhv, uint64_t n) {
  Compound<R>* c = new Compound<R>();
  ShapeSet<R> set(types, params, poses, hullv, nhv, n);
  c->shapes = set.shapes;
  c->poses = set.poses;
  c->pool = std::move(set.pool);  // the buffer moves with the vector: shape pointers stay valid
  c->build();
  return c;
}

template <class R, class O>
void compound_cast(const Compound<R>* c, const float* pose7, const float* rays, uint64_t n, float max_toi, int solid, int lowest,
                   int threads, uint32_t* part, O* toi, O* normal, uint64_t* stats) {
  Iso<R> iso = pose7 ? Iso<R>::from_pose7(pose7) : Iso<R>::identity();
  std::atomic<uint64_t> wide{0}, leaves{0};
  parallel_for(n, threads, [&](uint64_t i) {
    Ray<R> r;
    r.origin = Vec3<R>(R(rays[6 * i]), R(rays[6 * i + 1]), R(rays[6 * i + 2]));
    r.dir = Vec3<R>(R(rays[6 * i + 3]), R(rays[6 * i + 4]), R(rays[6 * i + 5]));
    if (pose7) r = Ray<R>{iso.inverse_transform_point(r.origin), iso.inverse_transform_vector(r.dir)};
    uint32_t p;
    R t;
    Vec3<R> nn;
    VisitStats st;
    bool ok = c->cast_local_ray_and_get_normal(r, R(max_toi), solid != 0, lowest != 0, &p, &t, &nn, stats ? &st : nullptr);
    if (stats) { wide += st.wide_visits; leaves += st.leaf_tests; }
    if (ok && pose7) nn = iso.transform_vector(nn);
    part[i] = ok ? p : UINT32_MAX;
    toi[i] = ok ? O(t) : O(0);
    normal[3 * i] = ok ? O(nn.x) : O(0);
    normal[3 * i + 1] = ok ? O(nn.y) : O(0);
    normal[3 * i + 2] = ok ? O(nn.z) : O(0);
  });
  if (stats) { stats[0] = wide.load(); stats[1] = leaves.load(); }
}


// Manifold record (same words as parrygpu_manifold): n_points, status, local_n1[3], local_n2[3],
// then MAX_POINTS x {local_p1[3], local_p2[3], dist, fid1, fid2, data}.
constexpr int MF_MAX_POINTS = 24;
constexpr int MF_WORDS = 8 + 10 * MF_MAX_POINTS;

inline float wf(uint32_t w) { float f; std::memcpy(&f, &w, 4); return f; }
inline uint32_t fw(float f) { uint32_t w; std::memcpy(&w, &f, 4); return w; }

inline void manifold_load(const uint32_t* r, Manifold<float>& m) {
  uint32_t n = r[0] > (uint32_t)MF_MAX_POINTS ? (uint32_t)MF_MAX_POINTS : r[0];
  m.local_n1 = Vec3<float>(wf(r[2]), wf(r[3]), wf(r[4]));
  m.local_n2 = Vec3<float>(wf(r[5]), wf(r[6]), wf(r[7]));
  m.points.resize(n);
  for (uint32_t i = 0; i < n; ++i) {
    const uint32_t* q = r + 8 + 10 * i;
    TrackedContact<float>& c = m.points[i];
    c.local_p1 = Vec3<float>(wf(q[0]), wf(q[1]), wf(q[2]));
    c.local_p2 = Vec3<float>(wf(q[3]), wf(q[4]), wf(q[5]));
    c.dist = wf(q[6]);
    c.fid1 = q[7];
    c.fid2 = q[8];
    c.data = wf(q[9]);
  }
}

inline void manifold_store(const Manifold<float>& m, uint32_t* r) {
  r[0] = (uint32_t)m.points.size();
  r[2] = fw(m.local_n1.x); r[3] = fw(m.local_n1.y); r[4] = fw(m.local_n1.z);
  r[5] = fw(m.local_n2.x); r[6] = fw(m.local_n2.y); r[7] = fw(m.local_n2.z);
  for (size_t i = 0; i < m.points.size() && i < (size_t)MF_MAX_POINTS; ++i) {
    uint32_t* q = r + 8 + 10 * i;
    const TrackedContact<float>& c = m.points[i];
    q[0] = fw(c.local_p1.x); q[1] = fw(c.local_p1.y); q[2] = fw(c.local_p1.z);
    q[3] = fw(c.local_p2.x); q[4] = fw(c.local_p2.y); q[5] = fw(c.local_p2.z);
    q[6] = fw(c.dist);
    q[7] = c.fid1;
    q[8] = c.fid2;
    q[9] = fw(c.data);
  }
}

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
// ---------------- convex shapes: AABBs and query::contact ----------------
void oracle_shape_aabbs_f32(const uint32_t* types, const float* params, const float* poses, const float* hullv, uint32_t nhv,
                            uint64_t n, float margin, float* out) {
  ShapeSet<float> set(types, params, poses, hullv, nhv, n);
  for (uint64_t i = 0; i < n; ++i) {
    Aabb<float> a = shape_aabb(set.shapes[i], set.poses[i]);
    if (margin > 0.0f) a = a.loosened(margin);
    out[6 * i + 0] = a.mins.x; out[6 * i + 1] = a.mins.y; out[6 * i + 2] = a.mins.z;
    out[6 * i + 3] = a.maxs.x; out[6 * i + 4] = a.maxs.y; out[6 * i + 5] = a.maxs.z;
  }
}
void oracle_contacts_f32(const uint32_t* types, const float* params, const float* poses, const float* hullv, uint32_t nhv,
                         uint64_t nshapes, const uint32_t* pairs, uint64_t npairs, float prediction, const float* init_dirs,
                         int threads, float* out, uint8_t* has, uint64_t* stats) {
  contacts<float, float>(types, params, poses, hullv, nhv, nshapes, pairs, npairs, prediction, init_dirs, threads, out, has, stats);
}
void oracle_contacts_f64(const uint32_t* types, const float* params, const float* poses, const float* hullv, uint32_t nhv,
                         uint64_t nshapes, const uint32_t* pairs, uint64_t npairs, float prediction, const float* init_dirs,
                         int threads, double* out, uint8_t* has, uint64_t* stats) {
  contacts<double, double>(types, params, poses, hullv, nhv, nshapes, pairs, npairs, prediction, init_dirs, threads, out, has, stats);
}

// ---------------- Compound (shape set) ray casts ----------------
void* oracle_compound_new_f32(const uint32_t* t, const float* p, const float* q, const float* v, uint32_t nv, uint64_t n) {
  return make_compound<float>(t, p, q, v, nv, n);
}
void* oracle_compound_new_f64(const uint32_t* t, const float* p, const float* q, const float* v, uint32_t nv, uint64_t n) {
  return make_compound<double>(t, p, q, v, nv, n);
}
void oracle_compound_free_f32(void* c) { delete (Compound<float>*)c; }
void oracle_compound_free_f64(void* c) { delete (Compound<double>*)c; }
void oracle_compound_cast_rays_f32(void* c, const float* pose7, const float* rays, uint64_t n, float max_toi, int solid, int lowest,
                                   int threads, uint32_t* part, float* toi, float* normal, uint64_t* stats) {
  compound_cast<float, float>((Compound<float>*)c, pose7, rays, n, max_toi, solid, lowest, threads, part, toi, normal, stats);
}
void oracle_compound_cast_rays_f64(void* c, const float* pose7, const float* rays, uint64_t n, float max_toi, int solid, int lowest,
                                   int threads, uint32_t* part, double* toi, double* normal, uint64_t* stats) {
  compound_cast<double, double>((Compound<double>*)c, pose7, rays, n, max_toi, solid, lowest, threads, part, toi, normal, stats);
}

// DefaultQueryDispatcher::contact_manifold_convex_convex per (a, b) row of `pairs`, updating the
// records in place. Unsupported pairs keep their record and get status 2; a row (0xFFFFFFFF,
// 0xFFFFFFFF) is an empty slot, skipped with its record untouched. stats: gjk_iters, epa_iters,
// epa_calls, unsupported pairs, largest point count.
// pseudo (may be null): rows of 12 floats (face, e01, e12, e20) of TrianglePseudoNormals; a triangle
// shape of index >= pseudo_first whose params word 2 holds j > 0 has the normal constraints of row
// j - 1. init_dirs (may be null): 3 floats per pair, the polyhedral generator's GJK start direction
// where the record holds no cached normal.
void oracle_manifolds_f32(const uint32_t* types, const float* params, const float* poses, const float* hullv, uint32_t nhv,
                          uint64_t nshapes, const void* poly, const uint32_t* pairs, uint64_t npairs, float prediction, int threads,
                          uint32_t* records, uint64_t* stats, const float* pseudo, uint64_t pseudo_first, const float* init_dirs) {
  ShapeSet<float> set(types, params, poses, hullv, nhv, nshapes);
  set.attach(params, (const PolyIn*)poly);
  std::atomic<uint64_t> gi{0}, ei{0}, ec{0}, un{0}, mx{0};
  auto constraints = [&](uint32_t i, TriPseudoNormals<float>* pn) -> const TriPseudoNormals<float>* {
    if (!pseudo || i < pseudo_first || types[i] != SHAPE_TRIANGLE) return nullptr;
    uint32_t j;
    std::memcpy(&j, params + 4 * (size_t)i + 2, 4);
    if (j == 0) return nullptr;
    const float* q = pseudo + 12 * (size_t)(j - 1);
    pn->face = Vec3<float>(q[0], q[1], q[2]);
    for (int e = 0; e < 3; ++e) pn->edges[e] = Vec3<float>(q[3 + 3 * e], q[4 + 3 * e], q[5 + 3 * e]);
    return pn;
  };
  parallel_for(npairs, threads, [&](uint64_t k) {
    uint32_t a = pairs[2 * k], b = pairs[2 * k + 1];
    if (a == 0xFFFFFFFFu && b == 0xFFFFFFFFu) return;
    uint32_t* r = records + (size_t)MF_WORDS * k;
    Manifold<float> m;
    manifold_load(r, m);
    GjkStats st;
    Iso<float> pos12 = set.poses[a].inv_mul(set.poses[b]);
    TriPseudoNormals<float> pa, pb;
    const TriPseudoNormals<float>* ca = constraints(a, &pa);
    const TriPseudoNormals<float>* cb = constraints(b, &pb);
    Vec3<float> learned;
    if (init_dirs) learned = Vec3<float>(init_dirs[3 * k], init_dirs[3 * k + 1], init_dirs[3 * k + 2]);
    bool ok = contact_manifold_convex_convex(pos12, set.shapes[a], set.shapes[b], prediction, m, &st, ca, cb, init_dirs ? &learned : nullptr);
    gi += st.gjk_iters; ei += st.epa_iters; ec += st.epa_calls;
    if (!ok) { un += 1; r[1] = 2; return; }
    r[1] = 0;
    uint64_t np = m.points.size(), cur = mx.load();
    while (np > cur && !mx.compare_exchange_weak(cur, np)) {}
    manifold_store(m, r);
  });
  if (stats) { stats[0] = gi.load(); stats[1] = ei.load(); stats[2] = ec.load(); stats[3] = un.load(); stats[4] = mx.load(); }
}

// TriMesh::triangle_normal_constraints of every triangle of a FIX_INTERNAL_EDGES mesh (12 floats per
// triangle: face, e01, e12, e20; valid = 1 when Some).
void oracle_trimesh_pseudo_normals_f32(const float* vtx, uint32_t nv, const uint32_t* idx, uint32_t nt, float* out, uint8_t* valid) {
  trimesh_pseudo_normals<float>(vtx, nv, idx, nt, out, valid);
}

// TrianglePseudoNormals::project_local_normal for n (pseudo-normals, direction) rows; ok = 1 when Some.
void oracle_project_local_normals_f32(const float* pn12, const float* dirs, uint64_t n, float* out, uint8_t* ok) {
  for (uint64_t i = 0; i < n; ++i) {
    const float* q = pn12 + 12 * i;
    TriPseudoNormals<float> pn;
    pn.face = Vec3<float>(q[0], q[1], q[2]);
    for (int e = 0; e < 3; ++e) pn.edges[e] = Vec3<float>(q[3 + 3 * e], q[4 + 3 * e], q[5 + 3 * e]);
    Vec3<float> d(dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]);
    ok[i] = project_local_normal_mut(pn, &d) ? 1 : 0;
    out[3 * i] = d.x; out[3 * i + 1] = d.y; out[3 * i + 2] = d.z;
  }
}

// Pose integration of the frame pipeline (decision D-5; parry has no integrator), f32, in this
// evaluation order: x += v dt; r = (0, w) q; q := (q + r dt/2) / |q + r dt/2|.
void oracle_integrate_f32(float* poses, const float* vel, uint64_t n, float dt) {
  for (uint64_t i = 0; i < n; ++i) {
    float* p = poses + 7 * i;
    const float* v = vel + 6 * i;
    float qi = p[0], qj = p[1], qk = p[2], qw = p[3];
    float wx = v[3], wy = v[4], wz = v[5];
    float h = 0.5f * dt;
    float ri = (wx * qw + wy * qk) - wz * qj;
    float rj = (wy * qw + wz * qi) - wx * qk;
    float rk = (wz * qw + wx * qj) - wy * qi;
    float rw = -((wx * qi + wy * qj) + wz * qk);
    qi = qi + ri * h;
    qj = qj + rj * h;
    qk = qk + rk * h;
    qw = qw + rw * h;
    float l = std::sqrt(((qi * qi + qj * qj) + qk * qk) + qw * qw);
    p[0] = qi / l;
    p[1] = qj / l;
    p[2] = qk / l;
    p[3] = qw / l;
    p[4] = p[4] + v[0] * dt;
    p[5] = p[5] + v[1] * dt;
    p[6] = p[6] + v[2] * dt;
  }
}

uint64_t oracle_pairs_count(void* p) { return ((PairBuf*)p)->v.size() / 2; }
void oracle_pairs_copy(void* p, uint32_t* out) { std::memcpy(out, ((PairBuf*)p)->v.data(), ((PairBuf*)p)->v.size() * 4); }
void oracle_pairs_free(void* p) { delete (PairBuf*)p; }

void oracle_cast_shapes_f32(const uint32_t* types, const float* params, const float* poses, const float* hullv, uint32_t nhv,
                            uint64_t nshapes, const uint32_t* pairs, uint64_t npairs, const float* vels, const float* opts, int threads,
                            float* out, uint8_t* status, uint64_t* stats) {
  cast_shapes_batch<float, float>(types, params, poses, hullv, nhv, nshapes, pairs, npairs, vels, opts, threads, out, status, stats);
}
void oracle_cast_shapes_f64(const uint32_t* types, const float* params, const float* poses, const float* hullv, uint32_t nhv,
                            uint64_t nshapes, const uint32_t* pairs, uint64_t npairs, const float* vels, const float* opts, int threads,
                            double* out, uint8_t* status, uint64_t* stats) {
  cast_shapes_batch<double, double>(types, params, poses, hullv, nhv, nshapes, pairs, npairs, vels, opts, threads, out, status, stats);
}

// pos1^-1 * pos2 for one pose1 and n poses2 (Isometry::inv_mul), as pose7.
void oracle_inv_mul_f32(const float* pose1, const float* poses2, uint64_t n, float* out) {
  Iso<float> p1 = Iso<float>::from_pose7(pose1);
  for (uint64_t i = 0; i < n; ++i) {
    Iso<float> r = p1.inv_mul(Iso<float>::from_pose7(poses2 + 7 * i));
    float* o = out + 7 * i;
    o[0] = r.rot.i; o[1] = r.rot.j; o[2] = r.rot.k; o[3] = r.rot.w;
    o[4] = r.tra.x; o[5] = r.tra.y; o[6] = r.tra.z;
  }
}

}  // extern "C"
