// Oracle (test infrastructure only): CPU restatement of parry3d's 3-D EPA
// (src/query/epa/epa3.rs:17-675, paths relative to the parry repository), including the pop order
// of Rust's std BinaryHeap (max-heap: push = append + sift_up; pop = take last, swap into the root,
// sift_down_to_bottom, sift_up), because ties between face distances decide which face EPA expands.
#pragma once
#include "gjk.hpp"

namespace oracle {

template <class R> struct FaceId {
  size_t id;
  R neg_dist;
};

// FaceId::cmp (epa3.rs:39-51): NaN compares Equal.
template <class R> inline int faceid_cmp(const FaceId<R>& a, const FaceId<R>& b) {
  if (a.neg_dist < b.neg_dist) return -1;
  if (a.neg_dist > b.neg_dist) return 1;
  return 0;
}

// Rust alloc::collections::BinaryHeap<T: Ord> restated for FaceId.
template <class R> struct RustHeap {
  std::vector<FaceId<R>> d;
  void clear() { d.clear(); }
  bool empty() const { return d.empty(); }
  size_t sift_up(size_t start, size_t pos) {
    FaceId<R> elem = d[pos];
    while (pos > start) {
      size_t parent = (pos - 1) / 2;
      if (faceid_cmp(elem, d[parent]) <= 0) break;
      d[pos] = d[parent];
      pos = parent;
    }
    d[pos] = elem;
    return pos;
  }
  void push(const FaceId<R>& x) {
    size_t old_len = d.size();
    d.push_back(x);
    sift_up(0, old_len);
  }
  void sift_down_to_bottom(size_t pos) {
    size_t end = d.size();
    size_t start = pos;
    FaceId<R> elem = d[pos];
    size_t child = 2 * pos + 1;
    while (end >= 2 && child <= end - 2) {
      child += (faceid_cmp(d[child], d[child + 1]) <= 0) ? 1 : 0;
      d[pos] = d[child];
      pos = child;
      child = 2 * pos + 1;
    }
    if (child == end - 1) {
      d[pos] = d[child];
      pos = child;
    }
    d[pos] = elem;
    sift_up(start, pos);
  }
  bool pop(FaceId<R>* out) {
    if (d.empty()) return false;
    FaceId<R> item = d.back();
    d.pop_back();
    if (!d.empty()) {
      std::swap(item, d[0]);
      sift_down_to_bottom(0);
    }
    *out = item;
    return true;
  }
  bool peek(FaceId<R>* out) const {
    if (d.empty()) return false;
    *out = d[0];
    return true;
  }
};

template <class R> struct EpaFace {
  size_t pts[3];
  size_t adj[3];
  Vec3<R> normal;
  R bcoords[3];
  bool deleted;
};

template <class R> struct Epa {
  std::vector<CSOPoint<R>> vertices;
  std::vector<EpaFace<R>> faces;
  std::vector<std::pair<size_t, size_t>> silhouette;  // (face id, opposite point id)
  RustHeap<R> heap;

  // Face::new_with_proj (epa3.rs:63-88)
  EpaFace<R> new_with_proj(const R bc[3], const size_t pts[3], const size_t adj[3]) {
    EpaFace<R> f;
    for (int i = 0; i < 3; ++i) { f.pts[i] = pts[i]; f.adj[i] = adj[i]; f.bcoords[i] = bc[i]; }
    Vec3<R> ab = vertices[pts[1]].point - vertices[pts[0]].point;
    Vec3<R> ac = vertices[pts[2]].point - vertices[pts[0]].point;
    Vec3<R> n;
    if (!try_normalize(cross(ab, ac), eps_default<R>(), &n)) n = Vec3<R>();
    f.normal = n;
    f.deleted = false;
    return f;
  }

  // Face::new (epa3.rs:90-118): returns the face and whether the origin projects inside it.
  EpaFace<R> new_face(const size_t pts[3], const size_t adj[3], bool* proj_inside) {
    Loc<R> loc;
    Vec3<R> o;
    Vec3<R> proj = project_triangle(vertices[pts[0]].point, vertices[pts[1]].point, vertices[pts[2]].point, o, &loc);
    R bc[3] = {0, 0, 0};
    if (loc.kind == LOC_VERTEX || loc.kind == LOC_EDGE) {
      if (loc.kind == LOC_VERTEX) bc[loc.id] = R(1);
      else {
        int i0 = loc.id == 0 ? 0 : (loc.id == 1 ? 1 : 0);
        int i1 = loc.id == 0 ? 1 : 2;
        bc[i0] = loc.bc[0];
        bc[i1] = loc.bc[1];
      }
      // PointProjection::is_inside = relative_eq!(proj, origin) (|component| <= EPSILON), then
      // is_inside_eps(origin, 100 * EPSILON)
      R e = eps_default<R>();
      bool is_inside = std::fabs(proj.x) <= e && std::fabs(proj.y) <= e && std::fabs(proj.z) <= e;
      R tol = e * R(100);
      *proj_inside = is_inside || norm_squared(proj) < tol * tol;
      return new_with_proj(bc, pts, adj);
    }
    if (loc.kind == LOC_FACE) {
      *proj_inside = true;
      return new_with_proj(loc.bc, pts, adj);
    }
    *proj_inside = false;
    return new_with_proj(bc, pts, adj);
  }

  void face_closest_points(const EpaFace<R>& f, Vec3<R>* p1, Vec3<R>* p2) const {
    *p1 = (vertices[f.pts[0]].orig1 * f.bcoords[0] + vertices[f.pts[1]].orig1 * f.bcoords[1]) + vertices[f.pts[2]].orig1 * f.bcoords[2];
    *p2 = (vertices[f.pts[0]].orig2 * f.bcoords[0] + vertices[f.pts[1]].orig2 * f.bcoords[1]) + vertices[f.pts[2]].orig2 * f.bcoords[2];
  }

  static size_t next_ccw_pt_id(const EpaFace<R>& f, size_t id) {
    if (f.pts[0] == id) return 1;
    if (f.pts[1] == id) return 2;
    return 0;
  }

  bool can_be_seen_by(const EpaFace<R>& f, size_t point, size_t opp) const {
    const Vec3<R>& p0 = vertices[f.pts[opp]].point;
    const Vec3<R>& p1 = vertices[f.pts[(opp + 1) % 3]].point;
    const Vec3<R>& p2 = vertices[f.pts[(opp + 2) % 3]].point;
    const Vec3<R>& pt = vertices[point].point;
    if (dot(pt - p0, f.normal) >= -gjk_eps_tol<R>()) return true;
    // Triangle::is_affinely_dependent (triangle.rs:534-546)
    R e = eps_default<R>() * R(100);
    R sq = norm_squared(cross(p2 - p1, pt - p1));
    return std::fabs(sq) <= e * e;
  }

  void compute_silhouette(size_t point, size_t id, size_t opp) {
    if (faces[id].deleted) return;
    if (!can_be_seen_by(faces[id], point, opp)) {
      silhouette.push_back({id, opp});
    } else {
      faces[id].deleted = true;
      size_t a1 = (opp + 2) % 3, a2 = opp;
      size_t adj1 = faces[id].adj[a1], adj2 = faces[id].adj[a2];
      size_t o1 = next_ccw_pt_id(faces[adj1], faces[id].pts[a1]);
      size_t o2 = next_ccw_pt_id(faces[adj2], faces[id].pts[a2]);
      compute_silhouette(point, adj1, o1);
      compute_silhouette(point, adj2, o2);
    }
  }

  // EPA::closest_points (epa3.rs:428-651). Returns false for None.
  bool closest_points(const Iso<R>& pos12, const Support<R>& g1, const Support<R>& g2, const VoronoiSimplex<R>& simplex,
                      Vec3<R>* p1, Vec3<R>* p2, Vec3<R>* n, GjkStats* st = nullptr) {
    const R eps = eps_default<R>();
    const R eps_tol = eps * R(100);
    vertices.clear(); faces.clear(); heap.clear(); silhouette.clear();
    if (st) st->epa_calls++;
    for (int i = 0; i < simplex.dim + 1; ++i) vertices.push_back(simplex.vertices[i]);
    auto faceid_new = [&](size_t id, R neg_dist, FaceId<R>* out) {
      if (neg_dist > gjk_eps_tol<R>()) return false;
      *out = {id, neg_dist};
      return true;
    };
    if (simplex.dim == 0) {
      *p1 = Vec3<R>(); *p2 = Vec3<R>(); *n = Vec3<R>(0, 1, 0);
      return true;
    } else if (simplex.dim == 3) {
      Vec3<R> dp1 = vertices[1].point - vertices[0].point;
      Vec3<R> dp2 = vertices[2].point - vertices[0].point;
      Vec3<R> dp3 = vertices[3].point - vertices[0].point;
      if (dot(cross(dp1, dp2), dp3) > R(0)) std::swap(vertices[1], vertices[2]);
      const size_t P[4][3] = {{0, 1, 2}, {1, 3, 2}, {0, 2, 3}, {0, 3, 1}};
      const size_t A[4][3] = {{3, 1, 2}, {3, 2, 0}, {0, 1, 3}, {2, 1, 0}};
      bool inside[4];
      for (int k = 0; k < 4; ++k) faces.push_back(new_face(P[k], A[k], &inside[k]));
      for (int k = 0; k < 4; ++k) {
        if (inside[k]) {
          R dist = dot(faces[k].normal, vertices[k].point);
          FaceId<R> fid;
          if (!faceid_new(k, -dist, &fid)) return false;
          heap.push(fid);
        }
      }
      if (!(inside[0] || inside[1] || inside[2] || inside[3])) return false;
    } else {
      if (simplex.dim == 1) {
        Vec3<R> v = vertices[1].point - vertices[0].point;
        // nalgebra orthonormal_subspace_basis(&[v]) in 3-D: first basis vector a x v.
        Vec3<R> a = std::fabs(v.x) > std::fabs(v.y) ? Vec3<R>(v.z, R(0), -v.x) : Vec3<R>(R(0), -v.z, v.y);
        a = normalize(a);
        Vec3<R> dir = cross(a, v);
        vertices.push_back(cso_from_shapes(pos12, g1, g2, dir));
      }
      const size_t P1[3] = {0, 1, 2}, P2[3] = {0, 2, 1}, A1[3] = {1, 1, 1}, A2[3] = {0, 0, 0};
      bool dummy;
      faces.push_back(new_face(P1, A1, &dummy));
      faces.push_back(new_face(P2, A2, &dummy));
      FaceId<R> f0, f1;
      if (!faceid_new(0, R(0), &f0)) return false;
      heap.push(f0);
      if (!faceid_new(1, R(0), &f1)) return false;
      heap.push(f1);
    }
    int niter = 0;
    R max_dist = std::numeric_limits<R>::max();
    FaceId<R> best_face_id;
    if (!heap.peek(&best_face_id)) return false;
    R old_dist = R(0);
    FaceId<R> face_id;
    while (heap.pop(&face_id)) {
      EpaFace<R> face = faces[face_id.id];
      if (face.deleted) continue;
      if (st) st->epa_iters++;
      CSOPoint<R> cso = cso_from_shapes(pos12, g1, g2, face.normal);
      size_t support_point_id = vertices.size();
      vertices.push_back(cso);
      R candidate_max_dist = dot(cso.point, face.normal);
      if (candidate_max_dist < max_dist) { best_face_id = face_id; max_dist = candidate_max_dist; }
      R curr_dist = -face_id.neg_dist;
      if (max_dist - curr_dist < eps_tol || (std::fabs(curr_dist - old_dist) < eps && candidate_max_dist < max_dist)) {
        const EpaFace<R>& bf = faces[best_face_id.id];
        face_closest_points(bf, p1, p2);
        *n = bf.normal;
        return true;
      }
      old_dist = curr_dist;
      faces[face_id.id].deleted = true;
      size_t o1 = next_ccw_pt_id(faces[face.adj[0]], face.pts[0]);
      size_t o2 = next_ccw_pt_id(faces[face.adj[1]], face.pts[1]);
      size_t o3 = next_ccw_pt_id(faces[face.adj[2]], face.pts[2]);
      compute_silhouette(support_point_id, face.adj[0], o1);
      compute_silhouette(support_point_id, face.adj[1], o2);
      compute_silhouette(support_point_id, face.adj[2], o3);
      size_t first_new_face_id = faces.size();
      if (st) {
        st->epa_max_sil = std::max<uint64_t>(st->epa_max_sil, silhouette.size());
        st->epa_max_faces = std::max<uint64_t>(st->epa_max_faces, faces.size() + silhouette.size());
        st->epa_max_verts = std::max<uint64_t>(st->epa_max_verts, vertices.size());
      }
      if (silhouette.empty()) return false;
      for (size_t e = 0; e < silhouette.size(); ++e) {
        size_t fid = silhouette[e].first, opp = silhouette[e].second;
        if (faces[fid].deleted) continue;
        size_t new_face_id = faces.size();
        size_t pt_id1 = faces[fid].pts[(opp + 2) % 3];
        size_t pt_id2 = faces[fid].pts[(opp + 1) % 3];
        size_t pts[3] = {pt_id1, pt_id2, support_point_id};
        size_t adj[3] = {fid, new_face_id + 1, new_face_id - 1};
        bool inside;
        EpaFace<R> nf = new_face(pts, adj, &inside);
        faces[fid].adj[(opp + 1) % 3] = new_face_id;
        faces.push_back(nf);
        if (inside) {
          const Vec3<R>& pt = vertices[faces[new_face_id].pts[0]].point;
          R dist = dot(faces[new_face_id].normal, pt);
          if (dist < curr_dist) {
            face_closest_points(face, p1, p2);
            *n = face.normal;
            return true;
          }
          FaceId<R> f;
          if (!faceid_new(new_face_id, -dist, &f)) return false;
          heap.push(f);
        }
      }
      if (first_new_face_id == faces.size()) return false;
      faces[first_new_face_id].adj[2] = faces.size() - 1;
      faces.back().adj[1] = first_new_face_id;
      silhouette.clear();
      niter += 1;
      if (niter > 100) break;
    }
    const EpaFace<R>& bf = faces[best_face_id.id];
    face_closest_points(bf, p1, p2);
    *n = bf.normal;
    return true;
  }
};

}  // namespace oracle
