// Oracle (test infrastructure only): CPU restatement of the nalgebra arithmetic that parry3d's
// query path relies on. Only tests/, the smoke check and the bench's CPU-baseline leg use this.
//
// Every formula below is written in the evaluation order nalgebra 0.34 uses, because parry's
// results (hit indices, pair sets, GJK branch decisions) depend on exact f32 rounding:
//   - dot(a, b)        = (a0*b0 + a1*b1) + a2*b2           (nalgebra blas.rs, fixed-size 3-D path)
//   - cross(a, b)      = (ay*bz - az*by, az*bx - ax*bz, ax*by - ay*bx)
//   - norm(v)          = sqrt(dot(v, v)); normalize(v) = v / norm(v) (component-wise division)
//   - q * v (unit quat) = t*w + (q.v x t) + v  with t = 2 (q.v x v)
//   - iso * p          = q * p + t ; iso^-1 * p = conj(q) * (p - t)
// The build compiles this with -ffp-contract=off so no multiply-add is fused, as in Rust.
// nalgebra itself is not vendored in the reference tree (crates/parry3d/Cargo.toml:78-80 pins
// nalgebra 0.34 / simba 0.9 by semver range only), so these restatements are unpinned at the
// bit level; the parity tests pin the path end-to-end on the reference's own known answers.
#pragma once
#include <cmath>
#include <cstdint>
#include <limits>
#include <algorithm>

namespace oracle {

// Rust f32::min / f32::max: NaN-ignoring (returns the other operand when one is NaN).
template <class R> inline R rmin(R a, R b) { return std::fmin(a, b); }
template <class R> inline R rmax(R a, R b) { return std::fmax(a, b); }

template <class R> struct Vec3 {
  R x, y, z;
  Vec3() : x(0), y(0), z(0) {}
  Vec3(R a, R b, R c) : x(a), y(b), z(c) {}
  R operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
  R& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
  Vec3 operator+(const Vec3& o) const { return {x + o.x, y + o.y, z + o.z}; }
  Vec3 operator-(const Vec3& o) const { return {x - o.x, y - o.y, z - o.z}; }
  Vec3 operator-() const { return {-x, -y, -z}; }
  Vec3 operator*(R s) const { return {x * s, y * s, z * s}; }
  Vec3 operator/(R s) const { return {x / s, y / s, z / s}; }
  Vec3& operator+=(const Vec3& o) { x += o.x; y += o.y; z += o.z; return *this; }
  Vec3& operator-=(const Vec3& o) { x -= o.x; y -= o.y; z -= o.z; return *this; }
  bool operator==(const Vec3& o) const { return x == o.x && y == o.y && z == o.z; }
  static Vec3 repeat(R v) { return {v, v, v}; }
};

template <class R> inline R dot(const Vec3<R>& a, const Vec3<R>& b) {
  R p0 = a.x * b.x; R p1 = a.y * b.y; R p2 = a.z * b.z;
  return (p0 + p1) + p2;
}
template <class R> inline Vec3<R> cross(const Vec3<R>& a, const Vec3<R>& b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class R> inline R norm_squared(const Vec3<R>& a) { return dot(a, a); }
template <class R> inline R norm(const Vec3<R>& a) { return std::sqrt(dot(a, a)); }
template <class R> inline Vec3<R> normalize(const Vec3<R>& a) { return a / norm(a); }
template <class R> inline Vec3<R> vinf(const Vec3<R>& a, const Vec3<R>& b) {
  return {rmin(a.x, b.x), rmin(a.y, b.y), rmin(a.z, b.z)};
}
template <class R> inline Vec3<R> vsup(const Vec3<R>& a, const Vec3<R>& b) {
  return {rmax(a.x, b.x), rmax(a.y, b.y), rmax(a.z, b.z)};
}
template <class R> inline Vec3<R> vabs(const Vec3<R>& a) {
  return {std::fabs(a.x), std::fabs(a.y), std::fabs(a.z)};
}
template <class R> inline Vec3<R> cmul(const Vec3<R>& a, const Vec3<R>& b) {
  return {a.x * b.x, a.y * b.y, a.z * b.z};
}
// nalgebra Vector::imax: index of the largest component, first index on ties.
template <class R> inline int imax(const Vec3<R>& v) {
  int ip = 0; R m = v.x;
  if (v.y > m) { m = v.y; ip = 1; }
  if (v.z > m) { ip = 2; }
  return ip;
}
template <class R> inline int iamax(const Vec3<R>& v) { return imax(vabs(v)); }
template <class R> inline int iamin(const Vec3<R>& v) {
  Vec3<R> a = vabs(v);
  int ip = 0; R m = a.x;
  if (a.y < m) { m = a.y; ip = 1; }
  if (a.z < m) { ip = 2; }
  return ip;
}

// Unit::try_new(v, min_norm): Some(v / |v|) when |v|^2 > min_norm^2.
template <class R> inline bool try_normalize(const Vec3<R>& v, R min_norm, Vec3<R>* out, R* n_out = nullptr) {
  R sq = norm_squared(v);
  if (sq > min_norm * min_norm) {
    R n = std::sqrt(sq);
    *out = v / n;
    if (n_out) *n_out = n;
    return true;
  }
  return false;
}

// Unit quaternion stored (i, j, k, w) like nalgebra's Quaternion coords.
template <class R> struct Quat {
  R i, j, k, w;
  Quat() : i(0), j(0), k(0), w(1) {}
  Quat(R a, R b, R c, R d) : i(a), j(b), k(c), w(d) {}
  Vec3<R> vec() const { return {i, j, k}; }
  Quat conj() const { return {-i, -j, -k, w}; }
  // nalgebra: UnitQuaternion * Vector3 (unit_quaternion ops, "t = 2 v x rhs; t*w + v x t + rhs").
  Vec3<R> rotate(const Vec3<R>& v) const {
    Vec3<R> qv = vec();
    Vec3<R> t = cross(qv, v) * R(2);
    Vec3<R> c = cross(qv, t);
    return (t * w + c) + v;
  }
  Vec3<R> inv_rotate(const Vec3<R>& v) const { return conj().rotate(v); }
  // Hamilton product self * o.
  Quat operator*(const Quat& o) const {
    // nalgebra Quaternion * Quaternion (quaternion_ops.rs): component formulas.
    return {w * o.i + i * o.w + j * o.k - k * o.j,
            w * o.j - i * o.k + j * o.w + k * o.i,
            w * o.k + i * o.j - j * o.i + k * o.w,
            w * o.w - i * o.i - j * o.j - k * o.k};
  }
  // 3x3 rotation matrix (nalgebra UnitQuaternion::to_rotation_matrix), row-major m[r][c].
  void to_matrix(R m[3][3]) const {
    R ww = w * w, ii = i * i, jj = j * j, kk = k * k;
    R ij = i * j * R(2), wk = w * k * R(2), wj = w * j * R(2);
    R ik = i * k * R(2), jk = j * k * R(2), wi = w * i * R(2);
    m[0][0] = ww + ii - jj - kk; m[0][1] = ij - wk;           m[0][2] = wj + ik;
    m[1][0] = wk + ij;           m[1][1] = ww - ii + jj - kk; m[1][2] = jk - wi;
    m[2][0] = ik - wj;           m[2][1] = wi + jk;           m[2][2] = ww - ii - jj + kk;
  }
};

template <class R> struct Iso {
  Quat<R> rot;
  Vec3<R> tra;
  Iso() {}
  Iso(const Quat<R>& q, const Vec3<R>& t) : rot(q), tra(t) {}
  static Iso identity() { return Iso(); }
  static Iso from_pose7(const float* p) {
    return Iso(Quat<R>(R(p[0]), R(p[1]), R(p[2]), R(p[3])), Vec3<R>(R(p[4]), R(p[5]), R(p[6])));
  }
  Vec3<R> transform_point(const Vec3<R>& p) const { return rot.rotate(p) + tra; }
  Vec3<R> transform_vector(const Vec3<R>& v) const { return rot.rotate(v); }
  Vec3<R> inverse_transform_point(const Vec3<R>& p) const { return rot.inv_rotate(p - tra); }
  Vec3<R> inverse_transform_vector(const Vec3<R>& v) const { return rot.inv_rotate(v); }
  // nalgebra Isometry::inverse_mut: rotation conj, translation conj * (-t).
  Iso inverse() const {
    Quat<R> ci = rot.conj();
    return Iso(ci, ci.rotate(-tra));
  }
  // self * o
  Iso operator*(const Iso& o) const {
    return Iso(rot * o.rot, rot.rotate(o.tra) + tra);
  }
  // Isometry::inv_mul(self, o) = self^-1 * o (nalgebra isometry.rs inv_mul).
  Iso inv_mul(const Iso& o) const {
    Quat<R> ci = rot.conj();
    return Iso(ci * o.rot, ci.rotate(o.tra - tra));
  }
};

// parry utils/isometry_ops.rs:14-19 absolute_transform_vector: |R| * v.
template <class R> inline Vec3<R> absolute_transform_vector(const Iso<R>& m, const Vec3<R>& v) {
  R mat[3][3];
  m.rot.to_matrix(mat);
  // nalgebra matrix * vector: column-major accumulation  r = c0*v0 + c1*v1 + c2*v2.
  Vec3<R> r;
  for (int row = 0; row < 3; ++row) {
    R a0 = std::fabs(mat[row][0]) * v.x;
    R a1 = std::fabs(mat[row][1]) * v.y;
    R a2 = std::fabs(mat[row][2]) * v.z;
    r[row] = (a0 + a1) + a2;
  }
  return r;
}

}  // namespace oracle
