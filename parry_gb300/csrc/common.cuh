// Device-side math shared by every kernel of libparrygpu.
//
// Parity rule: every floating-point expression is written in the evaluation order that parry3d
// (through nalgebra 0.34) uses, and the library is compiled with --fmad=false, so no multiply-add
// is contracted. IEEE division and square root are the nvcc defaults (-prec-div/-prec-sqrt true).
//   dot(a,b)   = (a.x*b.x + a.y*b.y) + a.z*b.z
//   cross(a,b) = (ay*bz - az*by, az*bx - ax*bz, ax*by - ay*bx)
//   q*v        = t*w + (q.v x t) + v,  t = 2 (q.v x v)          (unit quaternion rotation)
#pragma once
#include <cstdint>
#include <cfloat>
#include <cuda_runtime.h>

namespace pg {

struct V3 {
  float x, y, z;
};

__host__ __device__ __forceinline__ V3 v3(float x, float y, float z) { return V3{x, y, z}; }
__host__ __device__ __forceinline__ V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
__host__ __device__ __forceinline__ V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
__host__ __device__ __forceinline__ V3 operator-(V3 a) { return v3(-a.x, -a.y, -a.z); }
__host__ __device__ __forceinline__ V3 operator*(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
__host__ __device__ __forceinline__ V3 operator/(V3 a, float s) { return v3(a.x / s, a.y / s, a.z / s); }
__host__ __device__ __forceinline__ float dot(V3 a, V3 b) {
  float p0 = a.x * b.x, p1 = a.y * b.y, p2 = a.z * b.z;
  return (p0 + p1) + p2;
}
__host__ __device__ __forceinline__ V3 cross(V3 a, V3 b) {
  return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__host__ __device__ __forceinline__ float norm(V3 a) { return sqrtf(dot(a, a)); }
__host__ __device__ __forceinline__ V3 normalize(V3 a) { return a / norm(a); }
__host__ __device__ __forceinline__ V3 vmin(V3 a, V3 b) { return v3(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z)); }
__host__ __device__ __forceinline__ V3 vmax(V3 a, V3 b) { return v3(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z)); }
__host__ __device__ __forceinline__ float comp(V3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }

// Unit quaternion (i, j, k, w) + translation: the reference's Isometry<f32>.
struct Pose {
  float qi, qj, qk, qw;
  V3 t;
};

__host__ __device__ __forceinline__ V3 quat_rotate(float qi, float qj, float qk, float qw, V3 v) {
  V3 qv = v3(qi, qj, qk);
  V3 t = cross(qv, v) * 2.0f;
  V3 c = cross(qv, t);
  return (t * qw + c) + v;
}
__host__ __device__ __forceinline__ V3 pose_rotate(const Pose& p, V3 v) { return quat_rotate(p.qi, p.qj, p.qk, p.qw, v); }
__host__ __device__ __forceinline__ V3 pose_inv_rotate(const Pose& p, V3 v) { return quat_rotate(-p.qi, -p.qj, -p.qk, p.qw, v); }
__host__ __device__ __forceinline__ V3 pose_point(const Pose& p, V3 v) { return pose_rotate(p, v) + p.t; }
__host__ __device__ __forceinline__ V3 pose_inv_point(const Pose& p, V3 v) { return pose_inv_rotate(p, v - p.t); }

// Order-preserving float <-> uint encoding for atomicMin/atomicMax bounds reductions.
__device__ __forceinline__ uint32_t float_flip(float f) {
  uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float float_unflip(uint32_t u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

// Spread the low 10 bits of v so that there are two zero bits between each (30-bit Morton).
__host__ __device__ __forceinline__ uint32_t expand_bits10(uint32_t v) {
  v &= 0x3ffu;
  v = (v * 0x00010001u) & 0xFF0000FFu;
  v = (v * 0x00000101u) & 0x0F00F00Fu;
  v = (v * 0x00000011u) & 0xC30C30C3u;
  v = (v * 0x00000005u) & 0x49249249u;
  return v;
}
__host__ __device__ __forceinline__ uint32_t morton30(float x, float y, float z) {
  // x, y, z already normalised to [0, 1].
  uint32_t xi = (uint32_t)fminf(fmaxf(x * 1024.0f, 0.0f), 1023.0f);
  uint32_t yi = (uint32_t)fminf(fmaxf(y * 1024.0f, 0.0f), 1023.0f);
  uint32_t zi = (uint32_t)fminf(fmaxf(z * 1024.0f, 0.0f), 1023.0f);
  return (expand_bits10(xi) << 2) | (expand_bits10(yi) << 1) | expand_bits10(zi);
}

}  // namespace pg
