// Device view of the BVH node layout.
//
// BvhNodeDev mirrors the reference's 32-byte BvhNode (src/partitioning/bvh/bvh_tree.rs:456-467):
//   mins (3 x f32) | children (u32) | maxs (3 x f32) | data (u32: leaf count in the low 30 bits)
// A leaf has leaf count 1 and `children` = its leaf data; an internal node's `children` is the
// index of the WideNode holding its two children. WideNode = {left, right} = 64 bytes, 64-byte
// aligned, loaded as four float4.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

struct BvhNodeDev {
  float3 mins;
  uint32_t children;
  float3 maxs;
  uint32_t data;
};

struct __align__(64) WideNode {
  BvhNodeDev l;
  BvhNodeDev r;
};

static_assert(sizeof(BvhNodeDev) == 32, "BvhNode must be 32 bytes");
static_assert(sizeof(WideNode) == 64, "BvhNodeWide must be 64 bytes");

__device__ __forceinline__ void load_wide(const WideNode* __restrict__ base, uint32_t i, WideNode* out) {
  const float4* p = reinterpret_cast<const float4*>(base + i);
  float4 a = __ldg(p + 0), b = __ldg(p + 1), c = __ldg(p + 2), d = __ldg(p + 3);
  out->l.mins = make_float3(a.x, a.y, a.z);
  out->l.children = __float_as_uint(a.w);
  out->l.maxs = make_float3(b.x, b.y, b.z);
  out->l.data = __float_as_uint(b.w);
  out->r.mins = make_float3(c.x, c.y, c.z);
  out->r.children = __float_as_uint(c.w);
  out->r.maxs = make_float3(d.x, d.y, d.z);
  out->r.data = __float_as_uint(d.w);
}
