// Learned GJK warm start: a small MLP trained and evaluated with hand-written BF16 tensor-core
// kernels. Inference is one fused kernel on the fifth-generation tensor cores (k_mlp_infer_tc:
// tcgen05.mma from shared memory into TMEM accumulators, all five layers per 128-sample tile with
// the weights resident in shared memory); training runs per-layer mma.sync m16n8k16 GEMMs with FP32
// accumulation and separate bias / activation / gradient kernels. No reference counterpart: its only link to the
// reference is the init_dir parameter of contact_support_map_support_map_with_params
// (src/query/contact/contact_support_map_support_map.rs:40-62), and GJK from that start still
// decides the answer - a poor guess only costs iterations.
//
// Network: 48 (39 features + zero padding) -> 128 -> 128 -> 128 -> 128 -> 3, GELU (erf form) after
// each hidden layer, output normalised to a unit direction in the first shape's frame.
// Parameters: FP32 masters + Adam moments; BF16 copies feed the tensor cores. Activations between
// layers are BF16; pre-activations are kept in FP32 for the backward pass.
// Layout of the parameter vector (parrygpu_mlp_get_params): per layer W [out x in] then b [out].
#include "internal.hpp"
#include "common.cuh"
#include "tcgen05.cuh"
#include "contact_device.cuh"
#include <cuda_bf16.h>
#include <vector>
#include <cmath>

using namespace pg;

namespace {

constexpr int IN = PARRYGPU_MLP_IN;
constexpr int HID = PARRYGPU_MLP_HIDDEN;
constexpr int NL = PARRYGPU_MLP_LAYERS;
constexpr int OUT = 3;
constexpr int DIN[NL] = {IN, HID, HID, HID, HID};
constexpr int DOUT[NL] = {HID, HID, HID, HID, OUT};
__host__ __device__ constexpr int din(int l) { return l == 0 ? IN : HID; }
__host__ __device__ constexpr int dout(int l) { return l == NL - 1 ? OUT : HID; }
constexpr int DESC = 16;

__host__ __device__ constexpr uint64_t w_off(int l) {
  uint64_t o = 0;
  for (int i = 0; i < l; ++i) o += (uint64_t)dout(i) * din(i) + dout(i);
  return o;
}
__host__ __device__ constexpr uint64_t b_off(int l) { return w_off(l) + (uint64_t)dout(l) * din(l); }
constexpr uint64_t N_PARAMS = w_off(NL);

typedef __nv_bfloat16 bf16;

// ---------------------------------------------------------------- tensor-core GEMM
// C[M x N] (fp32, ldc) = sum_k A(m, k) B(k, n), A(m,k) = A_COL ? A[k*lda + m] : A[m*lda + k],
// B(k,n) = B_KN ? B[k*ldb + n] : B[n*ldb + k]. 64x64 CTA tile, 32-deep K steps, 4 warps of 32x32,
// operands staged K-contiguous in shared memory, mma.sync.m16n8k16 bf16 -> fp32. Split-K over
// gridDim.z writes partial tiles to C + z * M * ldc (reduced afterwards in a fixed order).
constexpr int GBM = 64, GBN = 64, GBK = 32, GPAD = 8;

__device__ __forceinline__ void mma_bf16(float* d, const uint32_t* a, const uint32_t* b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

template <bool A_COL, bool B_KN>
__global__ void __launch_bounds__(128) k_gemm(const bf16* __restrict__ A, int lda, const bf16* __restrict__ B, int ldb,
                                              float* __restrict__ C, int ldc, int M, int N, int K, int k_per_split) {
  __shared__ __align__(16) bf16 As[GBM][GBK + GPAD];
  __shared__ __align__(16) bf16 Bs[GBN][GBK + GPAD];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = warp >> 1, wn = warp & 1;
  const int m0 = blockIdx.y * GBM, n0 = blockIdx.x * GBN;
  const int kbeg = blockIdx.z * k_per_split;
  const int kend = min(K, kbeg + k_per_split);
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[i][j][q] = 0.0f;
  const bf16 zero = __float2bfloat16(0.0f);
  for (int k0 = kbeg; k0 < kend; k0 += GBK) {
    // stage A tile (64 x 32) as As[m][k]
#pragma unroll
    for (int e = 0; e < (GBM * GBK) / 128; ++e) {
      int idx = e * 128 + tid;
      int m, k;
      if (A_COL) { m = idx % GBM; k = idx / GBM; } else { k = idx % GBK; m = idx / GBK; }
      int gm = m0 + m, gk = k0 + k;
      bf16 v = zero;
      if (gm < M && gk < kend) v = A_COL ? A[(size_t)gk * lda + gm] : A[(size_t)gm * lda + gk];
      As[m][k] = v;
    }
    // stage B tile (32 x 64) as Bs[n][k]
#pragma unroll
    for (int e = 0; e < (GBN * GBK) / 128; ++e) {
      int idx = e * 128 + tid;
      int n, k;
      if (B_KN) { n = idx % GBN; k = idx / GBN; } else { k = idx % GBK; n = idx / GBK; }
      int gn = n0 + n, gk = k0 + k;
      bf16 v = zero;
      if (gn < N && gk < kend) v = B_KN ? B[(size_t)gk * ldb + gn] : B[(size_t)gn * ldb + gk];
      Bs[n][k] = v;
    }
    __syncthreads();
    const int g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int ks = 0; ks < GBK; ks += 16) {
      uint32_t af[2][4], bfr[4][2];
#pragma unroll
      for (int mi = 0; mi < 2; ++mi) {
        int r = wm * 32 + mi * 16 + g;
        af[mi][0] = *reinterpret_cast<const uint32_t*>(&As[r][ks + 2 * t]);
        af[mi][1] = *reinterpret_cast<const uint32_t*>(&As[r + 8][ks + 2 * t]);
        af[mi][2] = *reinterpret_cast<const uint32_t*>(&As[r][ks + 8 + 2 * t]);
        af[mi][3] = *reinterpret_cast<const uint32_t*>(&As[r + 8][ks + 8 + 2 * t]);
      }
#pragma unroll
      for (int ni = 0; ni < 4; ++ni) {
        int c = wn * 32 + ni * 8 + g;
        bfr[ni][0] = *reinterpret_cast<const uint32_t*>(&Bs[c][ks + 2 * t]);
        bfr[ni][1] = *reinterpret_cast<const uint32_t*>(&Bs[c][ks + 8 + 2 * t]);
      }
#pragma unroll
      for (int mi = 0; mi < 2; ++mi)
#pragma unroll
        for (int ni = 0; ni < 4; ++ni) mma_bf16(acc[mi][ni], af[mi], bfr[ni]);
    }
    __syncthreads();
  }
  float* Cz = C + (size_t)blockIdx.z * M * ldc;
  const int g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int mi = 0; mi < 2; ++mi)
#pragma unroll
    for (int ni = 0; ni < 4; ++ni) {
      int r = m0 + wm * 32 + mi * 16 + g;
      int c = n0 + wn * 32 + ni * 8 + 2 * t;
      if (r < M && c < N) Cz[(size_t)r * ldc + c] = acc[mi][ni][0];
      if (r < M && c + 1 < N) Cz[(size_t)r * ldc + c + 1] = acc[mi][ni][1];
      if (r + 8 < M && c < N) Cz[(size_t)(r + 8) * ldc + c] = acc[mi][ni][2];
      if (r + 8 < M && c + 1 < N) Cz[(size_t)(r + 8) * ldc + c + 1] = acc[mi][ni][3];
    }
}

// Sum of `splits` partial [n] arrays in a fixed order.
__global__ void k_reduce_splits(const float* __restrict__ part, int splits, size_t n, float* __restrict__ out) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  float s = 0.0f;
  for (int z = 0; z < splits; ++z) s += part[(size_t)z * n + i];
  out[i] = s;
}

// ---------------------------------------------------------------- elementwise kernels
__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float x) {
  float cdf = 0.5f * (1.0f + erff(x * 0.70710678118654752f));
  float pdf = 0.3989422804014327f * expf(-0.5f * x * x);
  return cdf + x * pdf;
}

// Z += b; A = bf16(gelu(Z)) (hidden layers) or Z += b only (output layer, A = nullptr).
__global__ void k_bias_act(float* __restrict__ Z, const float* __restrict__ b, int rows, int cols, bf16* __restrict__ A) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= (size_t)rows * cols) return;
  float z = Z[i] + b[i % cols];
  Z[i] = z;
  if (A) A[i] = __float2bfloat16(gelu(z));
}

// loss_b = 1 - cos(y, t); dY = d(mean loss)/dy (bf16). Block-reduced loss sum.
__global__ void k_cos_loss(const float* __restrict__ Y, const float* __restrict__ T, int rows, float inv_batch, bf16* __restrict__ dY,
                           float* __restrict__ loss_sum) {
  __shared__ float red[8];
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  float l = 0.0f;
  if (b < rows) {
    V3 y = v3(Y[3 * b], Y[3 * b + 1], Y[3 * b + 2]);
    V3 t = v3(T[3 * b], T[3 * b + 1], T[3 * b + 2]);
    float yy = y.x * y.x + y.y * y.y + y.z * y.z;
    V3 g;
    if (yy < 1e-20f) {
      l = 1.0f;
      g = t * (-inv_batch);
    } else {
      float ny = sqrtf(yy);
      float c = (y.x * t.x + y.y * t.y + y.z * t.z) / ny;
      l = 1.0f - c;
      g = (t / ny - y * (c / yy)) * (-inv_batch);
    }
    dY[3 * b] = __float2bfloat16(g.x);
    dY[3 * b + 1] = __float2bfloat16(g.y);
    dY[3 * b + 2] = __float2bfloat16(g.z);
  }
  for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = l;
  __syncthreads();
  if (threadIdx.x == 0) {
    float s = 0.0f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
    atomicAdd(loss_sum, s);
  }
}

// Output layer gradient as fp32 too (for its bias): dYf = dY (already scaled).
__global__ void k_bf16_to_f32(const bf16* __restrict__ x, size_t n, float* __restrict__ y) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) y[i] = __bfloat162float(x[i]);
}

// dZ = dA * gelu'(Z): fp32 (bias gradient) and bf16 (GEMM operand)
__global__ void k_gelu_back(const float* __restrict__ dA, const float* __restrict__ Z, size_t n, float* __restrict__ dZf,
                            bf16* __restrict__ dZ) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  float g = dA[i] * gelu_grad(Z[i]);
  dZf[i] = g;
  dZ[i] = __float2bfloat16(g);
}

// db[c] = sum over rows of dZ[r][c], fixed order
__global__ void k_colsum(const float* __restrict__ dZ, int rows, int cols, float* __restrict__ db) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cols) return;
  float s = 0.0f;
  for (int r = 0; r < rows; ++r) s += dZ[(size_t)r * cols + c];
  db[c] = s;
}

__global__ void k_adam(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v, size_t n, float lr,
                       float b1, float b2, float eps, float c1, float c2) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  float gi = g[i];
  float mi = b1 * m[i] + (1.0f - b1) * gi;
  float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

__global__ void k_f32_to_bf16(const float* __restrict__ x, size_t n, bf16* __restrict__ y) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) y[i] = __float2bfloat16(x[i]);
}

// Unit direction from the network output; falls back to the reference default (the relative
// translation in the features, else +x) for degenerate outputs.
__global__ void k_normalize_dirs(const float* __restrict__ Y, const float* __restrict__ feat, size_t n, float* __restrict__ dirs) {
  size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (k >= n) return;
  V3 y = v3(Y[3 * k], Y[3 * k + 1], Y[3 * k + 2]);
  float yy = dot(y, y);
  V3 d;
  if (yy > 1e-12f && isfinite(yy)) d = y / sqrtf(yy);
  else {
    V3 t = v3(feat[k * IN + 4], feat[k * IN + 5], feat[k * IN + 6]);
    float tt = dot(t, t);
    d = tt > 1.1920929e-7f * 1.1920929e-7f ? t / sqrtf(tt) : v3(1.f, 0.f, 0.f);
  }
  dirs[3 * k] = d.x;
  dirs[3 * k + 1] = d.y;
  dirs[3 * k + 2] = d.z;
}

__global__ void k_features_to_bf16(const float* __restrict__ f, size_t n, bf16* __restrict__ x) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n * IN) x[i] = __float2bfloat16(f[i]);
}

// ---------------------------------------------------------------- fused inference on tcgen05
// One CTA of 512 threads per SM, persistent over tiles of 128 samples, in two groups of 8 warps that
// take alternate tiles, so that the tensor cores run one group's layer while the other group turns
// its accumulator into activations. Shared memory holds every layer's BF16 weights once, as the B
// operand (N x K, K-major, canonical core-matrix layout: 8 rows x 16 bytes per 128-byte core
// matrix, core matrices along K 128 bytes apart, 8-row groups K/8 x 128 bytes apart), each group's
// tile activations as the A operand in the same layout, and the biases. Per layer a group's first
// thread issues K/16 tcgen05.mma (M = 128, N = 128, or 16 for the 3-wide output layer padded with
// zero rows, K = 16 each) into the group's 128-column FP32 TMEM accumulator and commits them to the
// group's mbarrier; the group's 8 warps then read the accumulator back (warp w of the group: TMEM
// lanes 32 (w % 4) .. + 31, columns 64 (w / 4) .. + 63), add the bias, apply GELU (tanh form with
// one special-function operation, gelu_th) and write the next layer's BF16 activations into
// shared memory. The output layer's 3 columns are normalised
// into the init direction (the fallback of k_normalize_dirs for degenerate outputs). Activations
// never leave the SM. `d_count` (may be null) bounds the rows on the device (min(n, *d_count));
// with `rows`, feature row k's direction goes to row rows[k] of `dirs`.
constexpr int TC_GROUPS = 2;
constexpr int TC_GROUP_THREADS = 256;
constexpr int TC_THREADS = TC_GROUPS * TC_GROUP_THREADS;
constexpr int TC_M = 128;
constexpr int TC_NOUT = 16;  // output layer rows padded to the smallest N of an M = 128 MMA
constexpr uint32_t TC_TMEM_COLS = 128;  // per group
constexpr uint32_t TC_WAIT_POLLS = 1u << 24;
__host__ __device__ constexpr int tc_rows(int l) { return l == NL - 1 ? TC_NOUT : dout(l); }
__host__ __device__ constexpr uint32_t tc_w_bytes(int l) { return (uint32_t)tc_rows(l) * din(l) * 2; }
__host__ __device__ constexpr uint32_t tc_w_off(int l) {
  uint32_t o = 0;
  for (int i = 0; i < l; ++i) o += tc_w_bytes(i);
  return o;
}
constexpr uint32_t TC_ACT_BYTES = TC_M * HID * 2;
constexpr uint32_t TC_ACT_OFF = tc_w_off(NL);                              // per group: 128 x 128 bf16
constexpr uint32_t TC_BIAS_OFF = TC_ACT_OFF + TC_GROUPS * TC_ACT_BYTES;    // (NL - 1) x 128 + 16 floats
constexpr uint32_t TC_BAR_OFF = TC_BIAS_OFF + ((NL - 1) * HID + TC_NOUT) * 4;
constexpr uint32_t TC_SMEM = TC_BAR_OFF + 32;  // 2 mbarriers, the TMEM address, 2 failure flags
static_assert(tc_w_off(1) % 1024 == 0 && TC_ACT_OFF % 1024 == 0 && TC_BAR_OFF % 8 == 0, "aligned shared-memory regions");

// Byte offset of element (r, k) of an R x K K-major operand in the canonical layout.
__device__ __forceinline__ uint32_t tc_off(uint32_t r, uint32_t k, uint32_t K) {
  return ((r >> 3) * (K >> 3) + (k >> 3)) * 128u + (r & 7u) * 16u + (k & 7u) * 2u;
}

// GELU for the inference epilogue in the tanh form of Hendrycks and Gimpel ("Gaussian Error Linear
// Units", 2016: 0.5 x (1 + tanh(u(x)))) with the tanh.approx.f32 instruction: one special-function
// operation per activation where the erf form (1 / (1 + p z) and exp) takes two. Their
// u = sqrt(2 / pi) (x + 0.044715 x^3) departs from the erf form by up to 4.7e-4; the odd polynomial
// here, fitted to the erf form by weighted least squares on [-7, 7] (x clamped there, where tanh
// has saturated), by at most 2.6e-5. What remains is tanh.approx's relative error (2^-11), below the
// BF16 rounding the activation takes next.
__device__ __forceinline__ float tanh_approx(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float gelu_th(float x) {
  const float c = fminf(fmaxf(x, -7.0f), 7.0f), c2 = c * c;
  const float u = c * fmaf(c2, fmaf(c2, -3.50979698e-4f, 3.70024110e-2f), 7.97511410e-1f);
  const float h = 0.5f * x;
  return fmaf(h, tanh_approx(u), h);
}

__device__ __forceinline__ uint32_t pack_bf16x2(float a, float b) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<const uint32_t*>(&v);
}

// Barrier of one group's 256 threads (named barrier 1 + group; 0 is __syncthreads).
__device__ __forceinline__ void group_sync(uint32_t g) { asm volatile("bar.sync %0, %1;" ::"r"(1u + g), "r"(TC_GROUP_THREADS) : "memory"); }

__global__ void __launch_bounds__(TC_THREADS, 1) k_mlp_infer_tc(const float* __restrict__ feat, uint64_t n, const bf16* __restrict__ wb,
                                                                const float* __restrict__ wf, float* __restrict__ dirs,
                                                                uint32_t* __restrict__ err, const unsigned long long* __restrict__ d_count,
                                                                const uint32_t* __restrict__ rows) {
  extern __shared__ __align__(1024) uint8_t tc_smem[];
  if (d_count && *d_count < n) n = *d_count;
  float* bias = reinterpret_cast<float*>(tc_smem + TC_BIAS_OFF);
  uint64_t* bars = reinterpret_cast<uint64_t*>(tc_smem + TC_BAR_OFF);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(tc_smem + TC_BAR_OFF + 16);
  uint32_t* fail = tslot + 1;  // [2]
  const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t g = warp / 8, gtid = tid % TC_GROUP_THREADS, gwarp = warp % 8;
  // weights (16-byte chunks of 8 bf16; padded rows of the output layer are zero) and biases
#pragma unroll
  for (int l = 0; l < NL; ++l) {
    const uint32_t K = din(l), chunks = (uint32_t)tc_rows(l) * (K / 8);
    for (uint32_t c = tid; c < chunks; c += TC_THREADS) {
      const uint32_t r = c / (K / 8), kc = c % (K / 8);
      uint4 v = make_uint4(0u, 0u, 0u, 0u);
      if (r < (uint32_t)dout(l)) v = *reinterpret_cast<const uint4*>(wb + w_off(l) + (size_t)r * K + kc * 8);
      *reinterpret_cast<uint4*>(tc_smem + tc_w_off(l) + tc_off(r, kc * 8, K)) = v;
    }
  }
  for (uint32_t i = tid; i < (NL - 1) * HID + TC_NOUT; i += TC_THREADS) {
    const uint32_t l = i / HID, j = i % HID;
    bias[i] = (l < NL - 1) ? wf[b_off(l) + j] : (j < OUT ? wf[b_off(NL - 1) + j] : 0.0f);
  }
  if (warp == 0) tmem_alloc(tslot, TC_GROUPS * TC_TMEM_COLS);
  if (tid == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    fail[0] = fail[1] = 0;
  }
  tc_fence_before_sync();
  __syncthreads();
  tc_fence_after_sync();
  uint8_t* act = tc_smem + TC_ACT_OFF + g * TC_ACT_BYTES;
  uint64_t* bar = &bars[g];
  const uint32_t tmem = *tslot + g * TC_TMEM_COLS;
  const uint32_t quarter = gwarp & 3, colblk = gwarp >> 2;
  const uint32_t row = quarter * 32 + lane;                       // this thread's TMEM lane = tile row
  const uint32_t tl = tmem + ((quarter * 32u) << 16);             // this warp's TMEM lanes
  uint32_t phase = 0;
  bool failed = false;
  const uint64_t tiles = (n + TC_M - 1) / TC_M;
  for (uint64_t tile = (uint64_t)blockIdx.x * TC_GROUPS + g; tile < tiles && !failed; tile += (uint64_t)gridDim.x * TC_GROUPS) {
    const uint64_t base = tile * TC_M;
    // features -> bf16 A operand (K = 48); rows past n are zero
    for (uint32_t c = gtid; c < TC_M * (IN / 8); c += TC_GROUP_THREADS) {
      const uint32_t r = c / (IN / 8), kc = c % (IN / 8);
      uint4 v = make_uint4(0u, 0u, 0u, 0u);
      if (base + r < n) {
        const float4* src = reinterpret_cast<const float4*>(feat + (base + r) * IN + kc * 8);
        const float4 a = src[0], b = src[1];
        v = make_uint4(pack_bf16x2(a.x, a.y), pack_bf16x2(a.z, a.w), pack_bf16x2(b.x, b.y), pack_bf16x2(b.z, b.w));
      }
      *reinterpret_cast<uint4*>(act + tc_off(r, kc * 8, IN)) = v;
    }
#pragma unroll
    for (int l = 0; l < NL; ++l) {
      const uint32_t K = din(l);
      // the operands written by the threads become visible to the tensor cores' (async) proxy
      fence_async_shared();
      tc_fence_before_sync();
      group_sync(g);
      if (gtid == 0) {
        tc_fence_after_sync();
        const uint32_t sbo = (K / 8) * 128u, idesc = umma_idesc_bf16(TC_M, (uint32_t)tc_rows(l));
        for (uint32_t ks = 0; ks < K / 16; ++ks) {
          const uint64_t ad = umma_desc_kmajor(act + ks * 256u, 128u, sbo);
          const uint64_t bd = umma_desc_kmajor(tc_smem + tc_w_off(l) + ks * 256u, 128u, sbo);
          umma_bf16(tmem, ad, bd, idesc, ks > 0);
        }
        umma_commit(bar);
      }
      if (!mbar_wait_bounded(bar, phase, TC_WAIT_POLLS)) atomicOr(&fail[g], 1u);
      group_sync(g);
      if (fail[g]) {  // the tensor cores did not answer: report, and leave without reading TMEM
        if (gtid == 0) atomicOr(err, ERR_TIMEOUT);
        mbar_wait_bounded(bar, phase, TC_WAIT_POLLS);
        failed = true;
        break;
      }
      phase ^= 1u;
      tc_fence_after_sync();
      if (l < NL - 1) {
        const float* bl = bias + l * HID;
#pragma unroll 1
        for (uint32_t c0 = colblk * 64; c0 < colblk * 64 + 64; c0 += 16) {
          float v[16];
          tmem_ld16(tl + c0, v);
          uint32_t w8[8];
#pragma unroll
          for (int j = 0; j < 8; ++j)
            w8[j] = pack_bf16x2(gelu_th(v[2 * j] + bl[c0 + 2 * j]), gelu_th(v[2 * j + 1] + bl[c0 + 2 * j + 1]));
          *reinterpret_cast<uint4*>(act + tc_off(row, c0, HID)) = make_uint4(w8[0], w8[1], w8[2], w8[3]);
          *reinterpret_cast<uint4*>(act + tc_off(row, c0 + 8, HID)) = make_uint4(w8[4], w8[5], w8[6], w8[7]);
        }
      } else if (colblk == 0) {
        float v[16];
        tmem_ld16(tl, v);
        const uint64_t k = base + row;
        if (k < n) {
          const float* bl = bias + (NL - 1) * HID;
          V3 y = v3(v[0] + bl[0], v[1] + bl[1], v[2] + bl[2]);
          const float yy = dot(y, y);
          V3 d;
          if (yy > 1e-12f && isfinite(yy)) d = y / sqrtf(yy);
          else {
            const V3 t = v3(feat[k * IN + 4], feat[k * IN + 5], feat[k * IN + 6]);
            const float tt = dot(t, t);
            d = tt > 1.1920929e-7f * 1.1920929e-7f ? t / sqrtf(tt) : v3(1.f, 0.f, 0.f);
          }
          const uint64_t o = rows ? rows[k] : k;
          dirs[3 * o] = d.x;
          dirs[3 * o + 1] = d.y;
          dirs[3 * o + 2] = d.z;
        }
      }
    }
    // the accumulator and activations are free for the group's next tile once its threads are done
    tc_fence_before_sync();
    group_sync(g);
    tc_fence_after_sync();
  }
  tc_fence_before_sync();
  __syncthreads();
  tc_fence_after_sync();
  if (warp == 0) tmem_dealloc(*tslot, TC_GROUPS * TC_TMEM_COLS);
}

// ---------------------------------------------------------------- features
// Principal moments: eigenvalues of a symmetric 3x3 matrix (closed form), descending.
__device__ void sym_eig3(float a00, float a01, float a02, float a11, float a12, float a22, float* e) {
  float p1 = a01 * a01 + a02 * a02 + a12 * a12;
  if (p1 <= 1e-30f) {
    float d[3] = {a00, a11, a22};
    for (int i = 0; i < 2; ++i)
      for (int j = 0; j < 2 - i; ++j)
        if (d[j] < d[j + 1]) { float t = d[j]; d[j] = d[j + 1]; d[j + 1] = t; }
    e[0] = d[0]; e[1] = d[1]; e[2] = d[2];
    return;
  }
  float q = (a00 + a11 + a22) / 3.0f;
  float p2 = (a00 - q) * (a00 - q) + (a11 - q) * (a11 - q) + (a22 - q) * (a22 - q) + 2.0f * p1;
  float p = sqrtf(p2 / 6.0f);
  float b00 = (a00 - q) / p, b11 = (a11 - q) / p, b22 = (a22 - q) / p, b01 = a01 / p, b02 = a02 / p, b12 = a12 / p;
  float det = b00 * (b11 * b22 - b12 * b12) - b01 * (b01 * b22 - b12 * b02) + b02 * (b01 * b12 - b11 * b02);
  float r = fminf(fmaxf(det * 0.5f, -1.0f), 1.0f);
  float phi = acosf(r) / 3.0f;
  e[0] = q + 2.0f * p * cosf(phi);
  e[2] = q + 2.0f * p * cosf(phi + 2.0943951023931953f);
  e[1] = 3.0f * q - e[0] - e[2];
}

// 16-float shape descriptor: AABB half extents (3), principal second moments of the shape's
// points (3), vertex count / 256, bounding radius, type one-hot (ball, cuboid, capsule, polyhedron),
// AABB volume, log(vertex count) / log(256), 2 zeros. One warp per shape: the lanes stride over a
// polyhedron's vertices (coalesced reads; the second pass over them hits the cache) and the sums,
// bounds and moments are warp-reduced; lane 0 writes the descriptor.
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_min(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

__global__ void k_shape_desc(const uint32_t* __restrict__ types, const float4* __restrict__ params, const float* __restrict__ pool, uint64_t n,
                             uint64_t n_vertices, float* __restrict__ desc) {
  const uint64_t i = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint32_t lane = threadIdx.x & 31;
  if (i >= n) return;  // whole warps leave together
  uint32_t t = types[i];
  float4 p = params[i];
  float he[3] = {0, 0, 0}, mom[3] = {0, 0, 0}, cnt = 1.0f, rad = 0.0f;
  if (t == 0) {
    he[0] = he[1] = he[2] = p.x;
    mom[0] = mom[1] = mom[2] = 0.2f * p.x * p.x;
    rad = p.x;
  } else if (t == 1) {
    he[0] = p.x; he[1] = p.y; he[2] = p.z;
    float d[3] = {p.x * p.x / 3.0f, p.y * p.y / 3.0f, p.z * p.z / 3.0f};
    sym_eig3(d[0], 0.f, 0.f, d[1], 0.f, d[2], mom);
    cnt = 8.0f;
    rad = sqrtf(p.x * p.x + p.y * p.y + p.z * p.z);
  } else if (t == 2) {
    he[0] = p.y; he[1] = p.x + p.y; he[2] = p.y;
    sym_eig3(0.25f * p.y * p.y, 0.f, 0.f, p.x * p.x / 3.0f + 0.25f * p.y * p.y, 0.f, 0.25f * p.y * p.y, mom);
    cnt = 2.0f;
    rad = p.x + p.y;
  } else {
    uint64_t first = __float_as_uint(p.x), c = __float_as_uint(p.y);
    if (c == 0 || first + c > n_vertices) c = 0;
    const float* v = pool + 3 * first;
    float mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, mx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX}, s[3] = {0, 0, 0}, r2max = 0.0f;
    for (uint64_t j = lane; j < c; j += 32) {
      for (int d = 0; d < 3; ++d) {
        float x = v[3 * j + d];
        mn[d] = fminf(mn[d], x); mx[d] = fmaxf(mx[d], x); s[d] += x;
      }
      r2max = fmaxf(r2max, v[3 * j] * v[3 * j] + v[3 * j + 1] * v[3 * j + 1] + v[3 * j + 2] * v[3 * j + 2]);
    }
    for (int d = 0; d < 3; ++d) { mn[d] = warp_min(mn[d]); mx[d] = warp_max(mx[d]); s[d] = warp_sum(s[d]); }
    rad = sqrtf(warp_max(r2max));
    float inv = c ? 1.0f / (float)c : 0.0f;
    float m[3] = {s[0] * inv, s[1] * inv, s[2] * inv};
    float cxx = 0, cxy = 0, cxz = 0, cyy = 0, cyz = 0, czz = 0;
    for (uint64_t j = lane; j < c; j += 32) {
      float x = v[3 * j] - m[0], y = v[3 * j + 1] - m[1], z = v[3 * j + 2] - m[2];
      cxx += x * x; cxy += x * y; cxz += x * z; cyy += y * y; cyz += y * z; czz += z * z;
    }
    cxx = warp_sum(cxx); cxy = warp_sum(cxy); cxz = warp_sum(cxz); cyy = warp_sum(cyy); cyz = warp_sum(cyz); czz = warp_sum(czz);
    sym_eig3(cxx * inv, cxy * inv, cxz * inv, cyy * inv, cyz * inv, czz * inv, mom);
    for (int d = 0; d < 3; ++d) he[d] = c ? 0.5f * (mx[d] - mn[d]) : 0.0f;
    cnt = (float)c;
    t = 3;
  }
  if (lane != 0) return;
  float* o = desc + 16 * i;
  o[0] = he[0]; o[1] = he[1]; o[2] = he[2];
  o[3] = mom[0]; o[4] = mom[1]; o[5] = mom[2];
  o[6] = cnt / 256.0f;
  o[7] = rad;
  for (int k = 0; k < 4; ++k) o[8 + k] = (t == (uint32_t)k) ? 1.0f : 0.0f;
  o[12] = 8.0f * he[0] * he[1] * he[2];
  o[13] = cnt > 0.0f ? logf(cnt) / logf(256.0f) : 0.0f;
  o[14] = 0.0f;
  o[15] = 0.0f;
}

// Pair features: relative pose of b in a's frame (quaternion with w >= 0, translation), desc(a), desc(b), zeros.
// Row k describes pair k, or pair rows[k] when a row list is given; `d_count` (may be null) holds a
// device-side row count: min(n, *d_count) rows.
__device__ void pair_features(const float* __restrict__ poses, const float* __restrict__ desc, uint32_t a, uint32_t b, uint64_t n_shapes,
                              float* __restrict__ o) {
  for (int j = 0; j < IN; ++j) o[j] = 0.0f;
  if (a >= n_shapes || b >= n_shapes) return;
  const float* pa = poses + 7 * (size_t)a;
  const float* pb = poses + 7 * (size_t)b;
  // q = conj(qa) * qb ; t = conj(qa) (tb - ta)
  float ai = -pa[0], aj = -pa[1], ak = -pa[2], aw = pa[3];
  float bi = pb[0], bj = pb[1], bk = pb[2], bw = pb[3];
  float qi = aw * bi + ai * bw + aj * bk - ak * bj;
  float qj = aw * bj - ai * bk + aj * bw + ak * bi;
  float qk = aw * bk + ai * bj - aj * bi + ak * bw;
  float qw = aw * bw - ai * bi - aj * bj - ak * bk;
  float sgn = qw < 0.0f ? -1.0f : 1.0f;
  V3 t = quat_rotate(ai, aj, ak, aw, v3(pb[4] - pa[4], pb[5] - pa[5], pb[6] - pa[6]));
  o[0] = sgn * qi; o[1] = sgn * qj; o[2] = sgn * qk; o[3] = sgn * qw;
  o[4] = t.x; o[5] = t.y; o[6] = t.z;
  for (int j = 0; j < DESC; ++j) { o[7 + j] = desc[16 * (size_t)a + j]; o[7 + DESC + j] = desc[16 * (size_t)b + j]; }
}

// 128 rows per block turn: each thread builds its row in shared memory, then the block stores the
// rows' contiguous span with 16-byte stores (f must be 16-byte aligned).
constexpr int PF_THREADS = 128;
__global__ void __launch_bounds__(PF_THREADS) k_pair_features(const float* __restrict__ poses, const float* __restrict__ desc,
                                                              const uint32_t* __restrict__ pairs, uint64_t n, uint64_t n_shapes,
                                                              float* __restrict__ f, const uint32_t* __restrict__ rows,
                                                              const unsigned long long* __restrict__ d_count) {
  __shared__ __align__(16) float tile[PF_THREADS * IN];
  if (d_count && *d_count < n) n = *d_count;
  for (uint64_t base = blockIdx.x * (uint64_t)PF_THREADS; base < n; base += (uint64_t)gridDim.x * PF_THREADS) {
    const uint64_t k = base + threadIdx.x;
    if (k < n) {
      const uint64_t p = rows ? rows[k] : k;
      pair_features(poses, desc, pairs[2 * p], pairs[2 * p + 1], n_shapes, tile + threadIdx.x * IN);
    }
    __syncthreads();
    const uint64_t m = n - base < (uint64_t)PF_THREADS ? n - base : (uint64_t)PF_THREADS;
    const float4* src = reinterpret_cast<const float4*>(tile);
    float4* dst = reinterpret_cast<float4*>(f + base * IN);
    for (uint32_t i = threadIdx.x; i < (uint32_t)m * (IN / 4); i += PF_THREADS) dst[i] = src[i];
    __syncthreads();
  }
}

uint64_t splitmix(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

}  // namespace

struct parrygpu_mlp {
  DevBuf w, g, m, v, wb;  // fp32 masters, grads, Adam moments; bf16 weights
  DevBuf gpart;           // split-K partial gradients
  DevBuf x, z[NL], a[NL - 1], dy, df, dz, dzf, dxa, loss;  // activations / gradients of one batch
  uint64_t cap = 0;       // batch capacity of the activation buffers
  uint64_t step = 0;      // Adam step
};

namespace {

template <bool AC, bool BK>
parrygpu_status gemm(parrygpu_ctx* ctx, const bf16* A, int lda, const bf16* B, int ldb, float* C, int ldc, int M, int N, int K, int splits = 1) {
  int kps = ((K + splits - 1) / splits + GBK - 1) / GBK * GBK;
  splits = (K + kps - 1) / kps;
  dim3 grid(div_up(N, GBN), div_up(M, GBM), splits);
  k_gemm<AC, BK><<<grid, 128, 0, ctx->stream>>>(A, lda, B, ldb, C, ldc, M, N, K, kps);
  PG_LAUNCHED(ctx);
  return PARRYGPU_OK;
}

parrygpu_status ensure_cap(parrygpu_ctx* ctx, parrygpu_mlp* mlp, uint64_t n) {
  if (n <= mlp->cap) return PARRYGPU_OK;
  PG_CUDA(ctx, mlp->x.reserve(n * IN * 2));
  for (int l = 0; l < NL; ++l) PG_CUDA(ctx, mlp->z[l].reserve(n * DOUT[l] * 4));
  for (int l = 0; l < NL - 1; ++l) PG_CUDA(ctx, mlp->a[l].reserve(n * HID * 2));
  PG_CUDA(ctx, mlp->dy.reserve(n * OUT * 2));
  PG_CUDA(ctx, mlp->df.reserve(n * HID * 4));
  PG_CUDA(ctx, mlp->dz.reserve(n * HID * 2));
  PG_CUDA(ctx, mlp->dzf.reserve(n * HID * 4));
  PG_CUDA(ctx, mlp->dxa.reserve(n * HID * 4));
  PG_CUDA(ctx, mlp->loss.reserve(16));
  uint64_t splits = (n + 511) / 512;
  PG_CUDA(ctx, mlp->gpart.reserve(splits * HID * HID * 4));
  mlp->cap = n;
  return PARRYGPU_OK;
}

inline const bf16* wbf(const parrygpu_mlp* m, int l) { return m->wb.as<bf16>() + w_off(l); }

// Forward of `n` samples whose bf16 features are in mlp->x; output in z[NL-1] (n x 3).
parrygpu_status forward(parrygpu_ctx* ctx, parrygpu_mlp* mlp, uint64_t n) {
  const bf16* in = mlp->x.as<bf16>();
  for (int l = 0; l < NL; ++l) {
    float* Z = mlp->z[l].as<float>();
    parrygpu_status s = gemm<false, false>(ctx, in, DIN[l], wbf(mlp, l), DIN[l], Z, DOUT[l], (int)n, DOUT[l], DIN[l]);
    if (s != PARRYGPU_OK) return s;
    bf16* A = l < NL - 1 ? mlp->a[l].as<bf16>() : nullptr;
    k_bias_act<<<div_up(n * DOUT[l], 256), 256, 0, ctx->stream>>>(Z, mlp->w.as<float>() + b_off(l), (int)n, DOUT[l], A);
    PG_LAUNCHED(ctx);
    in = A;
  }
  return PARRYGPU_OK;
}

// Backward for the batch in the activation buffers (targets t, n samples); gradients -> mlp->g.
parrygpu_status backward(parrygpu_ctx* ctx, parrygpu_mlp* mlp, const float* t, uint64_t n, uint64_t denom) {
  k_cos_loss<<<div_up(n, 256), 256, 0, ctx->stream>>>(mlp->z[NL - 1].as<float>(), t, (int)n, 1.0f / (float)denom, mlp->dy.as<bf16>(),
                                                      mlp->loss.as<float>());
  PG_LAUNCHED(ctx);
  // output layer: dZ = dY
  const bf16* dZ = mlp->dy.as<bf16>();
  k_bf16_to_f32<<<div_up(n * OUT, 256), 256, 0, ctx->stream>>>(dZ, n * OUT, mlp->dzf.as<float>());
  PG_LAUNCHED(ctx);
  for (int l = NL - 1; l >= 0; --l) {
    int o = DOUT[l], i = DIN[l];
    const bf16* Ain = l > 0 ? mlp->a[l - 1].as<bf16>() : mlp->x.as<bf16>();
    // dW = dZ^T . A_in  (K = batch, split for parallelism; fixed-order reduction)
    int splits = (int)((n + 511) / 512);
    parrygpu_status s = gemm<true, true>(ctx, dZ, o, Ain, i, mlp->gpart.as<float>(), i, o, i, (int)n, splits);
    if (s != PARRYGPU_OK) return s;
    int kps = (((int)n + splits - 1) / splits + GBK - 1) / GBK * GBK;
    int used = ((int)n + kps - 1) / kps;
    k_reduce_splits<<<div_up((size_t)o * i, 256), 256, 0, ctx->stream>>>(mlp->gpart.as<float>(), used, (size_t)o * i,
                                                                         mlp->g.as<float>() + w_off(l));
    PG_LAUNCHED(ctx);
    k_colsum<<<div_up(o, 128), 128, 0, ctx->stream>>>(mlp->dzf.as<float>(), (int)n, o, mlp->g.as<float>() + b_off(l));
    PG_LAUNCHED(ctx);
    if (l == 0) break;
    // dA_in = dZ . W ; dZ_in = dA_in * gelu'(Z_in)
    s = gemm<false, true>(ctx, dZ, o, wbf(mlp, l), i, mlp->df.as<float>(), i, (int)n, i, o);
    if (s != PARRYGPU_OK) return s;
    k_gelu_back<<<div_up(n * i, 256), 256, 0, ctx->stream>>>(mlp->df.as<float>(), mlp->z[l - 1].as<float>(), n * i, mlp->dzf.as<float>(),
                                                            mlp->dz.as<bf16>());
    PG_LAUNCHED(ctx);
    dZ = mlp->dz.as<bf16>();
  }
  return PARRYGPU_OK;
}

parrygpu_status refresh_bf16(parrygpu_ctx* ctx, parrygpu_mlp* mlp) {
  k_f32_to_bf16<<<div_up(N_PARAMS, 256), 256, 0, ctx->stream>>>(mlp->w.as<float>(), N_PARAMS, mlp->wb.as<bf16>());
  PG_LAUNCHED(ctx);
  return PARRYGPU_OK;
}

parrygpu_status load_features(parrygpu_ctx* ctx, parrygpu_mlp* mlp, const float* d_feat, uint64_t n) {
  k_features_to_bf16<<<div_up(n * IN, 256), 256, 0, ctx->stream>>>(d_feat, n, mlp->x.as<bf16>());
  PG_LAUNCHED(ctx);
  return PARRYGPU_OK;
}

}  // namespace

// The frame pipeline's learned seeding: features of the listed pairs, then the fused tensor-core
// inference writing each listed pair's row of the direction buffer.
parrygpu_status pg::launch_seed_dirs(parrygpu_ctx* ctx, const ShapeArrays& sh, const uint32_t* d_pairs, const LearnedSeed& seed,
                                     const unsigned long long* d_count, uint64_t cap) {
  if (cap == 0) return PARRYGPU_OK;
  const uint64_t sms = ctx->sm_count > 0 ? (uint64_t)ctx->sm_count : 152u;
  const uint64_t fgrid = div_up(cap, PF_THREADS) < sms * 16 ? div_up(cap, PF_THREADS) : sms * 16;
  k_pair_features<<<(uint32_t)fgrid, PF_THREADS, 0, ctx->stream>>>(sh.poses, seed.desc, d_pairs, cap, sh.n_shapes, seed.feat, seed.list, d_count);
  PG_LAUNCHED(ctx);
  const uint64_t tiles = (cap + TC_M - 1) / TC_M;
  k_mlp_infer_tc<<<(uint32_t)(tiles < sms ? tiles : sms), TC_THREADS, TC_SMEM, ctx->stream>>>(
      seed.feat, cap, static_cast<const bf16*>(seed.wb), seed.wf, seed.dirs, ctx->d_err, d_count, seed.list);
  PG_LAUNCHED(ctx);
  return PARRYGPU_OK;
}

// Descriptors of the scene's shapes and a snapshot of the network's weights, once per
// parrygpu_scene_set_mlp; also raises the inference kernel's shared-memory limit (outside any
// graph capture).
parrygpu_status pg::seed_prepare(parrygpu_ctx* ctx, const parrygpu_mlp* mlp, const ShapeArrays& sh, DevBuf& desc, DevBuf& wb, DevBuf& wf) {
  PG_CUDA(ctx, cudaFuncSetAttribute(k_mlp_infer_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TC_SMEM));
  PG_CUDA(ctx, desc.reserve(sh.n_shapes * 16 * 4));
  PG_CUDA(ctx, wb.reserve(N_PARAMS * 2));
  PG_CUDA(ctx, wf.reserve(N_PARAMS * 4));
  k_shape_desc<<<div_up(sh.n_shapes * 32, 256), 256, 0, ctx->stream>>>(sh.types, sh.params, sh.pool, sh.n_shapes, sh.n_vertices, desc.as<float>());
  PG_LAUNCHED(ctx);
  PG_CUDA(ctx, cudaMemcpyAsync(wb.ptr, mlp->wb.ptr, N_PARAMS * 2, cudaMemcpyDeviceToDevice, ctx->stream));
  PG_CUDA(ctx, cudaMemcpyAsync(wf.ptr, mlp->w.ptr, N_PARAMS * 4, cudaMemcpyDeviceToDevice, ctx->stream));
  return PARRYGPU_OK;
}

extern "C" {

uint64_t parrygpu_mlp_param_count(void) { return N_PARAMS; }

parrygpu_status parrygpu_mlp_create(parrygpu_ctx* ctx, uint64_t seed, parrygpu_mlp** out) {
  if (!ctx || !out) return PARRYGPU_INVALID_ARG;
  PG_CUDA(ctx, cudaSetDevice(ctx->device));
  parrygpu_mlp* m = new parrygpu_mlp();
  std::vector<float> host(N_PARAMS, 0.0f);
  uint64_t s = seed;
  for (int l = 0; l < NL; ++l) {
    float a = std::sqrt(6.0f / (float)(DIN[l] + DOUT[l]));
    for (uint64_t i = 0; i < (uint64_t)DOUT[l] * DIN[l]; ++i) {
      double u = (double)(splitmix(s) >> 11) * (1.0 / 9007199254740992.0);
      host[w_off(l) + i] = (float)((2.0 * u - 1.0) * a);
    }
  }
  cudaError_t e = m->w.reserve(N_PARAMS * 4);
  if (e == cudaSuccess) e = m->g.reserve(N_PARAMS * 4);
  if (e == cudaSuccess) e = m->m.reserve(N_PARAMS * 4);
  if (e == cudaSuccess) e = m->v.reserve(N_PARAMS * 4);
  if (e == cudaSuccess) e = m->wb.reserve(N_PARAMS * 2);
  if (e == cudaSuccess) e = cudaMemcpyAsync(m->w.ptr, host.data(), N_PARAMS * 4, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(m->m.ptr, 0, N_PARAMS * 4, ctx->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(m->v.ptr, 0, N_PARAMS * 4, ctx->stream);
  if (e != cudaSuccess) { parrygpu_mlp_destroy(m); return check_cuda(ctx, e, "mlp create"); }
  parrygpu_status st = refresh_bf16(ctx, m);
  if (st == PARRYGPU_OK) st = check_cuda(ctx, cudaStreamSynchronize(ctx->stream), "mlp create");
  if (st != PARRYGPU_OK) { parrygpu_mlp_destroy(m); return st; }
  *out = m;
  return PARRYGPU_OK;
}

void parrygpu_mlp_destroy(parrygpu_mlp* m) {
  if (!m) return;
  for (DevBuf* d : {&m->w, &m->g, &m->m, &m->v, &m->wb, &m->gpart, &m->x, &m->dy, &m->df, &m->dz, &m->dzf, &m->dxa, &m->loss}) d->release();
  for (int l = 0; l < NL; ++l) m->z[l].release();
  for (int l = 0; l < NL - 1; ++l) m->a[l].release();
  delete m;
}

parrygpu_status parrygpu_mlp_features(parrygpu_ctx* ctx, const parrygpu_shapes* shapes, const uint32_t* pairs, uint64_t n_pairs, float* features) {
  if (!ctx || !shapes) return PARRYGPU_INVALID_ARG;
  if (n_pairs == 0) return PARRYGPU_OK;
  if (!pairs || !features) return set_error(ctx, PARRYGPU_INVALID_ARG, "pairs and features are required");
  PG_CUDA(ctx, cudaSetDevice(ctx->device));
  const void *t, *p, *q, *v, *dp;
  parrygpu_status s;
  if ((s = stage_input(ctx, ctx->stage_in[0], shapes->types, shapes->n * 4, &t)) != PARRYGPU_OK) return s;
  if ((s = stage_input(ctx, ctx->stage_in[1], shapes->params, shapes->n * 16, &p)) != PARRYGPU_OK) return s;
  if ((s = stage_input(ctx, ctx->stage_in[2], shapes->poses, shapes->n * 28, &q)) != PARRYGPU_OK) return s;
  if ((s = stage_input(ctx, ctx->stage_in[3], shapes->vertices, shapes->n_vertices * 12, &v)) != PARRYGPU_OK) return s;
  if ((s = stage_input(ctx, ctx->stage_in[4], pairs, n_pairs * 8, &dp)) != PARRYGPU_OK) return s;
  void* d_f;
  bool copy;
  if ((s = stage_output(ctx, ctx->stage_out[0], features, n_pairs * IN * 4, &d_f, &copy)) != PARRYGPU_OK) return s;
  if (((uintptr_t)d_f & 15) != 0) return set_error(ctx, PARRYGPU_INVALID_ARG, "parrygpu_mlp_features needs a 16-byte aligned output");
  DevBuf& desc = ctx->stage_out[3];
  PG_CUDA(ctx, desc.reserve(shapes->n * 16 * 4));
  k_shape_desc<<<div_up(shapes->n * 32, 256), 256, 0, ctx->stream>>>((const uint32_t*)t, (const float4*)p, (const float*)v, shapes->n, shapes->n_vertices,
                                                                 desc.as<float>());
  PG_LAUNCHED(ctx);
  k_pair_features<<<div_up(n_pairs, PF_THREADS), PF_THREADS, 0, ctx->stream>>>((const float*)q, desc.as<float>(), (const uint32_t*)dp, n_pairs,
                                                                               shapes->n, (float*)d_f, nullptr, nullptr);
  PG_LAUNCHED(ctx);
  if (copy) PG_CUDA(ctx, cudaMemcpyAsync(features, d_f, n_pairs * IN * 4, cudaMemcpyDeviceToHost, ctx->stream));
  // host inputs or outputs: wait for their copies; all on the device: return at once, as the other calls do
  const bool staged = t != shapes->types || p != shapes->params || q != shapes->poses || dp != pairs ||
                      (shapes->n_vertices && v != shapes->vertices);
  if (copy || staged) return parrygpu_sync(ctx);
  return PARRYGPU_OK;
}

parrygpu_status parrygpu_mlp_train(parrygpu_ctx* ctx, parrygpu_mlp* mlp, const float* features, const float* targets, uint64_t n, uint32_t epochs,
                                   uint32_t batch, float lr, float* loss_per_epoch) {
  if (!ctx || !mlp || !features || !targets || n == 0 || batch == 0) return PARRYGPU_INVALID_ARG;
  PG_CUDA(ctx, cudaSetDevice(ctx->device));
  if (!is_device_ptr(features) || !is_device_ptr(targets))
    return set_error(ctx, PARRYGPU_INVALID_ARG, "parrygpu_mlp_train needs device-resident features and targets");
  parrygpu_status s = ensure_cap(ctx, mlp, batch);
  if (s != PARRYGPU_OK) return s;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  KernelTimer kt(ctx, "mlp_train");
  for (uint32_t ep = 0; ep < epochs; ++ep) {
    PG_CUDA(ctx, cudaMemsetAsync(mlp->loss.ptr, 0, 4, ctx->stream));
    for (uint64_t b0 = 0; b0 < n; b0 += batch) {
      uint64_t nb = n - b0 < batch ? n - b0 : batch;
      if ((s = load_features(ctx, mlp, features + b0 * IN, nb)) != PARRYGPU_OK) return s;
      if ((s = forward(ctx, mlp, nb)) != PARRYGPU_OK) return s;
      if ((s = backward(ctx, mlp, targets + b0 * 3, nb, nb)) != PARRYGPU_OK) return s;
      mlp->step += 1;
      float c1 = 1.0f - std::pow(b1, (float)mlp->step), c2 = 1.0f - std::pow(b2, (float)mlp->step);
      k_adam<<<div_up(N_PARAMS, 256), 256, 0, ctx->stream>>>(mlp->w.as<float>(), mlp->g.as<float>(), mlp->m.as<float>(), mlp->v.as<float>(),
                                                            N_PARAMS, lr, b1, b2, eps, c1, c2);
      PG_LAUNCHED(ctx);
      if ((s = refresh_bf16(ctx, mlp)) != PARRYGPU_OK) return s;
    }
    if (loss_per_epoch) {
      float l;
      PG_CUDA(ctx, cudaMemcpyAsync(&l, mlp->loss.ptr, 4, cudaMemcpyDeviceToHost, ctx->stream));
      PG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
      loss_per_epoch[ep] = l / (float)n;
    }
  }
  kt.stop();
  return parrygpu_sync(ctx);
}

parrygpu_status parrygpu_mlp_predict(parrygpu_ctx* ctx, const parrygpu_mlp* cmlp, const float* features, uint64_t n, float* dirs) {
  if (!ctx || !cmlp || !features || !dirs) return PARRYGPU_INVALID_ARG;
  if (n == 0) return PARRYGPU_OK;
  parrygpu_mlp* mlp = const_cast<parrygpu_mlp*>(cmlp);
  PG_CUDA(ctx, cudaSetDevice(ctx->device));
  const uint64_t chunk = 1 << 18;
  parrygpu_status s = ensure_cap(ctx, mlp, n < chunk ? n : chunk);
  if (s != PARRYGPU_OK) return s;
  const void* d_f;
  if ((s = stage_input(ctx, ctx->stage_in[7], features, n * IN * 4, &d_f)) != PARRYGPU_OK) return s;
  void* d_dirs;
  bool copy;
  if ((s = stage_output(ctx, ctx->stage_out[2], dirs, n * 12, &d_dirs, &copy)) != PARRYGPU_OK) return s;
  KernelTimer kt(ctx, "mlp_predict");
  if (ctx->cfg.mlp_infer != 2) {  // the fused tcgen05 kernel
    if ((reinterpret_cast<uintptr_t>(d_f) & 15u) != 0)
      return set_error(ctx, PARRYGPU_INVALID_ARG, "parrygpu_mlp_predict needs 16-byte aligned features");
    PG_CUDA(ctx, cudaFuncSetAttribute(k_mlp_infer_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TC_SMEM));
    const uint64_t tiles = (n + TC_M - 1) / TC_M;
    const uint32_t sms = ctx->sm_count > 0 ? (uint32_t)ctx->sm_count : 152u;
    const uint32_t grid = (uint32_t)(tiles < sms ? tiles : sms);
    k_mlp_infer_tc<<<grid, TC_THREADS, TC_SMEM, ctx->stream>>>((const float*)d_f, n, mlp->wb.as<bf16>(), mlp->w.as<float>(),
                                                             (float*)d_dirs, ctx->d_err, nullptr, nullptr);
    PG_LAUNCHED(ctx);
  } else {  // per-layer mma.sync GEMMs (the training path's forward)
    for (uint64_t b0 = 0; b0 < n; b0 += chunk) {
      uint64_t nb = n - b0 < chunk ? n - b0 : chunk;
      if ((s = load_features(ctx, mlp, (const float*)d_f + b0 * IN, nb)) != PARRYGPU_OK) return s;
      if ((s = forward(ctx, mlp, nb)) != PARRYGPU_OK) return s;
      k_normalize_dirs<<<div_up(nb, 256), 256, 0, ctx->stream>>>(mlp->z[NL - 1].as<float>(), (const float*)d_f + b0 * IN, nb,
                                                                (float*)d_dirs + b0 * 3);
      PG_LAUNCHED(ctx);
    }
  }
  kt.stop();
  if (copy) PG_CUDA(ctx, cudaMemcpyAsync(dirs, d_dirs, n * 12, cudaMemcpyDeviceToHost, ctx->stream));
  if (copy || d_f != features) return parrygpu_sync(ctx);
  return PARRYGPU_OK;
}

parrygpu_status parrygpu_mlp_loss_and_grads(parrygpu_ctx* ctx, const parrygpu_mlp* cmlp, const float* features, const float* targets, uint64_t n,
                                            float* loss, float* grads) {
  if (!ctx || !cmlp || !features || !targets || n == 0) return PARRYGPU_INVALID_ARG;
  parrygpu_mlp* mlp = const_cast<parrygpu_mlp*>(cmlp);
  PG_CUDA(ctx, cudaSetDevice(ctx->device));
  parrygpu_status s = ensure_cap(ctx, mlp, n);
  if (s != PARRYGPU_OK) return s;
  const void *d_f, *d_t;
  if ((s = stage_input(ctx, ctx->stage_in[6], features, n * IN * 4, &d_f)) != PARRYGPU_OK) return s;
  if ((s = stage_input(ctx, ctx->stage_in[7], targets, n * 12, &d_t)) != PARRYGPU_OK) return s;
  PG_CUDA(ctx, cudaMemsetAsync(mlp->loss.ptr, 0, 4, ctx->stream));
  if ((s = load_features(ctx, mlp, (const float*)d_f, n)) != PARRYGPU_OK) return s;
  if ((s = forward(ctx, mlp, n)) != PARRYGPU_OK) return s;
  if ((s = backward(ctx, mlp, (const float*)d_t, n, n)) != PARRYGPU_OK) return s;
  float l = 0.0f;
  PG_CUDA(ctx, cudaMemcpyAsync(&l, mlp->loss.ptr, 4, cudaMemcpyDeviceToHost, ctx->stream));
  if (grads) PG_CUDA(ctx, cudaMemcpyAsync(grads, mlp->g.ptr, N_PARAMS * 4, cudaMemcpyDefault, ctx->stream));
  PG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (loss) *loss = l / (float)n;
  return parrygpu_sync(ctx);
}

parrygpu_status parrygpu_mlp_get_params(parrygpu_ctx* ctx, const parrygpu_mlp* mlp, float* params) {
  if (!ctx || !mlp || !params) return PARRYGPU_INVALID_ARG;
  PG_CUDA(ctx, cudaSetDevice(ctx->device));
  PG_CUDA(ctx, cudaMemcpyAsync(params, mlp->w.ptr, N_PARAMS * 4, cudaMemcpyDefault, ctx->stream));
  PG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return PARRYGPU_OK;
}

parrygpu_status parrygpu_mlp_set_params(parrygpu_ctx* ctx, parrygpu_mlp* mlp, const float* params) {
  if (!ctx || !mlp || !params) return PARRYGPU_INVALID_ARG;
  PG_CUDA(ctx, cudaSetDevice(ctx->device));
  PG_CUDA(ctx, cudaMemcpyAsync(mlp->w.ptr, params, N_PARAMS * 4, cudaMemcpyDefault, ctx->stream));
  parrygpu_status s = refresh_bf16(ctx, mlp);
  if (s != PARRYGPU_OK) return s;
  PG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return PARRYGPU_OK;
}

}  // extern "C"
