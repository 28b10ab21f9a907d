// The dryLeaf surrogate network: 12 inputs -> 64 (SiLU) -> 64 (SiLU) -> 3,
// BF16 weights and activations, FP32 accumulation in tensor memory.
//
// Parameter vector (FP32 master copy, this order): W1 [64][12], b1 [64],
// W2 [64][64], b2 [64], W3 [3][64], b3 [3].  Normalisation vector: input
// mean [12], input 1/sd [12], output mean [3], output sd [3]; the network
// maps normalised inputs to normalised outputs.
//
// Packed image: the weights as BF16 tensor-core operands (K-major, no
// swizzle, tc05.cuh), built from the master copy after every update.
#pragma once
#include <cstdint>

#include "tc05.cuh"

namespace cg {
namespace sur {

constexpr int NIN = 12, NH = 64, NOUT = 3;
constexpr int KIN = 16;     // input width padded to one MMA K-step
constexpr int NOUTP = 16;   // output width padded to the smallest MMA N
constexpr int OFF_W1 = 0, OFF_B1 = 768, OFF_W2 = 832, OFF_B2 = 4928, OFF_W3 = 4992, OFF_B3 = 5184;
constexpr int NPARAM = 5187;
constexpr int NNORM = 30;   // mu_x[12], isd_x[12], mu_y[3], sd_y[3]

// packed image, byte offsets
constexpr int PK_W1 = 0;        // W1  as B operand: [64 out][16 in]
constexpr int PK_W2 = 2048;     // W2  as B operand: [64 out][64 in]
constexpr int PK_W3 = 10240;    // W3  as B operand: [16 out (3 used)][64 in]
constexpr int PK_W3T = 12288;   // W3^T as B operand of dA2 = dZ3 W3: [64 in][16 out]
constexpr int PK_W2T = 14336;   // W2^T as B operand of dA1 = dZ2 W2: [64 in][64 out]
constexpr int PK_BYTES = 22528;
constexpr int PK_FWD_BYTES = 12288;   // W1, W2, W3: all inference needs

// Rows of a training set: 12 raw features, 3 raw targets, 1 unused.
constexpr int ROW = 16;

// logistic sigmoid from the hardware tanh approximation (one MUFU op;
// relative error ~2^-11, below the BF16 rounding of the activations):
// sigmoid(z) = (1 + tanh(z / 2)) / 2
__device__ __forceinline__ float sigmoid_fast(float z) {
  float t;
  asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(0.5f * z));
  return fmaf(0.5f, t, 0.5f);
}
__device__ __forceinline__ float silu(float z) { return z * sigmoid_fast(z); }
__device__ __forceinline__ float dsilu(float z) {
  const float s = sigmoid_fast(z);
  return s * fmaf(z, 1.0f - s, 1.0f);
}

// Shared-memory layout of the in-loop / batch forward pass (bytes).
constexpr int FW_W = 0;                    // packed W1, W2, W3 (12288)
constexpr int FW_A0 = 12288;               // inputs  [128][16]  (4096)
constexpr int FW_A1 = 16384;               // hidden1 [128][64]  (16384)
constexpr int FW_A2 = FW_A1;               // hidden2 overwrites hidden1 once layer 2 has consumed it
constexpr int FW_BIAS = 32768;             // b1[64], b2[64], b3[4] FP32 (528)
constexpr int FW_NORM = FW_BIAS + 528;     // 30 floats (120), padded to 128
constexpr int FW_BAR = FW_NORM + 128;      // mbarrier (8) + tmem address (4) + flag (4)
constexpr int FW_STATS = FW_BAR + 16;      // block counters of the in-loop surrogate (tried, accepted)
constexpr int FW_SMEM = FW_STATS + 16;
constexpr uint32_t FW_TMEM_COLS = 64;      // D1, D2, D3 in turn at column 0

// One forward pass of the network for the 128 rows held by the 128 threads
// of the calling CTA (thread i = row i = tensor-memory lane i).  xn: this
// thread's 12 normalised inputs; y: its 3 normalised outputs.  Every thread
// of the CTA must call it (it synchronises the CTA).  Returns false if a
// tensor-core completion did not arrive within wait_ns, in which case the
// outputs are unusable: the caller must not call it again in this kernel,
// and must call settle() before freeing the tensor memory.
__device__ __forceinline__ bool forward128(uint8_t* smem, uint32_t taddr, uint32_t& phase, const float* xn, float* y,
                                           uint64_t wait_ns = tc::kWaitNs) {
  using namespace tc;
  const int s = threadIdx.x;
  const uint32_t lane = taddr + ((uint32_t)(s & ~31) << 16);
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + FW_BAR);
  const float* b1 = reinterpret_cast<const float*>(smem + FW_BIAS);
  const float* b2 = b1 + 64;
  const float* b3 = b1 + 128;
  const uint32_t sbase = smem_u32(smem);
  // inputs -> A0 row s
  {
    uint4 lo, hi;
    lo.x = pack_bf16x2(xn[0], xn[1]); lo.y = pack_bf16x2(xn[2], xn[3]);
    lo.z = pack_bf16x2(xn[4], xn[5]); lo.w = pack_bf16x2(xn[6], xn[7]);
    hi.x = pack_bf16x2(xn[8], xn[9]); hi.y = pack_bf16x2(xn[10], xn[11]);
    hi.z = 0u; hi.w = 0u;
    *reinterpret_cast<uint4*>(smem + FW_A0 + kmajor_offset(s, 0, KIN)) = lo;
    *reinterpret_cast<uint4*>(smem + FW_A0 + kmajor_offset(s, 8, KIN)) = hi;
  }
  bool ok = true;
  // layer 1: D1[128x64] = A0 W1^T
  fence_proxy_async();
  fence_before_sync();
  __syncthreads();
  if (s == 0) {
    fence_after_sync();
    mma_bf16(taddr + 0, kslice_desc(sbase + FW_A0, 0, KIN), kslice_desc(sbase + FW_W + PK_W1, 0, KIN),
             idesc_bf16(128, 64), 0);
    mma_commit(bar);
  }
  ok = mbar_wait(bar, phase, wait_ns);
  phase ^= 1u;
  if (__syncthreads_or(!ok)) return false;
  fence_after_sync();
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    float v[16];
    tmem_ld16(lane + 0 + c * 16, v);
    uint32_t w[8];
#pragma unroll
    for (int j = 0; j < 8; ++j)
      w[j] = pack_bf16x2(silu(v[2 * j] + b1[c * 16 + 2 * j]), silu(v[2 * j + 1] + b1[c * 16 + 2 * j + 1]));
    *reinterpret_cast<uint4*>(smem + FW_A1 + kmajor_offset(s, c * 16, NH)) = make_uint4(w[0], w[1], w[2], w[3]);
    *reinterpret_cast<uint4*>(smem + FW_A1 + kmajor_offset(s, c * 16 + 8, NH)) = make_uint4(w[4], w[5], w[6], w[7]);
  }
  // layer 2: D2[128x64] = A1 W2^T
  fence_proxy_async();
  fence_before_sync();
  __syncthreads();
  if (s == 0) {
    fence_after_sync();
#pragma unroll
    for (int j = 0; j < 4; ++j)
      mma_bf16(taddr + 0, kslice_desc(sbase + FW_A1, 16 * j, NH), kslice_desc(sbase + FW_W + PK_W2, 16 * j, NH),
               idesc_bf16(128, 64), j > 0);
    mma_commit(bar);
  }
  ok = mbar_wait(bar, phase, wait_ns);
  phase ^= 1u;
  if (__syncthreads_or(!ok)) return false;
  fence_after_sync();
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    float v[16];
    tmem_ld16(lane + 0 + c * 16, v);
    uint32_t w[8];
#pragma unroll
    for (int j = 0; j < 8; ++j)
      w[j] = pack_bf16x2(silu(v[2 * j] + b2[c * 16 + 2 * j]), silu(v[2 * j + 1] + b2[c * 16 + 2 * j + 1]));
    *reinterpret_cast<uint4*>(smem + FW_A2 + kmajor_offset(s, c * 16, NH)) = make_uint4(w[0], w[1], w[2], w[3]);
    *reinterpret_cast<uint4*>(smem + FW_A2 + kmajor_offset(s, c * 16 + 8, NH)) = make_uint4(w[4], w[5], w[6], w[7]);
  }
  // layer 3: D3[128x16] = A2 W3^T
  fence_proxy_async();
  fence_before_sync();
  __syncthreads();
  if (s == 0) {
    fence_after_sync();
#pragma unroll
    for (int j = 0; j < 4; ++j)
      mma_bf16(taddr + 0, kslice_desc(sbase + FW_A2, 16 * j, NH), kslice_desc(sbase + FW_W + PK_W3, 16 * j, NH),
               idesc_bf16(128, NOUTP), j > 0);
    mma_commit(bar);
  }
  ok = mbar_wait(bar, phase, wait_ns);
  phase ^= 1u;
  if (__syncthreads_or(!ok)) return false;
  fence_after_sync();
  {
    float v[16];
    tmem_ld16(lane + 0, v);
    y[0] = v[0] + b3[0];
    y[1] = v[1] + b3[1];
    y[2] = v[2] + b3[2];
  }
  // the next call overwrites A0 and tensor-memory columns read above
  fence_before_sync();
  __syncthreads();
  return true;
}

// After a failed wait: waits once more for the tensor-core pass that did not
// report, so the tensor memory it writes can be freed.  Always with the
// default limit (never the caller's debug limit): the pass was issued and
// completes in microseconds, and the memory must not be freed under it.
__device__ __forceinline__ void settle(uint8_t* smem, uint32_t phase) {
  tc::mbar_wait(reinterpret_cast<uint64_t*>(smem + FW_BAR), phase ^ 1u, tc::kWaitNs);
}

// Wait limit (ns) the host passes to the network kernels: the default, or
// the value of the environment variable CABLEGPU_DEBUG_TC_WAIT_NS read at
// each launch (0 makes every first wait give up, to test the fallback).
unsigned long long wait_limit_ns();

}  // namespace sur
}  // namespace cg
