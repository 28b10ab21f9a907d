// Training and batch inference of the dryLeaf surrogate network on the
// tensor cores (tcgen05, BF16 operands, FP32 accumulation in tensor memory),
// plus the host-side trainer (Adam) and the C ABI entry points of
// include/cablegpu.h that drive them.
//
// Training step on a batch: mlp_train_kernel (persistent, one CTA per SM,
// 128 samples per tile) runs forward, loss gradient and backward for each
// tile and accumulates the weight and bias gradients of all its tiles in
// tensor memory; mlp_update_kernel sums the per-CTA partial gradients in a
// fixed order (bitwise reproducible) and applies Adam to the FP32 master
// weights; mlp_pack_kernel rebuilds the BF16 operand image.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/cablegpu.h"
#include "cbm_physics.cuh"
#include "surrogate.cuh"
#include "surrogate_host.h"

using namespace cg;
using namespace cg::sur;

namespace {

// ------------------------------------------------------------------ training kernel smem (bytes)
constexpr int TR_W = 0;          // packed image (22528)
constexpr int TR_A0 = 22528;     // X      [128 s][16]      K-major
constexpr int TR_A1 = 26624;     // A1     [128 s][64]
constexpr int TR_A2 = 43008;     // A2     [128 s][64]
constexpr int TR_BT = 59392;     // [A1^T (64 rows); X^T (16 rows, row 12 = 1)] [80][128 s]
constexpr int TR_A2T = 79872;    // [A2^T (64 rows); 1 (row 64); 0 ...]        [80][128 s]
constexpr int TR_DZ3 = 100352;   // dZ3    [128 s][16]
constexpr int TR_DZ2 = 104448;   // dZ2    [128 s][64]
constexpr int TR_DZ3T = 120832;  // dZ3^T  [16][128 s]   (rows 0-2 used); must directly precede TR_DZCT
constexpr int TR_DZCT = 124928;  // [dZ2^T; dZ1^T] [128][128 s]
constexpr int TR_BIAS = 157696;  // b1[64], b2[64], b3[4]
constexpr int TR_NORM = TR_BIAS + 528;
constexpr int TR_RED = TR_NORM + 128;   // 4 warp partial losses
constexpr int TR_BAR = TR_RED + 16;
constexpr int TR_SMEM = TR_BAR + 16;
constexpr uint32_t TR_TMEM_COLS = 512;
// tensor-memory columns
constexpr uint32_t TC_D1 = 0, TC_D2 = 64, TC_D3 = 128, TC_DA2 = 192, TC_DA1 = 256, TC_W12 = 320, TC_W3 = 416;

static_assert(TR_DZ3T + 16 * 128 * 2 == TR_DZCT, "dZ3^T must be followed by the 112 rows the dW3 MMA reads past it");
static_assert(TR_SMEM <= 227 * 1024, "training kernel shared memory");

struct TrainArgs {
  const float* rows;          // [ntrain][ROW]
  long long ntrain;           // rows the permutation ranges over
  long long pos0;             // first permuted position of the batch
  int n;                      // batch size
  unsigned long long pa, pc;  // row = (pa * pos + pc) % ntrain
  const uint8_t* packed;
  const float* params;
  const float* norm;
  float* part;                // [gridDim.x][NPARAM]
  float* loss_part;           // [gridDim.x]
  float grad_scale;           // 2 / (n * NOUT)
  unsigned int* err;
};

__device__ __forceinline__ void st_bf16(uint8_t* p, float v) {
  *reinterpret_cast<__nv_bfloat16*>(p) = __float2bfloat16_rn(v);
}

__global__ void __launch_bounds__(128, 1) mlp_train_kernel(TrainArgs a) {
  using namespace tc;
  extern __shared__ __align__(1024) uint8_t smem[];
  const int s = threadIdx.x;
  const uint32_t sb = smem_u32(smem);
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + TR_BAR);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(smem + TR_BAR + 8);
  float* b1 = reinterpret_cast<float*>(smem + TR_BIAS);
  float* b2 = b1 + 64;
  float* b3 = b1 + 128;
  float* nrm = reinterpret_cast<float*>(smem + TR_NORM);
  float* red = reinterpret_cast<float*>(smem + TR_RED);

  // weights, biases, normalisation
  for (int i = s; i < PK_BYTES / 16; i += 128)
    reinterpret_cast<uint4*>(smem + TR_W)[i] = reinterpret_cast<const uint4*>(a.packed)[i];
  if (s < 64) { b1[s] = a.params[OFF_B1 + s]; b2[s] = a.params[OFF_B2 + s]; }
  if (s < 3) b3[s] = a.params[OFF_B3 + s];
  if (s < NNORM) nrm[s] = a.norm[s];
  // constant rows: X^T rows 12..15 (row 12 = 1 gives the bias gradients of
  // layers 1 and 2), ones row of the dW3 operand, zero rows of dZ3^T
  for (int k = 12; k < 16; ++k) st_bf16(smem + TR_BT + kmajor_offset(64 + k, s, 128), k == 12 ? 1.f : 0.f);
  for (int r = 64; r < 80; ++r) st_bf16(smem + TR_A2T + kmajor_offset(r, s, 128), r == 64 ? 1.f : 0.f);
  for (int r = 3; r < 16; ++r) st_bf16(smem + TR_DZ3T + kmajor_offset(r, s, 128), 0.f);
  if (s == 0) {
    mbar_init(bar, 1);
    fence_mbar_init();
  }
  if (s < 32) {
    tmem_alloc(tslot, TR_TMEM_COLS);
    tmem_relinquish();
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t taddr = *tslot;
  const uint32_t lane = taddr + ((uint32_t)(s & ~31) << 16);
  uint32_t phase = 0;
  bool ok = true;
  float loss = 0.f;
  const int ntiles = (a.n + 127) / 128;
  int done_tiles = 0;

  auto issue_and_wait = [&](auto&& issue) -> bool {
    fence_proxy_async();
    fence_before_sync();
    __syncthreads();
    if (s == 0) {
      fence_after_sync();
      issue();
      mma_commit(bar);
    }
    bool w = mbar_wait(bar, phase);
    phase ^= 1u;
    if (__syncthreads_or(!w)) return false;
    fence_after_sync();
    return true;
  };

  for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
    const int j = tile * 128 + s;
    const bool valid = j < a.n;
    float xn[NIN], tn[NOUT];
    if (valid) {
      const unsigned long long pos = (unsigned long long)(a.pos0 + j);
      const long long row = (long long)((a.pa * pos + a.pc) % (unsigned long long)a.ntrain);
      const float4* r = reinterpret_cast<const float4*>(a.rows + row * ROW);
      const float4 q0 = r[0], q1 = r[1], q2 = r[2], q3 = r[3];
      const float raw[16] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w,
                             q2.x, q2.y, q2.z, q2.w, q3.x, q3.y, q3.z, q3.w};
#pragma unroll
      for (int f = 0; f < NIN; ++f) xn[f] = (raw[f] - nrm[f]) * nrm[12 + f];
#pragma unroll
      for (int o = 0; o < NOUT; ++o) tn[o] = (raw[12 + o] - nrm[24 + o]) / nrm[27 + o];
    } else {
#pragma unroll
      for (int f = 0; f < NIN; ++f) xn[f] = 0.f;
#pragma unroll
      for (int o = 0; o < NOUT; ++o) tn[o] = 0.f;
    }
    // X row s and X^T column s
    {
      uint4 lo, hi;
      lo.x = pack_bf16x2(xn[0], xn[1]); lo.y = pack_bf16x2(xn[2], xn[3]);
      lo.z = pack_bf16x2(xn[4], xn[5]); lo.w = pack_bf16x2(xn[6], xn[7]);
      hi.x = pack_bf16x2(xn[8], xn[9]); hi.y = pack_bf16x2(xn[10], xn[11]);
      hi.z = 0u; hi.w = 0u;
      *reinterpret_cast<uint4*>(smem + TR_A0 + kmajor_offset(s, 0, KIN)) = lo;
      *reinterpret_cast<uint4*>(smem + TR_A0 + kmajor_offset(s, 8, KIN)) = hi;
#pragma unroll
      for (int f = 0; f < NIN; ++f) st_bf16(smem + TR_BT + kmajor_offset(64 + f, s, 128), xn[f]);
    }
    // layer 1
    ok = issue_and_wait([&] {
      mma_bf16(taddr + TC_D1, kslice_desc(sb + TR_A0, 0, KIN), kslice_desc(sb + TR_W + PK_W1, 0, KIN),
               idesc_bf16(128, 64), 0);
    });
    if (!ok) break;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      float v[16];
      tmem_ld16(lane + TC_D1 + c * 16, v);
      uint32_t w[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const float h0 = silu(v[2 * q] + b1[c * 16 + 2 * q]), h1 = silu(v[2 * q + 1] + b1[c * 16 + 2 * q + 1]);
        w[q] = pack_bf16x2(h0, h1);
        st_bf16(smem + TR_BT + kmajor_offset(c * 16 + 2 * q, s, 128), h0);
        st_bf16(smem + TR_BT + kmajor_offset(c * 16 + 2 * q + 1, s, 128), h1);
      }
      *reinterpret_cast<uint4*>(smem + TR_A1 + kmajor_offset(s, c * 16, NH)) = make_uint4(w[0], w[1], w[2], w[3]);
      *reinterpret_cast<uint4*>(smem + TR_A1 + kmajor_offset(s, c * 16 + 8, NH)) = make_uint4(w[4], w[5], w[6], w[7]);
    }
    // layer 2
    ok = issue_and_wait([&] {
#pragma unroll
      for (int q = 0; q < 4; ++q)
        mma_bf16(taddr + TC_D2, kslice_desc(sb + TR_A1, 16 * q, NH), kslice_desc(sb + TR_W + PK_W2, 16 * q, NH),
                 idesc_bf16(128, 64), q > 0);
    });
    if (!ok) break;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      float v[16];
      tmem_ld16(lane + TC_D2 + c * 16, v);
      uint32_t w[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const float h0 = silu(v[2 * q] + b2[c * 16 + 2 * q]), h1 = silu(v[2 * q + 1] + b2[c * 16 + 2 * q + 1]);
        w[q] = pack_bf16x2(h0, h1);
        st_bf16(smem + TR_A2T + kmajor_offset(c * 16 + 2 * q, s, 128), h0);
        st_bf16(smem + TR_A2T + kmajor_offset(c * 16 + 2 * q + 1, s, 128), h1);
      }
      *reinterpret_cast<uint4*>(smem + TR_A2 + kmajor_offset(s, c * 16, NH)) = make_uint4(w[0], w[1], w[2], w[3]);
      *reinterpret_cast<uint4*>(smem + TR_A2 + kmajor_offset(s, c * 16 + 8, NH)) = make_uint4(w[4], w[5], w[6], w[7]);
    }
    // layer 3
    ok = issue_and_wait([&] {
#pragma unroll
      for (int q = 0; q < 4; ++q)
        mma_bf16(taddr + TC_D3, kslice_desc(sb + TR_A2, 16 * q, NH), kslice_desc(sb + TR_W + PK_W3, 16 * q, NH),
                 idesc_bf16(128, NOUTP), q > 0);
    });
    if (!ok) break;
    // loss gradient dZ3 = grad_scale * (y - t): row s of dZ3, column s of dZ3^T
    {
      float v[16];
      tmem_ld16(lane + TC_D3, v);
      float dy[NOUT];
#pragma unroll
      for (int o = 0; o < NOUT; ++o) {
        const float d = v[o] + b3[o] - tn[o];
        loss += valid ? d * d : 0.f;
        dy[o] = valid ? a.grad_scale * d : 0.f;
      }
      *reinterpret_cast<uint4*>(smem + TR_DZ3 + kmajor_offset(s, 0, KIN)) =
          make_uint4(pack_bf16x2(dy[0], dy[1]), pack_bf16x2(dy[2], 0.f), 0u, 0u);
      *reinterpret_cast<uint4*>(smem + TR_DZ3 + kmajor_offset(s, 8, KIN)) = make_uint4(0u, 0u, 0u, 0u);
#pragma unroll
      for (int o = 0; o < NOUT; ++o) st_bf16(smem + TR_DZ3T + kmajor_offset(o, s, 128), dy[o]);
    }
    // dA2 = dZ3 W3 and dW3 (+ db3 via the ones row) += dZ3^T [A2 | 1]
    const uint32_t acc_w = done_tiles > 0 ? 1u : 0u;
    ok = issue_and_wait([&] {
      mma_bf16(taddr + TC_DA2, kslice_desc(sb + TR_DZ3, 0, KIN), kslice_desc(sb + TR_W + PK_W3T, 0, KIN),
               idesc_bf16(128, 64), 0);
#pragma unroll
      for (int q = 0; q < 8; ++q)
        mma_bf16(taddr + TC_W3, kslice_desc(sb + TR_DZ3T, 16 * q, 128), kslice_desc(sb + TR_A2T, 16 * q, 128),
                 idesc_bf16(128, 80), (q > 0) | acc_w);
    });
    if (!ok) break;
    // dZ2 = dA2 * silu'(z2)
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      float da[16], z[16];
      tmem_ld16(lane + TC_DA2 + c * 16, da);
      tmem_ld16(lane + TC_D2 + c * 16, z);
      uint32_t w[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const float g0 = da[2 * q] * dsilu(z[2 * q] + b2[c * 16 + 2 * q]);
        const float g1 = da[2 * q + 1] * dsilu(z[2 * q + 1] + b2[c * 16 + 2 * q + 1]);
        w[q] = pack_bf16x2(g0, g1);
        st_bf16(smem + TR_DZCT + kmajor_offset(c * 16 + 2 * q, s, 128), g0);
        st_bf16(smem + TR_DZCT + kmajor_offset(c * 16 + 2 * q + 1, s, 128), g1);
      }
      *reinterpret_cast<uint4*>(smem + TR_DZ2 + kmajor_offset(s, c * 16, NH)) = make_uint4(w[0], w[1], w[2], w[3]);
      *reinterpret_cast<uint4*>(smem + TR_DZ2 + kmajor_offset(s, c * 16 + 8, NH)) = make_uint4(w[4], w[5], w[6], w[7]);
    }
    // dA1 = dZ2 W2
    ok = issue_and_wait([&] {
#pragma unroll
      for (int q = 0; q < 4; ++q)
        mma_bf16(taddr + TC_DA1, kslice_desc(sb + TR_DZ2, 16 * q, NH), kslice_desc(sb + TR_W + PK_W2T, 16 * q, NH),
                 idesc_bf16(128, 64), q > 0);
    });
    if (!ok) break;
    // dZ1 = dA1 * silu'(z1): rows 64..127 of [dZ2^T; dZ1^T]
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      float da[16], z[16];
      tmem_ld16(lane + TC_DA1 + c * 16, da);
      tmem_ld16(lane + TC_D1 + c * 16, z);
#pragma unroll
      for (int q = 0; q < 16; ++q)
        st_bf16(smem + TR_DZCT + kmajor_offset(64 + c * 16 + q, s, 128), da[q] * dsilu(z[q] + b1[c * 16 + q]));
    }
    // [dW2 | . ; . | dW1] (+ db2, db1 in column 76) += [dZ2^T; dZ1^T] [A1 | X | 1]
    ok = issue_and_wait([&] {
#pragma unroll
      for (int q = 0; q < 8; ++q)
        mma_bf16(taddr + TC_W12, kslice_desc(sb + TR_DZCT, 16 * q, 128), kslice_desc(sb + TR_BT, 16 * q, 128),
                 idesc_bf16(128, 80), (q > 0) | acc_w);
    });
    if (!ok) break;
    ++done_tiles;
  }

  // per-CTA partial gradients and loss
  if (ok) {
    float* P = a.part + (size_t)blockIdx.x * NPARAM;
    const bool have = done_tiles > 0;
#pragma unroll 1
    for (int c = 0; c < 5; ++c) {
      float v[16], u[16];
      tmem_ld16(lane + TC_W12 + c * 16, v);
      tmem_ld16(lane + TC_W3 + c * 16, u);
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        const int col = c * 16 + q;
        const float gv = have ? v[q] : 0.f, gu = have ? u[q] : 0.f;
        if (s < 64) {
          if (col < 64) P[OFF_W2 + s * 64 + col] = gv;
          if (col == 76) P[OFF_B2 + s] = gv;
        } else {
          if (col >= 64 && col < 76) P[OFF_W1 + (s - 64) * NIN + (col - 64)] = gv;
          if (col == 76) P[OFF_B1 + (s - 64)] = gv;
        }
        if (s < NOUT) {
          if (col < 64) P[OFF_W3 + s * 64 + col] = gu;
          if (col == 64) P[OFF_B3 + s] = gu;
        }
      }
    }
    float l = loss;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
    if ((s & 31) == 0) red[s >> 5] = l;
  }
  if (!ok) mbar_wait(bar, phase ^ 1u);   // the pass that did not report, bounded
  fence_before_sync();
  __syncthreads();
  if (!ok) {
    if (s == 0) atomicOr(a.err, 1u);
  } else if (s == 0) {
    a.loss_part[blockIdx.x] = red[0] + red[1] + red[2] + red[3];
  }
  if (s < 32) tmem_dealloc(taddr, TR_TMEM_COLS);
}

// ------------------------------------------------------------------ forward over a batch
struct FwdArgs {
  const float* rows;   // [n][ROW]
  long long n;
  const uint8_t* packed;
  const float* params;
  const float* norm;
  float* y;            // [n][NOUT] raw outputs, may be null
  float* loss_part;    // [gridDim.x] sum of squared normalised errors, may be null
  unsigned int* err;
  unsigned long long wait_ns;   // tensor-core wait limit (wait_limit_ns)
};

__global__ void __launch_bounds__(128, 1) mlp_forward_kernel(FwdArgs a) {
  using namespace tc;
  extern __shared__ __align__(1024) uint8_t smem[];
  const int s = threadIdx.x;
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + FW_BAR);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(smem + FW_BAR + 8);
  float* b = reinterpret_cast<float*>(smem + FW_BIAS);
  float* nrm = reinterpret_cast<float*>(smem + FW_NORM);
  for (int i = s; i < PK_FWD_BYTES / 16; i += 128)
    reinterpret_cast<uint4*>(smem + FW_W)[i] = reinterpret_cast<const uint4*>(a.packed)[i];
  if (s < 64) { b[s] = a.params[OFF_B1 + s]; b[64 + s] = a.params[OFF_B2 + s]; }
  if (s < 3) b[128 + s] = a.params[OFF_B3 + s];
  if (s < NNORM) nrm[s] = a.norm[s];
  if (s == 0) { mbar_init(bar, 1); fence_mbar_init(); }
  if (s < 32) { tmem_alloc(tslot, FW_TMEM_COLS); tmem_relinquish(); }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t taddr = *tslot;
  uint32_t phase = 0;
  bool ok = true;
  float loss = 0.f;
  const long long ntiles = (a.n + 127) / 128;
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const long long j = tile * 128 + s;
    const bool valid = j < a.n;
    float xn[NIN], raw[16];
    if (valid) {
      const float4* r = reinterpret_cast<const float4*>(a.rows + j * ROW);
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const float4 v = r[q];
        raw[4 * q] = v.x; raw[4 * q + 1] = v.y; raw[4 * q + 2] = v.z; raw[4 * q + 3] = v.w;
      }
    } else {
#pragma unroll
      for (int q = 0; q < 16; ++q) raw[q] = nrm[q < NIN ? q : 0];
    }
#pragma unroll
    for (int f = 0; f < NIN; ++f) xn[f] = valid ? (raw[f] - nrm[f]) * nrm[12 + f] : 0.f;
    float y[NOUT];
    ok = forward128(smem, taddr, phase, xn, y, a.wait_ns);
    if (!ok) break;
    if (valid) {
#pragma unroll
      for (int o = 0; o < NOUT; ++o) {
        const float tn = (raw[12 + o] - nrm[24 + o]) / nrm[27 + o];
        loss += (y[o] - tn) * (y[o] - tn);
        if (a.y) a.y[j * NOUT + o] = y[o] * nrm[27 + o] + nrm[24 + o];
      }
    }
  }
  if (!ok) {
    settle(smem, phase);
    if (s == 0) atomicOr(a.err, 1u);
  }
  if (a.loss_part) {
    float l = loss;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
    if ((s & 31) == 0) atomicAdd(&a.loss_part[blockIdx.x], l);
  }
  fence_before_sync();
  __syncthreads();
  if (s < 32) tmem_dealloc(taddr, FW_TMEM_COLS);
}

// ------------------------------------------------------------------ in-step inference
// Predicted leaf-temperature change of the first Monin-Obukhov iteration of
// every tile.  The inputs are formed here from the radiation kernel's
// hand-off record (work_a, one array per word so each load is coalesced) and
// the plant-type tables, exactly as the canopy kernel sees them when that
// iteration starts: leaf and canopy air at tk, the wind speed and air
// temperature of the forcing, fwsoil_calc_std (cbl_fwsoil.F90:13-38).
// Persistent: each CTA walks 128-tile chunks.
struct InferArgs {
  const float* work_a;   // [CG_NA][ld]
  const uint8_t* iveg;
  const uint8_t* isoilm;
  const CgTables* tables;
  int medlyn;
  int mp, ld;
  const uint8_t* packed;
  const float* params;
  const float* norm;
  float* dt;           // [ld]
  unsigned int* status;
  unsigned long long wait_ns;   // tensor-core wait limit (wait_limit_ns)
};

__global__ void __launch_bounds__(128, 1) mlp_infer_soa_kernel(InferArgs a) {
  using namespace tc;
  extern __shared__ __align__(1024) uint8_t smem[];
  const int s = threadIdx.x;
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + FW_BAR);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(smem + FW_BAR + 8);
  float* b = reinterpret_cast<float*>(smem + FW_BIAS);
  float* nrm = reinterpret_cast<float*>(smem + FW_NORM);
  for (int i = s; i < PK_FWD_BYTES / 16; i += 128)
    reinterpret_cast<uint4*>(smem + FW_W)[i] = reinterpret_cast<const uint4*>(a.packed)[i];
  if (s < 64) { b[s] = a.params[OFF_B1 + s]; b[64 + s] = a.params[OFF_B2 + s]; }
  if (s < 3) b[128 + s] = a.params[OFF_B3 + s];
  if (s < NNORM) nrm[s] = a.norm[s];
  if (s == 0) { mbar_init(bar, 1); fence_mbar_init(); }
  if (s < 32) { tmem_alloc(tslot, FW_TMEM_COLS); tmem_relinquish(); }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t taddr = *tslot;
  uint32_t phase = 0;
  bool ok = true;
  const int nchunks = (a.mp + 127) / 128;
  // the record words the inputs need, loaded one chunk ahead so the loads
  // of chunk c + gridDim.x are in flight while chunk c's tensor-core passes
  // run
  constexpr int NW = 17;
  constexpr int words[NW] = {0, 1, 2, 3, 5, 8, 32, 33, 38, 39, 46, 47, 48, 49, 50, 51, 0};
  auto fetch = [&](int c, float* w, int& iv, int& so) {
    const int t = c * 128 + s;
    if (c < nchunks && t < a.mp) {
#pragma unroll
      for (int q = 0; q < NW - 1; ++q) w[q] = __ldg(a.work_a + (size_t)words[q] * a.ld + t);
      iv = a.iveg[t] - 1;
      so = a.isoilm[t] - 1;
    } else {
      iv = -1;
      so = -1;
    }
  };
  float w[NW];
  int iv, so;
  fetch(blockIdx.x, w, iv, so);
  for (int c = blockIdx.x; c < nchunks; c += gridDim.x) {
    const int t = c * 128 + s;
    const bool valid = iv >= 0;
    float xn[NIN], y[NOUT];
    if (valid) {
      const CgPftTable& V = a.tables->pft;
      const CgSoilTable& S = a.tables->soil;
      const float tk = w[0], qv = w[1], pmb = w[2], ua = w[3], ca = w[4], vlaiw = w[5], sc = w[6] + w[7];
      const float dva = (qsatfjh(tk - TFRZ, pmb) - qv) * RMAIR / RMH2O * pmb * 100.0f;
      // fwsoil from the soil liquid water the radiation kernel recorded
      const float swilt = S.swilt[so], sfc = S.sfc[so];
      float rwater = 0.f;
#pragma unroll
      for (int k = 0; k < CG_MS; ++k)
        rwater += V.froot[k][iv] * fmaxf(1.0e-9f, fminf(1.0f, (w[10 + k] - swilt) / (sfc - swilt)));
      rwater = fmaxf(1.0e-9f, rwater);
      const float fwsoil = a.medlyn ? fmaxf(1.0e-4f, fminf(1.0f, rwater)) : fmaxf(1.0e-9f, fminf(1.0f, V.vbeta[iv] * rwater));
      const float f[NIN] = {w[8], w[9], tk, fmaxf(dva, 0.0f), ca, V.vcmax[iv] * sc,
                            V.ejmax[iv] * (1.0f - V.frac4[iv]) * sc, a.medlyn ? V.g1[iv] : V.a1gs[iv],
                            fwsoil, vlaiw, ua, tk};
#pragma unroll
      for (int q = 0; q < NIN; ++q) xn[q] = (f[q] - nrm[q]) * nrm[12 + q];
    } else {
#pragma unroll
      for (int q = 0; q < NIN; ++q) xn[q] = 0.f;
    }
    fetch(c + gridDim.x, w, iv, so);
    ok = forward128(smem, taddr, phase, xn, y, a.wait_ns);
    if (!ok) break;
    if (valid) a.dt[t] = y[2] * nrm[29] + nrm[26];
  }
  if (!ok) {
    settle(smem, phase);
    // no prediction for the rest: the canopy kernel starts those tiles as usual
    for (int c = blockIdx.x; c < nchunks; c += gridDim.x) {
      const int t = c * 128 + s;
      if (t < a.mp) a.dt[t] = __int_as_float(0x7fc00000);
    }
    if (s == 0) atomicOr(a.status, 2u);
  }
  fence_before_sync();
  __syncthreads();
  if (s < 32) tmem_dealloc(taddr, FW_TMEM_COLS);
}

// ------------------------------------------------------------------ update, pack, statistics
struct AdamArgs {
  float* params;
  float* m;
  float* v;
  const float* part;   // [nblk][NPARAM]
  int nblk;
  float* grad_out;     // optional: the summed gradient
  int apply;           // 0: gradient only
  float lr, beta1, beta2, eps;
  float bc1, bc2;      // 1 - beta^t
};

__global__ void mlp_update_kernel(AdamArgs a) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= NPARAM) return;
  float g = 0.f;
  for (int b = 0; b < a.nblk; ++b) g += a.part[(size_t)b * NPARAM + p];
  if (a.grad_out) a.grad_out[p] = g;
  if (!a.apply) return;
  const float m = a.beta1 * a.m[p] + (1.f - a.beta1) * g;
  const float v = a.beta2 * a.v[p] + (1.f - a.beta2) * g * g;
  a.m[p] = m;
  a.v[p] = v;
  a.params[p] -= a.lr * (m / a.bc1) / (sqrtf(v / a.bc2) + a.eps);
}

// BF16 operand image of the current master weights
__global__ void mlp_pack_kernel(const float* __restrict__ P, uint8_t* __restrict__ pk) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;   // one bf16 element of the image
  if (i >= PK_BYTES / 2) return;
  const int byte = 2 * i;
  float val = 0.f;
  // invert kmajor_offset for the region the element belongs to
  auto rc = [](int off, int K, int& r, int& k) {
    const int grp = off / ((K / 8) * 128), rem = off % ((K / 8) * 128);
    const int kc = rem / 128, in = rem % 128;
    r = grp * 8 + in / 16;
    k = kc * 8 + (in % 16) / 2;
  };
  int r, k;
  if (byte < PK_W2) {            // W1 [64][16]
    rc(byte - PK_W1, KIN, r, k);
    if (k < NIN) val = P[OFF_W1 + r * NIN + k];
  } else if (byte < PK_W3) {     // W2 [64][64]
    rc(byte - PK_W2, NH, r, k);
    val = P[OFF_W2 + r * NH + k];
  } else if (byte < PK_W3T) {    // W3 [16][64]
    rc(byte - PK_W3, NH, r, k);
    if (r < NOUT) val = P[OFF_W3 + r * NH + k];
  } else if (byte < PK_W2T) {    // W3^T [64][16]: (in r, out k)
    rc(byte - PK_W3T, KIN, r, k);
    if (k < NOUT) val = P[OFF_W3 + k * NH + r];
  } else {                       // W2^T [64][64]: (in r, out k)
    rc(byte - PK_W2T, NH, r, k);
    val = P[OFF_W2 + k * NH + r];
  }
  *reinterpret_cast<__nv_bfloat16*>(pk + byte) = __float2bfloat16_rn(val);
}

// per-column sums and sums of squares (FP64) of rows [0, n)
__global__ void column_stats_kernel(const float* __restrict__ rows, long long n, double* __restrict__ acc) {
  __shared__ double sh[2 * 15];
  if (threadIdx.x < 30) sh[threadIdx.x] = 0.0;
  __syncthreads();
  double s1[15], s2[15];
  for (int c = 0; c < 15; ++c) { s1[c] = 0.0; s2[c] = 0.0; }
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    for (int c = 0; c < 15; ++c) {
      const double x = rows[i * ROW + c];
      s1[c] += x;
      s2[c] += x * x;
    }
  }
  for (int c = 0; c < 15; ++c) {
    atomicAdd(&sh[c], s1[c]);
    atomicAdd(&sh[15 + c], s2[c]);
  }
  __syncthreads();
  if (threadIdx.x < 30) atomicAdd(&acc[threadIdx.x], sh[threadIdx.x]);
}

// ------------------------------------------------------------------ host trainer
#define SUR_CUDA(call)                                                          \
  do {                                                                          \
    cudaError_t e_ = (call);                                                    \
    if (e_ != cudaSuccess) {                                                    \
      err = std::string(#call ": ") + cudaGetErrorString(e_);                   \
      return CABLEGPU_ERR_CUDA;                                                 \
    }                                                                           \
  } while (0)

uint64_t splitmix(uint64_t& x) {
  uint64_t z = (x += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
double unit(uint64_t& x) { return ((splitmix(x) >> 11) + 0.5) * (1.0 / 9007199254740992.0); }

uint64_t gcd64(uint64_t a, uint64_t b) {
  while (b) { uint64_t t = a % b; a = b; b = t; }
  return a;
}

}  // namespace

int sur_alloc(SurNet& n, std::string& err) {
  int dev = 0, sms = 0;
  SUR_CUDA(cudaGetDevice(&dev));
  SUR_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  n.nblk = sms;
  SUR_CUDA(cudaMalloc(&n.params, NPARAM * sizeof(float)));
  SUR_CUDA(cudaMalloc(&n.m, NPARAM * sizeof(float)));
  SUR_CUDA(cudaMalloc(&n.v, NPARAM * sizeof(float)));
  SUR_CUDA(cudaMalloc(&n.norm, NNORM * sizeof(float)));
  SUR_CUDA(cudaMalloc(&n.packed, PK_BYTES));
  SUR_CUDA(cudaMalloc(&n.part, (size_t)n.nblk * NPARAM * sizeof(float)));
  SUR_CUDA(cudaMalloc(&n.loss_part, (size_t)n.nblk * sizeof(float)));
  SUR_CUDA(cudaMalloc(&n.grad, NPARAM * sizeof(float)));
  SUR_CUDA(cudaMalloc(&n.err, sizeof(unsigned int)));
  SUR_CUDA(cudaMemset(n.m, 0, NPARAM * sizeof(float)));
  SUR_CUDA(cudaMemset(n.v, 0, NPARAM * sizeof(float)));
  SUR_CUDA(cudaMemset(n.err, 0, sizeof(unsigned int)));
  SUR_CUDA(cudaFuncSetAttribute(mlp_train_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, TR_SMEM));
  SUR_CUDA(cudaFuncSetAttribute(mlp_forward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, FW_SMEM));
  SUR_CUDA(cudaFuncSetAttribute(mlp_infer_soa_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, FW_SMEM));
  return CABLEGPU_OK;
}

void sur_free(SurNet& n) {
  for (void* p : {(void*)n.params, (void*)n.m, (void*)n.v, (void*)n.norm, (void*)n.packed, (void*)n.part,
                  (void*)n.loss_part, (void*)n.grad, (void*)n.err})
    if (p) cudaFree(p);
  n = SurNet();
}

unsigned long long cg::sur::wait_limit_ns() {
  const char* v = std::getenv("CABLEGPU_DEBUG_TC_WAIT_NS");
  if (!v || !*v) return tc::kWaitNs;
  char* end = nullptr;
  const unsigned long long x = std::strtoull(v, &end, 10);
  return (end && *end == 0) ? std::min(x, (unsigned long long)tc::kWaitNs) : tc::kWaitNs;
}

int sur_infer(const SurNet& n, const float* work_a, const uint8_t* iveg, const uint8_t* isoilm, const CgTables* tables,
              int medlyn, int mp, int ld, float* dt, unsigned int* status, cudaStream_t st, std::string& err) {
  InferArgs a;
  a.work_a = work_a; a.iveg = iveg; a.isoilm = isoilm; a.tables = tables; a.medlyn = medlyn; a.mp = mp; a.ld = ld; a.packed = n.packed; a.params = n.params; a.norm = n.norm; a.dt = dt;
  a.status = status;
  a.wait_ns = wait_limit_ns();
  const int chunks = (mp + 127) / 128;
  const int grid = std::max(1, std::min(chunks, 8 * n.nblk));
  mlp_infer_soa_kernel<<<grid, 128, FW_SMEM, st>>>(a);
  SUR_CUDA(cudaGetLastError());
  return CABLEGPU_OK;
}

int sur_pack(SurNet& n, cudaStream_t st, std::string& err) {
  mlp_pack_kernel<<<(PK_BYTES / 2 + 255) / 256, 256, 0, st>>>(n.params, n.packed);
  SUR_CUDA(cudaGetLastError());
  return CABLEGPU_OK;
}

int sur_check_err(SurNet& n, cudaStream_t st, std::string& err) {
  unsigned int h = 0;
  SUR_CUDA(cudaMemcpyAsync(&h, n.err, sizeof(h), cudaMemcpyDeviceToHost, st));
  SUR_CUDA(cudaStreamSynchronize(st));
  if (h) {
    err = "surrogate kernel: a tensor-core completion did not arrive in time";
    SUR_CUDA(cudaMemsetAsync(n.err, 0, sizeof(unsigned int), st));
    return CABLEGPU_ERR_CUDA;
  }
  return CABLEGPU_OK;
}

// Gradient (and optionally an Adam update) for positions [pos0, pos0+nb) of
// the permutation row = (pa * pos + pc) % ntrain of d_rows.
int sur_step(SurNet& n, const float* d_rows, long long ntrain, long long pos0, int nb, unsigned long long pa,
             unsigned long long pc, bool apply, float lr, cudaStream_t st, std::string& err) {
  TrainArgs a;
  a.rows = d_rows; a.ntrain = ntrain; a.pos0 = pos0; a.n = nb; a.pa = pa; a.pc = pc;
  a.packed = n.packed; a.params = n.params; a.norm = n.norm; a.part = n.part; a.loss_part = n.loss_part;
  a.grad_scale = 2.0f / ((float)nb * NOUT);
  a.err = n.err;
  mlp_train_kernel<<<n.nblk, 128, TR_SMEM, st>>>(a);
  SUR_CUDA(cudaGetLastError());
  AdamArgs u;
  u.params = n.params; u.m = n.m; u.v = n.v; u.part = n.part; u.nblk = n.nblk; u.grad_out = n.grad;
  u.apply = apply ? 1 : 0;
  u.lr = lr; u.beta1 = 0.9f; u.beta2 = 0.999f; u.eps = 1e-8f;
  if (apply) ++n.adam_t;
  u.bc1 = 1.f - std::pow(0.9f, (float)std::max(1, n.adam_t));
  u.bc2 = 1.f - std::pow(0.999f, (float)std::max(1, n.adam_t));
  mlp_update_kernel<<<(NPARAM + 255) / 256, 256, 0, st>>>(u);
  SUR_CUDA(cudaGetLastError());
  if (apply) return sur_pack(n, st, err);
  return CABLEGPU_OK;
}

// Sum of squared normalised errors over rows [0, nrows) of d_rows.
int sur_eval(SurNet& n, const float* d_rows, long long nrows, float* y_dev, double* sse, cudaStream_t st,
             std::string& err) {
  SUR_CUDA(cudaMemsetAsync(n.loss_part, 0, n.nblk * sizeof(float), st));
  FwdArgs f;
  f.rows = d_rows; f.n = nrows; f.packed = n.packed; f.params = n.params; f.norm = n.norm; f.y = y_dev;
  f.loss_part = n.loss_part; f.err = n.err;
  f.wait_ns = wait_limit_ns();
  mlp_forward_kernel<<<n.nblk, 128, FW_SMEM, st>>>(f);
  SUR_CUDA(cudaGetLastError());
  std::vector<float> lp(n.nblk);
  SUR_CUDA(cudaMemcpyAsync(lp.data(), n.loss_part, n.nblk * sizeof(float), cudaMemcpyDeviceToHost, st));
  int rc = sur_check_err(n, st, err);
  if (rc) return rc;
  double s = 0.0;
  for (float x : lp) s += x;
  *sse = s;
  return CABLEGPU_OK;
}

// Normalisation from the rows [0, ntrain): input mean and 1/sd, output
// mean and sd (sd floored so constant columns stay finite).
int sur_set_norm(SurNet& n, const float* d_rows, long long ntrain, cudaStream_t st, std::string& err) {
  double* acc = nullptr;
  SUR_CUDA(cudaMalloc(&acc, 30 * sizeof(double)));
  SUR_CUDA(cudaMemsetAsync(acc, 0, 30 * sizeof(double), st));
  column_stats_kernel<<<256, 256, 0, st>>>(d_rows, ntrain, acc);
  double h[30];
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(h, acc, sizeof(h), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(acc);
  if (e != cudaSuccess) { err = std::string("column statistics: ") + cudaGetErrorString(e); return CABLEGPU_ERR_CUDA; }
  float nv[NNORM];
  for (int c = 0; c < 15; ++c) {
    const double mu = h[c] / (double)ntrain;
    const double var = std::max(0.0, h[15 + c] / (double)ntrain - mu * mu);
    const double sd = std::max(std::sqrt(var), 1e-6 * std::max(1.0, std::fabs(mu)));
    if (c < NIN) { nv[c] = (float)mu; nv[12 + c] = (float)(1.0 / sd); }
    else { nv[24 + (c - NIN)] = (float)mu; nv[27 + (c - NIN)] = (float)sd; }
  }
  SUR_CUDA(cudaMemcpyAsync(n.norm, nv, sizeof(nv), cudaMemcpyHostToDevice, st));
  SUR_CUDA(cudaStreamSynchronize(st));
  return CABLEGPU_OK;
}

// He-normal initial weights from a splitmix64 stream (Box-Muller).
void sur_init_params(float* P, unsigned long long seed) {
  uint64_t x = seed ^ 0x5DEECE66Dull;
  auto normal = [&]() {
    const double u1 = unit(x), u2 = unit(x);
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
  };
  for (int i = 0; i < NPARAM; ++i) P[i] = 0.f;
  for (int i = 0; i < NH * NIN; ++i) P[OFF_W1 + i] = (float)(normal() * std::sqrt(2.0 / NIN));
  for (int i = 0; i < NH * NH; ++i) P[OFF_W2 + i] = (float)(normal() * std::sqrt(2.0 / NH));
  for (int i = 0; i < NOUT * NH; ++i) P[OFF_W3 + i] = (float)(normal() * std::sqrt(1.0 / NH));
}

// Trains on rows [0, ntrain) of d_rows for `epochs` epochs of batches of
// `batch` rows (one affine permutation of the rows per epoch), evaluating
// the mean squared normalised error on rows [ntrain, ntrain + nval) after
// each epoch.  losses: [epochs][2] (train, validation), may be null.
int sur_fit(SurNet& n, const float* d_rows, long long ntrain, long long nval, int epochs, int batch, float lr,
            unsigned long long seed, bool init, float* losses, cudaStream_t st, std::string& err) {
  if (ntrain < 1 || batch < 128 || epochs < 1) { err = "fit: bad arguments"; return CABLEGPU_ERR_ARG; }
  int rc;
  if (init) {
    std::vector<float> P(NPARAM);
    sur_init_params(P.data(), seed);
    SUR_CUDA(cudaMemcpyAsync(n.params, P.data(), NPARAM * sizeof(float), cudaMemcpyHostToDevice, st));
    SUR_CUDA(cudaMemsetAsync(n.m, 0, NPARAM * sizeof(float), st));
    SUR_CUDA(cudaMemsetAsync(n.v, 0, NPARAM * sizeof(float), st));
    n.adam_t = 0;
    if ((rc = sur_set_norm(n, d_rows, ntrain, st, err))) return rc;
  }
  if ((rc = sur_pack(n, st, err))) return rc;
  uint64_t rs = seed * 0x2545F4914F6CDD1Dull + 1;
  std::vector<float> lp(n.nblk);
  for (int e = 0; e < epochs; ++e) {
    uint64_t pa = 1 + splitmix(rs) % (uint64_t)ntrain;
    while (gcd64(pa, (uint64_t)ntrain) != 1) pa = pa % (uint64_t)ntrain + 1;
    const uint64_t pc = splitmix(rs) % (uint64_t)ntrain;
    double sse = 0.0;
    for (long long p0 = 0; p0 < ntrain; p0 += batch) {
      const int nb = (int)std::min<long long>(batch, ntrain - p0);
      if ((rc = sur_step(n, d_rows, ntrain, p0, nb, pa, pc, true, lr, st, err))) return rc;
      SUR_CUDA(cudaMemcpyAsync(lp.data(), n.loss_part, n.nblk * sizeof(float), cudaMemcpyDeviceToHost, st));
      SUR_CUDA(cudaStreamSynchronize(st));
      for (float x : lp) sse += x;
    }
    if ((rc = sur_check_err(n, st, err))) return rc;
    double vse = 0.0;
    if (nval > 0 && (rc = sur_eval(n, d_rows + ntrain * ROW, nval, nullptr, &vse, st, err))) return rc;
    if (losses) {
      losses[2 * e] = (float)(sse / ((double)ntrain * NOUT));
      losses[2 * e + 1] = nval > 0 ? (float)(vse / ((double)nval * NOUT)) : 0.f;
    }
  }
  return CABLEGPU_OK;
}

// ------------------------------------------------------------------ C ABI (context-free)
namespace {
struct HostRun {
  SurNet net;
  float* rows = nullptr;
  cudaStream_t st = nullptr;
  std::string err;
  ~HostRun() {
    sur_free(net);
    if (rows) cudaFree(rows);
    if (st) cudaStreamDestroy(st);
  }
};
thread_local std::string g_mlp_error;

int host_setup(HostRun& h, const float* params, const float* norm, const float* rows, long long n) {
  std::string& err = h.err;
  SUR_CUDA(cudaStreamCreateWithFlags(&h.st, cudaStreamNonBlocking));
  int rc = sur_alloc(h.net, h.err);
  if (rc) return rc;
  SUR_CUDA(cudaMalloc(&h.rows, (size_t)std::max<long long>(n, 1) * ROW * sizeof(float)));
  SUR_CUDA(cudaMemcpyAsync(h.rows, rows, (size_t)n * ROW * sizeof(float), cudaMemcpyHostToDevice, h.st));
  if (params) SUR_CUDA(cudaMemcpyAsync(h.net.params, params, NPARAM * sizeof(float), cudaMemcpyHostToDevice, h.st));
  if (norm) SUR_CUDA(cudaMemcpyAsync(h.net.norm, norm, NNORM * sizeof(float), cudaMemcpyHostToDevice, h.st));
  return sur_pack(h.net, h.st, h.err);
}
}  // namespace

extern "C" {

int cablegpu_mlp_sizes(int* nparam, int* nnorm, int* row) {
  if (nparam) *nparam = NPARAM;
  if (nnorm) *nnorm = NNORM;
  if (row) *row = ROW;
  return CABLEGPU_OK;
}

int cablegpu_mlp_forward(const float* params, const float* norm, const float* rows, long long n, float* y) {
  if (!params || !norm || !rows || !y || n < 1) return CABLEGPU_ERR_ARG;
  HostRun h;
  int rc = host_setup(h, params, norm, rows, n);
  if (!rc) {
    float* dy = nullptr;
    double sse = 0.0;
    std::string& err = h.err;
    auto body = [&]() -> int {
      SUR_CUDA(cudaMalloc(&dy, (size_t)n * NOUT * sizeof(float)));
      int r = sur_eval(h.net, h.rows, n, dy, &sse, h.st, h.err);
      if (r) return r;
      SUR_CUDA(cudaMemcpyAsync(y, dy, (size_t)n * NOUT * sizeof(float), cudaMemcpyDeviceToHost, h.st));
      SUR_CUDA(cudaStreamSynchronize(h.st));
      return CABLEGPU_OK;
    };
    rc = body();
    if (dy) cudaFree(dy);
  }
  if (rc) g_mlp_error = h.err;
  return rc;
}

int cablegpu_mlp_grad(const float* params, const float* norm, const float* rows, long long n, float* grad,
                      float* loss) {
  if (!params || !norm || !rows || !grad || n < 1 || n > (1 << 30)) return CABLEGPU_ERR_ARG;
  HostRun h;
  int rc = host_setup(h, params, norm, rows, n);
  if (!rc) {
    std::string& err = h.err;
    auto body = [&]() -> int {
      int r = sur_step(h.net, h.rows, n, 0, (int)n, 1, 0, false, 0.f, h.st, h.err);
      if (r) return r;
      std::vector<float> lp(h.net.nblk);
      SUR_CUDA(cudaMemcpyAsync(grad, h.net.grad, NPARAM * sizeof(float), cudaMemcpyDeviceToHost, h.st));
      SUR_CUDA(cudaMemcpyAsync(lp.data(), h.net.loss_part, h.net.nblk * sizeof(float), cudaMemcpyDeviceToHost, h.st));
      r = sur_check_err(h.net, h.st, h.err);
      if (r) return r;
      double s = 0.0;
      for (float x : lp) s += x;
      if (loss) *loss = (float)(s / ((double)n * NOUT));
      return CABLEGPU_OK;
    };
    rc = body();
  }
  if (rc) g_mlp_error = h.err;
  return rc;
}

int cablegpu_mlp_fit(const float* rows, long long ntrain, long long nval, int epochs, int batch, float lr,
                     unsigned long long seed, float* params_out, float* norm_out, float* losses) {
  if (!rows || !params_out || !norm_out || ntrain < 1 || nval < 0) return CABLEGPU_ERR_ARG;
  HostRun h;
  int rc = host_setup(h, nullptr, nullptr, rows, ntrain + nval);
  if (!rc) rc = sur_fit(h.net, h.rows, ntrain, nval, epochs, batch, lr, seed, true, losses, h.st, h.err);
  if (!rc) {
    std::string& err = h.err;
    auto body = [&]() -> int {
      SUR_CUDA(cudaMemcpyAsync(params_out, h.net.params, NPARAM * sizeof(float), cudaMemcpyDeviceToHost, h.st));
      SUR_CUDA(cudaMemcpyAsync(norm_out, h.net.norm, NNORM * sizeof(float), cudaMemcpyDeviceToHost, h.st));
      SUR_CUDA(cudaStreamSynchronize(h.st));
      return CABLEGPU_OK;
    };
    rc = body();
  }
  if (rc) g_mlp_error = h.err;
  return rc;
}

const char* cablegpu_mlp_last_error(void) { return g_mlp_error.c_str(); }

}  // extern "C"
