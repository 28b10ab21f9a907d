// Blackwell (sm_103a) tensor-core primitives in inline PTX: tensor memory
// allocation, tcgen05.mma with shared-memory operand descriptors, commit to
// an mbarrier, and tensor-memory loads.  Used by the surrogate network's
// kernels (surrogate.cu) and by the canopy kernel's in-loop surrogate.
//
// Operand layout: "K-major, no swizzle".  An R x K bf16 matrix (R a multiple
// of 8, K of 16) is stored as core matrices of 8 rows x 8 elements (16 bytes
// per row, 128 contiguous bytes); core matrices adjacent along K are 128
// bytes apart (leading byte offset), 8-row groups are K/8 * 128 bytes apart
// (stride byte offset).  Element (r, k) sits at byte
//   (r / 8) * (K / 8) * 128 + (k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2.
// One MMA consumes K = 16, i.e. the two core-matrix columns starting at
// byte (k0 / 8) * 128 of the buffer.
#pragma once
#include <cstdint>

namespace cg {
namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// byte offset of element (r, k) in a K-major no-swizzle R x K bf16 matrix
__host__ __device__ __forceinline__ constexpr uint32_t kmajor_offset(uint32_t r, uint32_t k, uint32_t K) {
  return (r >> 3) * (K >> 3) * 128u + (k >> 3) * 128u + (r & 7u) * 16u + (k & 7u) * 2u;
}

// Shared-memory matrix descriptor (tcgen05 format): start address, leading
// and stride byte offsets (all >> 4), descriptor version 1 at bits 46-48,
// base offset 0, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1u << 46;
  return d;
}
// descriptor of the K = 16 slice starting at column k0 of a K-major matrix
// with K columns at shared address base
__device__ __forceinline__ uint64_t kslice_desc(uint32_t base, uint32_t k0, uint32_t K) {
  return smem_desc(base + (k0 >> 3) * 128u, 128u, (K >> 3) * 128u);
}

// Instruction descriptor of kind::f16 with BF16 A and B (both K-major), FP32
// accumulator, M x N tile.
__host__ __device__ __forceinline__ constexpr uint32_t idesc_bf16(uint32_t M, uint32_t N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((N >> 3) << 17) | ((M >> 4) << 24);
}

// ---------------------------------------------------------------- mbarrier
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ uint64_t globaltimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}
// Default wait limit: 0.2 s of wall time (a tensor-core pass completes in
// microseconds).
constexpr uint64_t kWaitNs = 200000000ull;
// Waits for the phase with parity `parity` to complete.  Gives up and
// returns false after max_ns nanoseconds of wall time, so no caller can wait
// forever.  max_ns == 0 gives up at once without polling: the debug setting
// that exercises the callers' give-up path deterministically.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint64_t max_ns = kWaitNs) {
  if (max_ns == 0) return false;
  const uint32_t addr = smem_u32(bar);
  const uint64_t t0 = globaltimer_ns();
  while (true) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(addr), "r"(parity)
        : "memory");
    if (done) return true;
    if (globaltimer_ns() - t0 > max_ns) return false;
  }
}

// ---------------------------------------------------------------- tensor memory
// alloc / relinquish / dealloc are executed by one whole warp
__device__ __forceinline__ void tmem_alloc(uint32_t* smem_dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(smem_dst)),
               "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// makes generic-proxy shared-memory writes visible to the tensor core
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// D[tmem] = A * B (+ D if accumulate), issued by one thread
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
// arrives on `bar` once every MMA this thread issued before has completed
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// 16 consecutive FP32 columns of this thread's tensor-memory lane (the warp
// reads its own 32 lanes), waiting for the load to complete.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];\n\t"
      "tcgen05.wait::ld.sync.aligned;\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// ---------------------------------------------------------------- bf16 packing
// round-to-nearest-even FP32 -> BF16 of two values, lo in the low half
__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
  uint32_t r;
  asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
  return r;
}

}  // namespace tc
}  // namespace cg
