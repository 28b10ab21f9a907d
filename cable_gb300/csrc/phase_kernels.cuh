// Kernel wrapper and host launcher for one phase of the timestep.  Each
// phase_X.cu translation unit includes this with CG_PHASE set, so the three
// phases compile in parallel and each can carry its own floating-point flags.
#pragma once
#include <cuda_runtime.h>
#include "cbm_step.cuh"

namespace cg {

constexpr int kPhaseBlock = 128;   // default threads per block; launches take any multiple of 32 up to 256
// Registers per thread (occupancy versus spills), set per phase translation
// unit; independent of the block size chosen at launch.
#ifndef CG_MAXNREG
#define CG_MAXNREG 128
#endif
// the cap of the FP64-solve instantiations of the soil kernels (their FP64
// elimination keeps more values live)
#ifndef CG_MAXNREG_S64
#define CG_MAXNREG_S64 CG_MAXNREG
#endif

// Launch one phase over D.mp tiles: a = radiation, b = canopy, c1 = snow
// pack, c2 = soil heat, c3 = soil water, carbon and balances.  clock, when non-null, holds ktau on the device (graph replay).
void launch_phase_a(bool diag, cudaStream_t s, const CgDev& D, const CgTables* T, const StepParams& P,
                    const int* clock, int block = kPhaseBlock);
void launch_phase_b(bool diag, cudaStream_t s, const CgDev& D, const CgTables* T, const StepParams& P,
                    const int* clock, int block = kPhaseBlock);
// canopy whose first dryLeaf iteration starts from the surrogate (D.sur_dt)
void launch_phase_b_sur(bool diag, cudaStream_t s, const CgDev& D, const CgTables* T, const StepParams& P,
                    const int* clock, int block = kPhaseBlock);
// canopy that also appends dryLeaf training rows to D.harvest
void launch_phase_b_harvest(bool diag, cudaStream_t s, const CgDev& D, const CgTables* T, const StepParams& P,
                    const int* clock, int block = kPhaseBlock);
void launch_phase_c1(bool diag, cudaStream_t s, const CgDev& D, const CgTables* T, const StepParams& P,
                    const int* clock, int block = kPhaseBlock);
void launch_phase_c2(bool diag, cudaStream_t s, const CgDev& D, const CgTables* T, const StepParams& P,
                    const int* clock, int block = kPhaseBlock);
void launch_phase_c3(bool diag, cudaStream_t s, const CgDev& D, const CgTables* T, const StepParams& P,
                    const int* clock, int block = kPhaseBlock);

// the canopy kernel's constant-memory copy of the plant-type table
void upload_canopy_pft_table(const CgPftTable& pft, cudaStream_t s);
// sets the canopy kernels' shared-memory limit for the dryLeaf pool and the
// L1 preference of the others (once per device, before the first launch)
void prepare_canopy_kernels();
// the L1 preference of the other phases' kernels (prepare_phase_kernels)
void prepare_phase_a();
void prepare_phase_c1();
void prepare_phase_c2();
void prepare_phase_c3();
// The step kernels use no shared memory; their register spills and local
// arrays are served by L1.  Without a preference an SM keeps the
// L1 / shared-memory split of the kernel it ran before, so after a kernel
// with a large shared-memory footprint (the surrogate network, the canopy's
// dryLeaf block pool) the next ones ran with a small L1.  The largest L1
// split is their stated preference.
template <class K>
void prefer_max_l1(K* kernel) {
  cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxL1);
}
inline void prepare_phase_kernels() {
  prepare_phase_a();
  prepare_canopy_kernels();
  prepare_phase_c1();
  prepare_phase_c2();
  prepare_phase_c3();
}

#ifdef CG_PHASE
// CG_PHASE_COUPLED 1: the phase has a second instantiation for the coupled
// calls (StepParams::mode != 0), so that the offline one carries none of
// their code; 0: one instantiation that tests the mode at run time.
#ifndef CG_PHASE_COUPLED
#define CG_PHASE_COUPLED 0
#endif
// CG_PHASE_SOLVE 1: the phase solves a soil tridiagonal system and has an
// instantiation per solve precision (StepParams::solve64: FP64 on the
// reference's direct form, or FP32 on the step's change).
#ifndef CG_PHASE_SOLVE
#define CG_PHASE_SOLVE 0
#endif
template <bool kDiag, bool kCoupled, bool kS64>
__global__ void __maxnreg__(kS64 ? CG_MAXNREG_S64 : CG_MAXNREG)
    CG_PHASE_KERNEL(CgDev D, const CgTables* __restrict__ T, StepParams P, const int* __restrict__ clock) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= D.mp) return;
  StepParams p = P;
  if (clock) { p.ktau = clock[0]; p.step_index = clock[0] - 1; }
#if CG_PHASE_SOLVE
  CG_PHASE<kDiag, kCoupled, kS64>(D, T, p, t);
#elif CG_PHASE_COUPLED
  CG_PHASE<kDiag, kCoupled>(D, T, p, t);
#else
  CG_PHASE<kDiag>(D, T, p, t);
#endif
}

// (internal linkage: every phase translation unit has its own copy under
// this name, launching its own kernel)
namespace {
template <bool kS64>
void launch_instance(bool diag, cudaStream_t s, const CgDev& D, const CgTables* T, const StepParams& P,
                     const int* clock, int block) {
  const int grid = (D.mp + block - 1) / block;
#if CG_PHASE_COUPLED
  if (P.mode != 0) {
    if (diag) CG_PHASE_KERNEL<true, true, kS64><<<grid, block, 0, s>>>(D, T, P, clock);
    else CG_PHASE_KERNEL<false, true, kS64><<<grid, block, 0, s>>>(D, T, P, clock);
    return;
  }
#endif
  if (diag) CG_PHASE_KERNEL<true, false, kS64><<<grid, block, 0, s>>>(D, T, P, clock);
  else CG_PHASE_KERNEL<false, false, kS64><<<grid, block, 0, s>>>(D, T, P, clock);
}
}  // namespace

void CG_PHASE_PREPARE() {
  prefer_max_l1(CG_PHASE_KERNEL<false, false, false>);
  prefer_max_l1(CG_PHASE_KERNEL<true, false, false>);
#if CG_PHASE_COUPLED
  prefer_max_l1(CG_PHASE_KERNEL<false, true, false>);
  prefer_max_l1(CG_PHASE_KERNEL<true, true, false>);
#endif
#if CG_PHASE_SOLVE
  prefer_max_l1(CG_PHASE_KERNEL<false, false, true>);
  prefer_max_l1(CG_PHASE_KERNEL<true, false, true>);
#if CG_PHASE_COUPLED
  prefer_max_l1(CG_PHASE_KERNEL<false, true, true>);
  prefer_max_l1(CG_PHASE_KERNEL<true, true, true>);
#endif
#endif
}

void CG_PHASE_LAUNCH(bool diag, cudaStream_t s, const CgDev& D, const CgTables* T, const StepParams& P,
                     const int* clock, int block) {
#if CG_PHASE_SOLVE
  if (P.solve64) {
    launch_instance<true>(diag, s, D, T, P, clock, block);
    return;
  }
#endif
  launch_instance<false>(diag, s, D, T, P, clock, block);
}
#endif

}  // namespace cg
