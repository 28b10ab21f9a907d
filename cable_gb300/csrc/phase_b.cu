// Phase B of the cbm() timestep kernel set -- canopy: define_canopy (Monin-Obukhov loop with dryLeaf / wetLeaf, soil evaporation).
#include "cbm_step.cuh"

namespace cg {
// the plain canopy kernel's phase, in the <kDiag, kCoupled> form the shared
// kernel wrapper instantiates
template <bool kDiag, bool kCoupled>
__device__ __forceinline__ void phase_b_plain(const CgDev& D, const CgTables* __restrict__ T, const StepParams& P,
                                              int t) {
  phase_b<kDiag, false, false, kCoupled>(D, T, P, t);
}
}  // namespace cg

#define CG_PHASE phase_b_plain
#define CG_PHASE_KERNEL cbm_phase_b_kernel
#define CG_PHASE_LAUNCH launch_phase_b
#define CG_PHASE_COUPLED 1
#include "phase_kernels.cuh"

namespace cg {

// The canopy kernel that also records dryLeaf training rows.
template <bool kDiag>
__global__ void __maxnreg__(CG_MAXNREG)
    cbm_phase_b_harvest_kernel(CgDev D, const CgTables* __restrict__ T, StepParams P, const int* __restrict__ clock) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= D.mp) return;
  StepParams p = P;
  if (clock) { p.ktau = clock[0]; p.step_index = clock[0] - 1; }
  phase_b<kDiag, true>(D, T, p, t);
}

void launch_phase_b_harvest(bool diag, cudaStream_t s, const CgDev& D, const CgTables* T, const StepParams& P,
                            const int* clock, int block) {
  const int grid = (D.mp + block - 1) / block;
  if (diag) cbm_phase_b_harvest_kernel<true><<<grid, block, 0, s>>>(D, T, P, clock);
  else cbm_phase_b_harvest_kernel<false><<<grid, block, 0, s>>>(D, T, P, clock);
}

// The canopy kernel whose first dryLeaf iteration starts from the
// surrogate network's prediction (D.sur_dt).
template <bool kDiag>
__global__ void __maxnreg__(CG_MAXNREG)
    cbm_phase_b_sur_kernel(CgDev D, const CgTables* __restrict__ T, StepParams P, const int* __restrict__ clock) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= D.mp) return;
  StepParams p = P;
  if (clock) { p.ktau = clock[0]; p.step_index = clock[0] - 1; }
  phase_b<kDiag, false, true>(D, T, p, t);
}

void launch_phase_b_sur(bool diag, cudaStream_t s, const CgDev& D, const CgTables* T, const StepParams& P,
                        const int* clock, int block) {
  const int grid = (D.mp + block - 1) / block;
  if (diag) cbm_phase_b_sur_kernel<true><<<grid, block, 0, s>>>(D, T, P, clock);
  else cbm_phase_b_sur_kernel<false><<<grid, block, 0, s>>>(D, T, P, clock);
}

void upload_canopy_pft_table(const CgPftTable& pft, cudaStream_t s) {
  cudaMemcpyToSymbolAsync(c_pft, &pft, sizeof(CgPftTable), 0, cudaMemcpyHostToDevice, s);
}

}  // namespace cg
