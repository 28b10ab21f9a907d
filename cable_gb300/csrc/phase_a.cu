// Phase A of the cbm() timestep kernel set -- radiation: ruff_resist, define_air, init_radiation, albedo, interception, radiation.
#define CG_PHASE phase_a
#define CG_PHASE_KERNEL cbm_phase_a_kernel
#define CG_PHASE_LAUNCH launch_phase_a
#include "phase_kernels.cuh"

namespace cg {

// The radiation kernel that also writes the dryLeaf surrogate's inputs.
template <bool kDiag>
__global__ void __launch_bounds__(kPhaseBlock, CG_MIN_BLOCKS)
    cbm_phase_a_sur_kernel(CgDev D, const CgTables* __restrict__ T, StepParams P, const int* __restrict__ clock) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= D.mp) return;
  StepParams p = P;
  if (clock) { p.ktau = clock[0]; p.step_index = clock[0] - 1; }
  phase_a<kDiag, true>(D, T, p, t);
}

void launch_phase_a_sur(bool diag, cudaStream_t s, const CgDev& D, const CgTables* T, const StepParams& P,
                        const int* clock) {
  const int grid = (D.mp + kPhaseBlock - 1) / kPhaseBlock;
  if (diag) cbm_phase_a_sur_kernel<true><<<grid, kPhaseBlock, 0, s>>>(D, T, P, clock);
  else cbm_phase_a_sur_kernel<false><<<grid, kPhaseBlock, 0, s>>>(D, T, P, clock);
}

}  // namespace cg
