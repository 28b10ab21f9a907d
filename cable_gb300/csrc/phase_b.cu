// Phase B of the cbm() timestep kernel set -- canopy: define_canopy (Monin-Obukhov loop with dryLeaf / wetLeaf,
// soil evaporation).  One kernel template for the plain, training-row harvesting, surrogate-started and coupled
// variants, each with the dryLeaf passes scheduled per lane or as a block pool (dryleaf.cuh).
#include "phase_kernels.cuh"

namespace cg {

// register cap of the pooling instantiations (their pass runs while the
// thread's own tile's canopy state stays live)
#ifndef CG_MAXNREG_POOL
#define CG_MAXNREG_POOL CG_MAXNREG
#endif

template <bool kDiag, bool kHarvest, bool kSur, bool kCoupled, bool kPool>
__global__ void __maxnreg__(kPool ? CG_MAXNREG_POOL : CG_MAXNREG)
    cbm_phase_b_kernel(CgDev D, const CgTables* __restrict__ T, StepParams P, const int* __restrict__ clock) {
  extern __shared__ __align__(16) float dl_sm[];
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  // a pooling block's threads beyond the last tile run as ghosts (phase_b)
  if (!kPool && t >= D.mp) return;
  StepParams p = P;
  if (clock) { p.ktau = clock[0]; p.step_index = clock[0] - 1; }
  phase_b<kDiag, kHarvest, kSur, kCoupled, kPool>(D, T, p, t, dl_sm);
}

namespace {
// the largest block the pool's shared memory is sized for (launches take
// 32..256 threads)
constexpr int kPoolMaxBlock = 256;

template <bool kDiag, bool kHarvest, bool kSur, bool kCoupled>
void launch_variant(cudaStream_t s, const CgDev& D, const CgTables* T, const StepParams& P, const int* clock,
                    int block) {
  const int grid = (D.mp + block - 1) / block;
  if (P.canopy_pool)
    cbm_phase_b_kernel<kDiag, kHarvest, kSur, kCoupled, true>
        <<<grid, block, dlp::smem_bytes(block, kSur), s>>>(D, T, P, clock);
  else
    cbm_phase_b_kernel<kDiag, kHarvest, kSur, kCoupled, false><<<grid, block, 0, s>>>(D, T, P, clock);
}

template <bool kHarvest, bool kSur, bool kCoupled>
void prepare_variant() {
  const int bytes = dlp::smem_bytes(kPoolMaxBlock, kSur);
  cudaFuncSetAttribute(cbm_phase_b_kernel<false, kHarvest, kSur, kCoupled, true>,
                       cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  cudaFuncSetAttribute(cbm_phase_b_kernel<true, kHarvest, kSur, kCoupled, true>,
                       cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  prefer_max_l1(cbm_phase_b_kernel<false, kHarvest, kSur, kCoupled, false>);
  prefer_max_l1(cbm_phase_b_kernel<true, kHarvest, kSur, kCoupled, false>);
}
}  // namespace

void launch_phase_b(bool diag, cudaStream_t s, const CgDev& D, const CgTables* T, const StepParams& P,
                    const int* clock, int block) {
  if (P.mode != 0) {
    if (diag) launch_variant<true, false, false, true>(s, D, T, P, clock, block);
    else launch_variant<false, false, false, true>(s, D, T, P, clock, block);
    return;
  }
  if (diag) launch_variant<true, false, false, false>(s, D, T, P, clock, block);
  else launch_variant<false, false, false, false>(s, D, T, P, clock, block);
}

// The canopy kernel that also records dryLeaf training rows.
void launch_phase_b_harvest(bool diag, cudaStream_t s, const CgDev& D, const CgTables* T, const StepParams& P,
                            const int* clock, int block) {
  if (diag) launch_variant<true, true, false, false>(s, D, T, P, clock, block);
  else launch_variant<false, true, false, false>(s, D, T, P, clock, block);
}

// The canopy kernel whose first dryLeaf iteration starts from the surrogate
// network's prediction (D.sur_dt).
void launch_phase_b_sur(bool diag, cudaStream_t s, const CgDev& D, const CgTables* T, const StepParams& P,
                        const int* clock, int block) {
  if (diag) launch_variant<true, false, true, false>(s, D, T, P, clock, block);
  else launch_variant<false, false, true, false>(s, D, T, P, clock, block);
}

void prepare_canopy_kernels() {
  prepare_variant<false, false, false>();
  prepare_variant<false, false, true>();
  prepare_variant<true, false, false>();
  prepare_variant<false, true, false>();
}

void upload_canopy_pft_table(const CgPftTable& pft, cudaStream_t s) {
  cudaMemcpyToSymbolAsync(c_pft, &pft, sizeof(CgPftTable), 0, cudaMemcpyHostToDevice, s);
}

}  // namespace cg
