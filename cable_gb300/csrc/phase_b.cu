// Phase B of the cbm() timestep kernel set -- canopy: define_canopy (Monin-Obukhov loop with dryLeaf / wetLeaf, soil evaporation).
#define CG_PHASE phase_b
#define CG_PHASE_KERNEL cbm_phase_b_kernel
#define CG_PHASE_LAUNCH launch_phase_b
#include "phase_kernels.cuh"
