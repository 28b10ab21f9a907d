// Phase C1 of the cbm() timestep kernel set -- snow pack: snowcheck, snowdensity, snow_accum, snow_melting, snowl_adjust.
#define CG_PHASE phase_c1
#define CG_PHASE_KERNEL cbm_phase_c1_kernel
#define CG_PHASE_LAUNCH launch_phase_c1
#define CG_PHASE_PREPARE prepare_phase_c1
#define CG_PHASE_COUPLED 1
#include "phase_kernels.cuh"
