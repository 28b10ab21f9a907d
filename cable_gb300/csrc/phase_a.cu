// Phase A of the cbm() timestep kernel set -- radiation: ruff_resist, define_air, init_radiation, albedo, interception, radiation.
#define CG_PHASE phase_a
#define CG_PHASE_KERNEL cbm_phase_a_kernel
#define CG_PHASE_LAUNCH launch_phase_a
#define CG_PHASE_PREPARE prepare_phase_a
#define CG_PHASE_COUPLED 1
#include "phase_kernels.cuh"

