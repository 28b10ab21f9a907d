// Phase C2 of the cbm() timestep kernel set -- soil heat: stempv (Thomas solve in FP64 on the reference's direct
// form, or in FP32 on the step's change), second snow_melting, remove_trans, soilfreeze.
#define CG_PHASE phase_c2
#define CG_PHASE_KERNEL cbm_phase_c2_kernel
#define CG_PHASE_LAUNCH launch_phase_c2
#define CG_PHASE_PREPARE prepare_phase_c2
#define CG_PHASE_COUPLED 1
#define CG_PHASE_SOLVE 1
#include "phase_kernels.cuh"
