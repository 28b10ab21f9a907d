/*
 * cablegpu.h - C ABI of the GB300 implementation of CABLE's per-timestep
 * tile physics (the offline cbm() call, and the ACCESS coupling's
 * cbm_expl / cbm_impl: cablegpu_step_explicit / cablegpu_step_implicit).
 *
 * Replaces, for the offline driver, the reference interface
 *   SUBROUTINE cbm(ktau, dels, air, bgc, canopy, met, bal, rad, rough, soil,
 *                  ssnow, sum_flux, veg, climate, xk, c1, rhoch)
 *   src/offline/cbl_model_driver_offline.F90:38-40
 * called once per timestep from the serial driver
 *   src/offline/cable_serial.F90:594-595
 * and from the MPI worker (src/offline/cable_mpiworker.F90:503).
 *
 * Model: the library owns device-resident structure-of-arrays copies of the
 * per-tile state.  The caller (the Fortran shim in
 * cable_gb300/fortran/cable_cbm_gpu.F90, or any C/Python host) uploads the
 * tile parameters and state once, then calls cablegpu_step() once per
 * timestep (or cablegpu_run() for many steps, replayed as a CUDA graph) and
 * downloads fields only when it needs them (output steps, restart files).
 *
 * Array convention: every per-tile field is a host array of nlayer * mp
 * elements in Fortran column-major order of the reference's (mp, nlayer)
 * arrays, i.e. element (tile i, layer k) at [k * mp + i]; the element type
 * is the field's dtype (CABLEGPU_F32 = REAL, CABLEGPU_F64 = REAL(r_2),
 * CABLEGPU_I32 = INTEGER).
 *
 * Errors: every function returns 0 on success and a negative CABLEGPU_ERR_*
 * code otherwise; cablegpu_last_error() describes the last failure.  No
 * entry point traps or aborts.  Calls on one context are not thread-safe and
 * run in order on the context's CUDA stream.
 */
#ifndef CABLEGPU_H
#define CABLEGPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CABLEGPU_OK 0
#define CABLEGPU_ERR_ARG (-1)        /* bad argument (null, out of range, unknown field) */
#define CABLEGPU_ERR_CUDA (-2)       /* a CUDA runtime call failed */
#define CABLEGPU_ERR_NONFINITE (-3)  /* a step produced a non-finite output flux */
#define CABLEGPU_ERR_STATE (-4)      /* call not valid in the context's current state */
#define CABLEGPU_ERR_IO (-5)         /* a file could not be read or written, or is not a valid file */

#define CABLEGPU_F32 0
#define CABLEGPU_F64 1
#define CABLEGPU_I32 2
#define CABLEGPU_DF32 3   /* files only: double-FP32 pairs, `width` high rows then `width` low rows */

#define CABLEGPU_KIND_PARAM 0   /* static per-tile parameter (veg / soil / forcing jitter) */
#define CABLEGPU_KIND_STATE 1   /* prognostic state carried between steps */
#define CABLEGPU_KIND_OUTPUT 2  /* written every step */
#define CABLEGPU_KIND_DIAG 3    /* written every step when diagnostics are enabled */
#define CABLEGPU_KIND_FORCING 4 /* met forcing of the last step, when capture is enabled */
#define CABLEGPU_KIND_WORK 5    /* per-tile records handed between the kernels of one step */

#define CABLEGPU_NFORCING 13    /* fsd_vis fsd_nir fld precip precip_sn tk pmb ua qv ca coszen doy hod */

typedef struct cablegpu_ctx cablegpu_ctx;

/* Static description of the tiles (veg%iveg, soil%isoilm, veg%vlai,
 * rad%latitude).  The three forcing-jitter arrays only drive the built-in
 * synthetic forcing generator and may be NULL (defaults 0 h, 288 K, 1.0). */
typedef struct {
  int mp;
  const int* iveg;       /* [mp] plant functional type 1..17 */
  const int* isoilm;     /* [mp] soil type 1..9 */
  const float* vlai;     /* [mp] leaf area index */
  const float* lat;      /* [mp] latitude, degrees north */
  const float* lonphase; /* [mp] local-time offset of the synthetic forcing, hours in [0, 24) */
  const float* tbase;    /* [mp] base air temperature of the synthetic forcing, K */
  const float* swscale;  /* [mp] shortwave scale factor of the synthetic forcing */
  int order;             /* device tile order: 0 = grouped by plant and soil type (default; warps
                            then follow coherent code paths), 1 = as given, 2 = grouped by plant
                            type, local solar hour, latitude band and LAI (warps then share
                            iteration counts), 3 = order 2 within consecutive chunks of 2^18
                            tiles (keeps host-order I/O of cablegpu_step_host L2-local), -1 =
                            chosen by the autotuner (cablegpu_autotune) on these tiles.  Field I/O is always in the caller's order and
                            results do not depend on this choice. */
} cablegpu_tiles;

/* Creates a context on CUDA device `device` for tiles->mp tiles and uploads
 * the tile description.  Replaces the per-run set-up the reference driver
 * does before its time loop (load_parameters, cable_serial.F90:399).
 * 1 <= tiles->mp <= CABLEGPU_MAX_TILES, else CABLEGPU_ERR_ARG: the kernels
 * address a tile's row of a multi-row field (up to 64 rows: the
 * diagnostics block, the hand-off records) with 32-bit offsets, and a
 * context of that many tiles takes ~34 GB of device memory; a larger grid
 * is split over several contexts. */
#define CABLEGPU_MAX_TILES 33554176
int cablegpu_create(const cablegpu_tiles* tiles, int device, cablegpu_ctx** out);
int cablegpu_destroy(cablegpu_ctx* ctx);

/* Cold-start state, as the reference initialises a run without a restart
 * file (cable_parameters.F90 write_default_params :1188-1262, :1607-1650;
 * cable_initialise.F90 get_default_inits :72-144; derived_parameters
 * owetfac :2246-2254): snow water equivalent, soil temperature and soil
 * moisture per tile (host arrays [mp]; layers start uniform).  */
int cablegpu_cold_start(cablegpu_ctx* ctx, const double* snowd0, const double* tgg0, const double* wb0);

/* Cold start that allocates nothing (no counterpart in the reference).
 * Same result as cablegpu_cold_start, but the three input arrays are staged
 * in a fixed 1.5 MiB device array compiled into the library instead of a
 * buffer cudaMalloc'd and cudaFree'd per call.  For callers that cannot
 * allocate or free at that point: a host model restarting tiles while other
 * streams of the device are busy (cudaFree synchronises the device), one
 * whose memory pool owns every free byte, or one in a region where another
 * thread captures a CUDA graph in global mode.  Limits: at most
 * CABLEGPU_NOALLOC_MAX_TILES tiles (larger contexts get CABLEGPU_ERR_ARG);
 * the staging array is shared by all contexts on a device, so calls must not
 * overlap (from any thread); the call returns after its kernel ran.  The
 * first call on a device resolves the array's address and may load the
 * library's device code, so make it before any stream capture begins.  The
 * address is kept for the life of the process: a cudaDeviceReset of that
 * device invalidates it, so do not use this entry point on a device after
 * resetting it (cablegpu_cold_start has no such restriction). */
#define CABLEGPU_NOALLOC_MAX_TILES 65536
int cablegpu_cold_start_noalloc(cablegpu_ctx* ctx, const double* snowd0, const double* tgg0, const double* wb0);

/* Field registry. */
int cablegpu_num_fields(void);
int cablegpu_field_info(int id, const char** name, int* nlayer, int* dtype, int* kind);
int cablegpu_field_id(const char* name);
/* Host <-> device copies of one field (host array [nlayer * mp], field dtype).
 * set: the reference's derived-type components are written by the caller
 * (e.g. a restart read, cable_initialise.F90 get_restart_data :163-664);
 * get: the caller reads them back (output / restart write). */
int cablegpu_set_field(cablegpu_ctx* ctx, int id, const void* host);
int cablegpu_get_field(cablegpu_ctx* ctx, int id, void* host);
/* Copies n fields to host buffers in one call (host[i] as for
 * cablegpu_get_field of field ids[i]): the gathers and device-to-host copies
 * go out back to back on the context's stream and the call waits once,
 * where n calls of cablegpu_get_field wait n times.  The per-step copy-back
 * of a driver (the Fortran shim's groups of driver-read fields; the
 * reference's types are filled in place between cbm() calls, which needs no
 * copy).  Stops at the first bad id with CABLEGPU_ERR_ARG; fields before it
 * have been copied. */
int cablegpu_get_fields(cablegpu_ctx* ctx, int n, const int* ids, void* const* host);
/* Device pointer and leading dimension (elements between layers) of a field,
 * for callers that keep their own device-side pipelines. */
int cablegpu_field_device_ptr(cablegpu_ctx* ctx, int id, void** dptr, int* ld);

/* Met forcing for the next step from host memory, [CABLEGPU_NFORCING][mp]
 * float (the met_type fields get_met_data fills, cable_input.F90).  Stays in
 * effect for every later step until replaced or until synthetic forcing is
 * selected. */
int cablegpu_set_forcing(cablegpu_ctx* ctx, const float* host_forcing);
/* Built-in seeded synthetic forcing generated inside the step kernel. */
int cablegpu_set_synthetic_forcing(cablegpu_ctx* ctx, unsigned long long seed, int doy0);

/* switches: bit mask of the reference's science switches (cable_user,
 * cable_runtime_opts_mod.F90:28-123); 0 = the offline defaults.
 *   CABLEGPU_SW_MEDLYN            gs_switch = 'medlyn' instead of 'leuning'
 *                                 (cbl_dryLeaf.F90:412-433)
 *   CABLEGPU_SW_SOIL_THERMAL_FIX  soil_thermal_fix: total_soil_conductivity in
 *                                 stempv (cbl_stempv.F90:57-61,
 *                                 cbl_conductivity.F90:10-85) and the soil
 *                                 heat parameters rewritten as
 *                                 cable_parameters.F90:2165-2227 does
 *   CABLEGPU_SW_LITTER            litter: litter resistances to soil heat and
 *                                 vapour transfer in define_canopy
 *                                 (cable_canopy.F90:471-476, :521-530,
 *                                 :808-854, :979-997; cbl_pot_evap_snow.F90
 *                                 :155-157; cbl_within_canopy.F90:80-84) with
 *                                 the static litter carbon of pft_params.nml
 *   CABLEGPU_SW_L_REV_CORR        l_rev_corr: revised soil-coupling
 *                                 derivatives (cable_canopy.F90:916-922,
 *                                 :993-1014); its other uses act only in the
 *                                 coupled model (cable_runtime%um) or on
 *                                 fns_cor, which is 0 offline
 *   CABLEGPU_SW_FWSOIL_NONLINEAR  fwsoil_switch = 'non-linear extrapolation'
 *                                 (cbl_fwsoil.F90:44-88)
 *   CABLEGPU_SW_FWSOIL_LAI_KTAUL  fwsoil_switch = 'Lai and Ktaul 2000'
 *                                 (cbl_fwsoil.F90:90-112)
 *   CABLEGPU_SW_POTEV_PM          ssnow_potev = 'P-M': Penman-Monteith soil
 *                                 potential evaporation
 *                                 (cbl_pot_evap_snow.F90:9-78), which reads
 *                                 canopy%ga of the last step (output row 6)
 *   CABLEGPU_SW_NEW_REDUCE_SOILEVP  l_new_reduce_soilevp
 *                                 (cbl_latent_heat.F90:205-210)
 *   CABLEGPU_SW_NEW_RUNOFF_SPEED  l_new_runoff_speed (cbl_smoisturev.F90:112,
 *                                 :153-197)
 *   CABLEGPU_SW_DIAG_SOIL_RESP_OFF  diag_soil_resp = 'OFF': the rs20 soil
 *                                 respiration scheme (cable_carbon.F90:256-276;
 *                                 the offline cable.nml sets 'ON')
 * An unknown bit, or both fwsoil bits, is an error.
 * diag: 1 = write the per-tile diagnostics fields every step.
 * capture_forcing: 1 = keep a copy of each step's forcing (field "forcing"). */
#define CABLEGPU_SW_MEDLYN 1
#define CABLEGPU_SW_SOIL_THERMAL_FIX 2
#define CABLEGPU_SW_LITTER 4
#define CABLEGPU_SW_L_REV_CORR 8
#define CABLEGPU_SW_FWSOIL_NONLINEAR 16
#define CABLEGPU_SW_FWSOIL_LAI_KTAUL 32
#define CABLEGPU_SW_POTEV_PM 64
#define CABLEGPU_SW_NEW_REDUCE_SOILEVP 128
#define CABLEGPU_SW_NEW_RUNOFF_SPEED 256
#define CABLEGPU_SW_DIAG_SOIL_RESP_OFF 512
int cablegpu_set_options(cablegpu_ctx* ctx, int switches, int diag, int capture_forcing);

/* Arithmetic of the two soil tridiagonal (Thomas) solves, heat (stempv,
 * cbl_stempv.F90:201-214) and moisture (smoisturev, cbl_smoisturev.F90:422):
 *   CABLEGPU_SOLVE_FP64        (default) the reference's: each system in FP64
 *                              on its direct form (cbl_trimb.F90:17-53), the
 *                              coefficients formed in FP32
 *   CABLEGPU_SOLVE_FP32_CHANGE the same systems solved in FP32 for the step's
 *                              change of the state (right-hand side formed
 *                              from differences of the old state), the soil
 *                              water applied as interface fluxes; faster, and
 *                              within the tolerances of the FP64 solve
 * Applies to the steps issued after the call. */
#define CABLEGPU_SOLVE_FP64 0
#define CABLEGPU_SOLVE_FP32_CHANGE 1
int cablegpu_set_soil_solve(cablegpu_ctx* ctx, int mode);

/* Scheduling of the canopy kernel's dryLeaf passes (cbl_dryLeaf.F90:10-666,
 * up to 20 passes per tile and Monin-Obukhov iteration, converging after
 * different numbers of passes):
 *   CABLEGPU_CANOPY_LANES (default) each thread runs its own tile's passes
 *   CABLEGPU_CANOPY_POOL  the tiles of a thread block iterate as a pool in
 *                         shared memory: each round runs one pass of every
 *                         tile still iterating, one tile per thread (a warp
 *                         vote and one atomic per warp build the next
 *                         round's list), so threads whose tile converged take
 *                         other tiles' passes; slower on GB300 (the slot
 *                         traffic and the per-round barrier cost more than
 *                         the idle lanes it recovers)
 * Results are identical; only the speed differs.  Applies to the steps issued
 * after the call. */
#define CABLEGPU_CANOPY_POOL 0
#define CABLEGPU_CANOPY_LANES 1
int cablegpu_set_canopy_schedule(cablegpu_ctx* ctx, int mode);

/* One timestep, ktau 1-based (cbm(ktau, dels, ...) followed by the driver's
 * balance checks).  Asynchronous; errors of the step surface at the next
 * synchronising call. */
int cablegpu_step(cablegpu_ctx* ctx, int ktau, float dels);

/* ACCESS coupling: the two halves of a coupled timestep, replacing
 *   SUBROUTINE cbm_expl(mp, nrb, ktau, dels, air, bgc, canopy, met, bal, rad,
 *                       rough, soil, ssnow, sum_flux, veg, climate)
 *   SUBROUTINE cbm_impl(cycleno, numcycles, mp, nrb, ktau, dels, air, bgc,
 *                       canopy, met, bal, rad, rough, soil, ssnow, sum_flux,
 *                       veg, climate)
 *   src/coupled/AM3/control/cable/CM3/cbl_cbm_mod.F90:10-182, :184-396
 * called from cable_explicit_driver.F90:266 and cable_implicit_driver.F90:200.
 * Forcing comes as for cablegpu_step (cablegpu_set_forcing / the synthetic
 * generator); between the two calls the host model updates the air
 * temperature and humidity (cable_implicit_driver.F90:189-198).
 *
 * cablegpu_step_explicit: radiation and canopy fluxes from the current state
 * (three kernel launches: radiation, canopy, radiative temperature).  The canopy water, soil wetness factor and surface
 * temperature are left as they were (cbl_cbm_mod.F90:150-152); the canopy's
 * soil resistance (rtsoil) and ga are kept, as in the reference.  Outputs:
 * all eight rows of "out", trad from the start-of-step surface temperature
 * (:172-179).  lai_refresh != 0 when the host model's radiation call ran since
 * the last explicit call: the snow-reduced LAI (canopy%vlaiw, state field
 * "vlaiw") is then recomputed from the current snow state
 * (cable_land_albedo_mod_cbl.F90:263); otherwise the carried value is used
 * (cable_roughness.F90:176-186 skips it in coupled calls).  The first
 * explicit call of a run passes lai_refresh = 1.
 *
 * cablegpu_step_implicit: canopy, soil and snow, snow ageing and carbon (the
 * five kernels), with the online energy-balance corrections of soil_snow
 * (cbl_soilsnow_main.F90:164-183) and of cbm_impl (:317-357) applied to
 * out's fe, fh and (with l_rev_corr) rnet and ga, and trad with the
 * correction term (:374-381).  1 <= cycleno <= numcycles; on every cycle but
 * the last the prognostic bank (cbl_prognostic_bank.F90) is restored after
 * the call, as cable_implicit_main.F90:190-213 does, so only the last cycle
 * advances the state.  The offline driver's lakes fix and balance checks do
 * not run in either call (ebal_tot, wbal_tot and owb are left alone).  Both
 * calls use the plain dryLeaf iteration (the surrogate start and the
 * training-row harvest apply to cablegpu_step / cablegpu_run only). */
int cablegpu_step_explicit(cablegpu_ctx* ctx, int ktau, float dels, int lai_refresh);
int cablegpu_step_implicit(cablegpu_ctx* ctx, int ktau, float dels, int cycleno, int numcycles);
/* Timing helper (no counterpart in the reference): nsteps coupled timesteps
 * ktau0.. of cablegpu_step_explicit(lai_refresh = 1) followed by numcycles
 * cablegpu_step_implicit cycles, timed with CUDA events on the context's
 * stream; *ms_total receives the elapsed milliseconds. */
int cablegpu_coupled_timed(cablegpu_ctx* ctx, int ktau0, int nsteps, float dels, int numcycles, float* ms_total);
/* nsteps timesteps ktau0 .. ktau0+nsteps-1, replayed from a captured CUDA
 * graph.  Asynchronous. */
int cablegpu_run(cablegpu_ctx* ctx, int ktau0, int nsteps, float dels);
/* One timestep with host-memory I/O, pipelined: uploads host_forcing
 * ([CABLEGPU_NFORCING][mp] float, as for cablegpu_set_forcing) on a copy
 * stream, runs the step, and downloads the 8 output fluxes (field "out",
 * [8][mp] float) into host_out.  Asynchronous: copies of one step overlap the
 * kernels of its neighbours (two staging slots), so host_forcing must stay
 * unchanged and host_out unread until cablegpu_synchronize; pinned host
 * memory makes the copies asynchronous.  The forcing applies to this step
 * only.  Replaces the per-step get_met_data -> cbm -> write_output sequence
 * of the offline driver (cable_serial.F90:594-640). */
int cablegpu_step_host(cablegpu_ctx* ctx, int ktau, float dels, const float* host_forcing, float* host_out);
/* Page-locks (and releases) an existing host buffer, such as the Fortran
 * shim's forcing and output arrays, so that the copies of
 * cablegpu_step_host run asynchronously at full speed (cudaHostRegister /
 * cudaHostUnregister).  No counterpart in the reference (host I/O). */
int cablegpu_host_register(void* ptr, size_t bytes);
int cablegpu_host_unregister(void* ptr);
/* Allocates bytes of zeroed page-locked host memory for such buffers from
 * the CUDA driver's own pinned allocator (cudaHostAlloc).  On Grace-hosted
 * GB300s the end-to-end step from such buffers ran at 3.0-3.7 ms (against
 * 2.95-3.1 ms device-resident), and from arrays on 64 KB pages page-locked
 * with cablegpu_host_register at 3.7-7.1 ms.  *out receives the address;
 * cablegpu_host_free(ptr) releases it (CABLEGPU_ERR_ARG for an address not
 * from cablegpu_host_alloc).  CABLEGPU_ERR_ARG for bytes == 0 or a null
 * out, CABLEGPU_ERR_CUDA when the allocation fails.  No counterpart in the
 * reference (host I/O). */
int cablegpu_host_alloc(size_t bytes, void** out);
int cablegpu_host_free(void* ptr);
/* Layout of the host buffers of cablegpu_step_host and of the records of
 * cablegpu_run_forcing_file: 0 (default) the caller's tile order, 1 the
 * context's device tile order (cablegpu_tile_order), which spares the kernels
 * the per-step gather and scatter of caller positions and lets the context
 * keep its fastest tile order; a driver fills its arrays through the order
 * index once instead.  Applies to the steps issued after the call. */
int cablegpu_set_host_layout(cablegpu_ctx* ctx, int layout);
/* order_out[s] ([mp]) receives the caller's index of the tile in device
 * slot s. */
int cablegpu_tile_order(cablegpu_ctx* ctx, int* order_out);
/* Waits for all queued work; returns CABLEGPU_ERR_NONFINITE if any step
 * since the last call produced a non-finite output flux.  Which tiles, and
 * what else went wrong where, is in the per-tile field "tile_status" (one
 * byte per tile, read with cablegpu_get_field as int): the kernels OR these
 * bits into it every step and never clear it (the caller clears it with
 * cablegpu_set_field); nothing traps.
 *   CABLEGPU_TILE_NONFINITE       an output flux or the radiative temperature
 *                                 was not finite
 *   CABLEGPU_TILE_DRYLEAF_NOCONV  a dryLeaf iteration ended at its 20-pass
 *                                 limit without meeting its 0.1 K criterion
 *                                 (the best iterate is kept, as the
 *                                 reference does); recorded with
 *                                 diagnostics on
 *   CABLEGPU_TILE_FORCING_RANGE   a forcing value outside the driver's
 *                                 check ranges (SWdown, LWdown, Qair, Rainf,
 *                                 Wind, Tair, PSurf: cable_input.F90:2683-2689,
 *                                 cable_checks.F90:60-70), or not finite
 *   CABLEGPU_TILE_OUTPUT_RANGE    an output outside the reference's output
 *                                 ranges (Qle, Qh, Qg, Rnet, VegT, RadT,
 *                                 SoilTemp: cable_checks.F90:71-123)
 *   CABLEGPU_TILE_EVAPFBL         the condition under which the reference
 *                                 prints 'oldevapfbl not right'
 *                                 (cbl_dryLeaf.F90:626-641) and keeps the
 *                                 latest layer extraction; recorded with
 *                                 diagnostics on */
#define CABLEGPU_TILE_NONFINITE 1
#define CABLEGPU_TILE_DRYLEAF_NOCONV 2
#define CABLEGPU_TILE_FORCING_RANGE 4
#define CABLEGPU_TILE_OUTPUT_RANGE 8
#define CABLEGPU_TILE_EVAPFBL 16
int cablegpu_synchronize(cablegpu_ctx* ctx);

/* Timing helpers for benchmarks: CUDA events on the context's stream.
 * run_timed: total milliseconds of cablegpu_run(ktau0, nsteps).
 * kernel_timed: average milliseconds of one step kernel launch, each launch
 * bracketed by its own events. */
int cablegpu_run_timed(cablegpu_ctx* ctx, int ktau0, int nsteps, float dels, float* ms_total);
int cablegpu_kernel_timed(cablegpu_ctx* ctx, int ktau0, int nsteps, float dels, float* ms_per_launch);
/* phase_timed: average milliseconds of each kernel of a step (radiation,
 * canopy, snow pack, soil heat, soil water, and the surrogate network, 0
 * when it is off), each bracketed by its own events; ms_per_phase has 6
 * elements. */
int cablegpu_phase_timed(cablegpu_ctx* ctx, int ktau0, int nsteps, float dels, float* ms_per_phase);
/* Number of kernel launches of the timestep issued by this context so far:
 * five per step (radiation, canopy, snow pack, soil heat, soil water), plus
 * one single-thread kernel per step that advances the step counter when the
 * steps run as a replayed CUDA graph (cablegpu_run). */
long long cablegpu_launch_count(cablegpu_ctx* ctx);

/* Launch configuration.  set_blocks: threads per block of the five step
 * kernels (radiation, canopy, snow pack, soil heat, soil water), each a
 * multiple of 32 in [32, 256]; results do not depend on them.  get_config:
 * the tile order the context was built with and the current block sizes. */
int cablegpu_set_blocks(cablegpu_ctx* ctx, const int* block5);
int cablegpu_get_config(cablegpu_ctx* ctx, int* order, int* block5);
/* Block sizes tuned on the context itself: times block sizes 32, 64, 128
 * and 256 of each step kernel over `nsteps` steps (1..64) from step ktau0 of
 * length dels on the context's own tiles, current state and forcing source,
 * keeps each kernel's fastest (cablegpu_set_blocks) and returns them and the
 * step time (ms) they give.  The state is copied before the timed steps and
 * put back after each candidate (one temporary device copy of the context's
 * fields), so the context's state, outputs and status are as before the
 * call; results never depend on the block sizes.  Unlike cablegpu_autotune,
 * which times a cold-started sample without snow, this sees the tiles'
 * actual snow layers and soil state.  No counterpart in the reference
 * (scheduling, not physics). */
int cablegpu_tune_blocks(cablegpu_ctx* ctx, int ktau0, int nsteps, float dels, int* block5_out, float* ms_out);
/* Autotuner: times tile orders 0-3 and block sizes 32, 64, 128, 256 of each
 * step kernel on an evenly strided sample of `sample_tiles` of the tiles
 * (synthetic forcing, nsteps timed steps per candidate) and returns the
 * fastest order, the fastest block size of each kernel and the step time
 * (ms) they give on the sample.  cablegpu_create with tiles->order == -1
 * runs it on up to 4,194,304 of the tiles and builds the context with its
 * choice. */
int cablegpu_autotune(const cablegpu_tiles* tiles, int device, int sample_tiles, int nsteps, int* order_out,
                      int* block5_out, float* ms_out);

/* ---- Binary restart, forcing and output files ------------------------------
 * Binary equivalents of the reference's netCDF files: the restart file
 * (cable_output_impl.F90 write_restart :278-311, cable_initialise.F90
 * get_restart_data :163-664), the met file read every step
 * (cable_input.F90 get_met_data) and the per-step output file.  One
 * container, little-endian: a 128-byte header (magic "CABLEGPU", version 1,
 * kind, mp, field and record counts, ktau, doy0, dels, record size), a
 * directory of 48-byte entries (name[32], dtype, width, offset), then from
 * byte 4096 the records, 4096-byte aligned; a record holds every field as
 * one [width][mp] block in caller tile order, 64-byte aligned.
 *   restart: 1 record; the tile description (KIND_PARAM fields), every
 *            prognostic field (KIND_STATE) and the last step's outputs
 *            (KIND_OUTPUT: ga and trad are restart variables of the
 *            reference too), named as the field registry, the
 *            double-FP32 soil water and ice as their exact word pairs
 *            (CABLEGPU_DF32), so a resumed run is bitwise the
 *            uninterrupted one
 *   forcing: one record per step, one field "met" of width
 *            CABLEGPU_NFORCING ([CABLEGPU_NFORCING][mp] float, rows as for
 *            cablegpu_set_forcing)
 *   output:  one record per step, one field "out" ([8][mp] float, the rows of
 *            the field "out") */
#define CABLEGPU_FILE_RESTART 1
#define CABLEGPU_FILE_FORCING 2
#define CABLEGPU_FILE_OUTPUT 3

/* Writes the context's state after step `ktau` to `path`.  Synchronous. */
int cablegpu_restart_write(cablegpu_ctx* ctx, const char* path, int ktau);
/* Loads the prognostic state of a restart file into the context; the file's
 * tiles must be the context's (same mp, iveg and isoilm in the same caller
 * order; CABLEGPU_ERR_ARG otherwise) and hold every prognostic and output
 * field.
 * *ktau (may be NULL) receives the step the file was written after: the
 * run continues with ktau + 1. */
int cablegpu_restart_read(cablegpu_ctx* ctx, const char* path, int* ktau);
/* Writes a forcing file of `nsteps` records from host memory
 * ([nsteps][CABLEGPU_NFORCING][mp] float).  No context or GPU needed. */
int cablegpu_forcing_file_write(const char* path, int mp, int nsteps, int doy0, float dels, const float* forcing);
/* Header of any of the three files (each pointer may be NULL).  No context or
 * GPU needed. */
int cablegpu_file_info(const char* path, int* kind, long long* mp, int* nrecords, int* nfields, int* ktau, int* doy0,
                       float* dels);
/* Runs steps ktau0 .. ktau0+nsteps-1 on the records record0 .. of a forcing
 * file (its dels), through the pipelined host path of cablegpu_step_host: a
 * reader thread fills three pinned buffers from the file ahead of the GPU, and
 * when `output_path` is not NULL a writer thread appends each step's output
 * record to a new output file behind it.  Returns when every step is done and
 * written: the offline driver's time loop (cable_serial.F90:493-738:
 * get_met_data, cbm, cable_output_write) with the file I/O overlapping the
 * steps. */
int cablegpu_run_forcing_file(cablegpu_ctx* ctx, const char* forcing_path, int record0, int ktau0, int nsteps,
                              const char* output_path);

/* Copies a built-in parameter table (no context or GPU needed): table 0 is
 * the per-plant-type table of pft_params.nml with derived entries "dleaf"
 * and "froot" (6 x 17, layer-major), table 1 the per-soil table of
 * cable_soilparm.nml with derived entries (hsbh, ibp2, i2bp3, pwb_min,
 * cnsd, and the soil_thermal_fix inputs cnsdv, ktmp), table 2 the same
 * per-soil table with the soil_thermal_fix parameter set applied (css,
 * rhosoil, cnsd rewritten).  `n` is the capacity of `out`. */
int cablegpu_param_table(int table, const char* name, float* out, int n);

/* ---------------------------------------------------------------- dryLeaf surrogate
 * No counterpart in the reference: a small network (12 inputs -> 64 -> 64 ->
 * 3, SiLU, BF16 tensor-core kernels with FP32 accumulation) that predicts
 * the converged result of the dryLeaf leaf energy-balance / photosynthesis /
 * stomatal-conductance iteration (cbl_dryLeaf.F90:10-666) from the state
 * the iteration starts from.  With the surrogate enabled, each Monin-Obukhov
 * iteration of each vegetated tile runs one dryLeaf pass from the predicted
 * leaf temperature; the tile accepts it when that pass moves the leaf
 * temperature by at most `gate` K (the leaf energy-balance residual of the
 * prediction; the plain iteration itself stops at 0.1 K) and otherwise runs
 * the plain iteration from its usual start, so every accepted tile meets the
 * plain iteration's own convergence test.
 *
 * Inputs (training-row columns 0-11): sunlit and shaded absorbed PAR (W/m2),
 * leaf temperature at entry (K), leaf-surface vapour pressure deficit (Pa),
 * air CO2 (mol/mol), canopy vcmax and C3 jmax (mol/m2/s, scaled by the
 * sunlit+shaded leaf scaling), stomatal slope (a1gs, or g1 under medlyn),
 * soil-moisture stress factor, LAI, wind speed at the reference height
 * (m/s), air temperature (K).  Targets (columns 12-14): stomatal conductance to
 * water (mol/m2/s), net assimilation (mol/m2/s), leaf temperature change
 * over the iteration (K).  Column 15 is unused. */

/* Failure handling: the network kernels wait on the tensor cores with a
 * bounded wait (0.2 s of wall time).  A wait that gives up makes the kernel
 * wait once more (bounded) for the pass it issued, free its tensor memory
 * and return; in a step, every tile then runs the plain dryLeaf iteration
 * and cablegpu_synchronize returns CABLEGPU_ERR_CUDA, and the context-free
 * calls below return CABLEGPU_ERR_CUDA.  Debugging aid: the environment
 * variable CABLEGPU_DEBUG_TC_WAIT_NS, read at each network-kernel launch,
 * lowers the limit of the first waits (0: give up at once without
 * polling), to exercise that path; the final wait keeps its full limit. */

/* Runs nsteps plain steps that also append one training row for each
 * sampled (vegetated tile, Monin-Obukhov iteration), sampled with
 * probability `prob` from a counter-based hash of (tile, step, iteration,
 * seed), into a device buffer of `capacity` rows.  *nrows: rows filled. */
int cablegpu_harvest(cablegpu_ctx* ctx, int ktau0, int nsteps, float dels, float prob, unsigned long long seed,
                     long long capacity, long long* nrows);
/* Copies the first n harvested rows ([n][16] float) to the host. */
int cablegpu_harvest_rows(cablegpu_ctx* ctx, float* host, long long n);
/* Trains a fresh network on the harvested rows with the library's own
 * tensor-core forward/backward kernels and Adam: the last val_frac of the
 * rows are held out; epochs of batches of `batch` rows, one random
 * permutation per epoch.  losses: [epochs][2] mean squared normalised
 * error (train, validation), may be NULL. */
int cablegpu_surrogate_train(cablegpu_ctx* ctx, int epochs, int batch, float lr, float val_frac,
                             unsigned long long seed, float* losses);
/* Get (set = 0) or set (set = 1) the network: params [5187] (W1 [64][12],
 * b1 [64], W2 [64][64], b2 [64], W3 [3][64], b3 [3]) and norm [30] (input
 * mean [12], input 1/sd [12], output mean [3], output sd [3]). */
int cablegpu_surrogate_weights(cablegpu_ctx* ctx, float* params, float* norm, int set);
/* mode 0: surrogate off.  1 (strict): a tile whose prediction does not
 * close within `gate` K restarts the plain iteration from its usual start
 * (its result is bitwise the plain kernel's).  2 (warm): the plain
 * iteration continues from the prediction with `gate` as its convergence
 * test.  gate in (0, 0.1] K.  Each step then runs one more kernel (the
 * network over all tiles, on the tensor cores). */
int cablegpu_set_surrogate(cablegpu_ctx* ctx, int mode, float gate_kelvin);
/* Tiles x Monin-Obukhov iterations that tried the surrogate and that
 * accepted it since the last reset; reset = 1 zeroes the counters. */
int cablegpu_surrogate_stats(cablegpu_ctx* ctx, long long* tried, long long* accepted, int reset);

/* Context-free network kernels on host arrays (rows in the training-row
 * layout above): forward pass (y [n][3], raw units), loss and gradient of
 * the mean squared normalised error (grad [5187]), and training of a fresh
 * network on rows [0, ntrain) validated on [ntrain, ntrain + nval). */
int cablegpu_mlp_sizes(int* nparam, int* nnorm, int* row);
int cablegpu_mlp_forward(const float* params, const float* norm, const float* rows, long long n, float* y);
int cablegpu_mlp_grad(const float* params, const float* norm, const float* rows, long long n, float* grad,
                      float* loss);
int cablegpu_mlp_fit(const float* rows, long long ntrain, long long nval, int epochs, int batch, float lr,
                     unsigned long long seed, float* params_out, float* norm_out, float* losses);
const char* cablegpu_mlp_last_error(void);

/* Checks one per-tile veg or soil parameter of the driver (the arrays
 * init_veg_from_vegin and derived_parameters fill per tile,
 * cable_parameters.F90:3277-3345, :1759-2343; host array [mp] float in the
 * caller's order, [6][mp] for "froot") against the value the kernels use for
 * each tile: the built-in table entry of its plant type (iveg) or soil type
 * (isoilm), as cablegpu_param_table gives them (the soil_thermal_fix set when
 * that switch is on).  Returns CABLEGPU_ERR_ARG, naming the first tile that
 * differs by more than 1e-6 relative in cablegpu_last_error, so a driver
 * whose per-tile parameters depart from the reference's tables is refused
 * rather than run with the tables.  name: an entry of cablegpu_param_table
 * table 0 or 1.  The bare-soil albedo is per tile on the device (field
 * "albsoil") and needs no check. */
int cablegpu_check_tile_param(cablegpu_ctx* ctx, const char* name, const float* host_values);

const char* cablegpu_last_error(cablegpu_ctx* ctx);

#ifdef __cplusplus
}
#endif
#endif /* CABLEGPU_H */
