!==============================================================================
! cable_cbm_gpu.F90 - drop-in replacement of the offline MODULE
! cable_cbm_module (src/offline/cbl_model_driver_offline.F90:29-231) that runs
! the per-timestep tile physics on the GPU through the C ABI declared in
! include/cablegpu.h.
!
! The offline driver keeps calling
!     CALL cbm(ktau, dels, air, bgc, canopy, met, bal, rad, rough, soil,  &
!              ssnow, sum_flux, veg, climate, xk, c1, rhoch)
! (src/offline/cable_serial.F90:594-595, cable_mpiworker.F90:503) with the
! same derived types.  On the first call this module creates a device
! context for the mp tiles, uploads the tile description (veg%iveg,
! soil%isoilm, veg%vlai, rad%latitude) and the prognostic state the driver
! initialised (defaults or restart file), after checking the per-tile veg
! and soil parameters against the per-type tables the kernels use.  Every
! call then uploads that step's met forcing, advances the device state by one
! step and copies back into the derived types everything the driver reads
! before its next call: the eight output fluxes (canopy%fe, fh, fgpp, frday,
! tv, rnet, ga, rad%trad), the runoff and melt rates, screen temperature,
! carbon fluxes, energy and water terms, balances and the soil and snow
! profiles (driver_fields_to_host).  The rest of the prognostic state stays
! on the device; call cbm_gpu_state_to_host before writing a restart file
! and cbm_gpu_finalize at the end of the run.
!
! Build: compile cablegpu_c.F90, cablegpu_shim.F90 and this file in place of
! cbl_model_driver_offline.F90 and link cable_gb300/lib/libcablegpu.so.
! soil_struc 'default' with the science switches gs_switch, fwsoil_switch
! ('standard', 'non-linear extrapolation', 'Lai and Ktaul 2000'),
! ssnow_potev ('HDM', 'P-M'), soil_thermal_fix, litter, l_rev_corr,
! l_new_reduce_soilevp, l_new_runoff_speed and diag_soil_resp; other
! configurations stay on the CPU path of the reference.
!==============================================================================

MODULE cable_cbm_module
  USE, INTRINSIC :: iso_c_binding
  USE cablegpu_c
  USE cablegpu_shim
  IMPLICIT NONE

  PRIVATE
  PUBLIC cbm, cbm_gpu_state_to_host, cbm_gpu_finalize

CONTAINS

  SUBROUTINE cbm(ktau, dels, air, bgc, canopy, met, bal, rad, rough, soil, ssnow, sum_flux, veg, climate, xk, c1, &
                 rhoch)
    USE cable_def_types_mod
    TYPE(air_type), INTENT(INOUT) :: air
    TYPE(bgc_pool_type), INTENT(INOUT) :: bgc
    TYPE(canopy_type), INTENT(INOUT) :: canopy
    TYPE(met_type), INTENT(INOUT) :: met
    TYPE(balances_type), INTENT(INOUT) :: bal
    TYPE(radiation_type), INTENT(INOUT) :: rad
    TYPE(roughness_type), INTENT(INOUT) :: rough
    TYPE(soil_snow_type), INTENT(INOUT) :: ssnow
    TYPE(sum_flux_type), INTENT(INOUT) :: sum_flux
    TYPE(climate_type), INTENT(IN) :: climate
    TYPE(soil_parameter_type), INTENT(INOUT) :: soil
    TYPE(veg_parameter_type), INTENT(INOUT) :: veg
    REAL, INTENT(IN) :: dels
    INTEGER, INTENT(IN) :: ktau
    REAL :: c1(mp, nrb), rhoch(mp, nrb), xk(mp, nrb)

    IF (.NOT. C_ASSOCIATED(ctx)) CALL gpu_setup(bal, bgc, canopy, rad, soil, ssnow, veg)
    IF (mp /= mp_gpu) STOP 'cablegpu: mp changed between calls'

    ! met_type fields get_met_data filled for this step (cable_input.F90),
    ! gathered into device order
    forc(:, 1) = met%fsd(slot_tile, 1)
    forc(:, 2) = met%fsd(slot_tile, 2)
    forc(:, 3) = met%fld(slot_tile)
    forc(:, 4) = met%precip(slot_tile)
    forc(:, 5) = met%precip_sn(slot_tile)
    forc(:, 6) = met%tk(slot_tile)
    forc(:, 7) = met%pmb(slot_tile)
    forc(:, 8) = met%ua(slot_tile)
    forc(:, 9) = met%qv(slot_tile)
    forc(:, 10) = met%ca(slot_tile)
    forc(:, 11) = met%coszen(slot_tile)
    forc(:, 12) = met%doy(slot_tile)
    forc(:, 13) = met%hod(slot_tile)
    ! one step with the forcing upload and the output download; the driver
    ! writes the fluxes after every step, so wait for them (errors of the
    ! step surface here)
    CALL check(cablegpu_step_host(ctx, INT(ktau, c_int), REAL(dels, c_float), C_LOC(forc), C_LOC(outb)), &
               'step_host')
    CALL check(cablegpu_synchronize(ctx), 'synchronize')
    canopy%fe(slot_tile) = outb(:, 1)
    canopy%fh(slot_tile) = outb(:, 2)
    canopy%fgpp(slot_tile) = outb(:, 3)
    canopy%frday(slot_tile) = outb(:, 4)
    canopy%tv(slot_tile) = outb(:, 5)
    canopy%rnet(slot_tile) = outb(:, 6)
    canopy%ga(slot_tile) = outb(:, 7)
    rad%trad(slot_tile) = outb(:, 8)
    ! everything else the driver reads before the next call
    CALL driver_fields_to_host(dels, bal, canopy, rad, ssnow)
  END SUBROUTINE cbm

END MODULE cable_cbm_module
