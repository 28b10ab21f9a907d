!==============================================================================
! cable_cbm_coupled_gpu.F90 - drop-in replacement of the ACCESS (CM3)
! MODULE cable_cbm_module (src/coupled/AM3/control/cable/CM3/cbl_cbm_mod.F90)
! that runs its two calls on the GPU through the C ABI of include/cablegpu.h:
!     CALL cbm_expl(mp, nrb, ktau, dels, air, bgc, canopy, met, bal, rad,  &
!                   rough, soil, ssnow, sum_flux, veg, climate)
!     (cable_explicit_driver.F90:266)
!     CALL cbm_impl(cycleno, numcycles, mp, nrb, ktau, dels, air, bgc,     &
!                   canopy, met, bal, rad, rough, soil, ssnow, sum_flux,   &
!                   veg, climate)
!     (cable_implicit_driver.F90:200)
! The first call creates the device context and uploads the tiles and the
! prognostic state (cablegpu_shim.F90).  Every call uploads the met fields
! the host model set for it (the implicit driver's updated air temperature
! and humidity included, cable_implicit_driver.F90:189-198) and canopy%vlaiw,
! which the host model's radiation call computed and update_canopy copied
! (cbl_um_update_canopy.F90:27); it then runs the call and copies the
! fluxes back.  The prognostic state stays on the device: the implicit
! call's prognostic bank for cycles other than the last
! (cable_implicit_main.F90:190-213) is kept there too.  Call
! cbm_gpu_state_to_host before the host model reads CABLE's prognostics
! back (implicit_unpack) or writes a dump, and cbm_gpu_finalize at the end.
!
! Build: compile cablegpu_c.F90, cablegpu_shim.F90 and this file in place of
! cbl_cbm_mod.F90 and link cable_gb300/lib/libcablegpu.so.  Science switches
! as for the offline replacement (cable_cbm_gpu.F90).
!==============================================================================

MODULE cable_cbm_module
  USE, INTRINSIC :: iso_c_binding
  USE cablegpu_c
  USE cablegpu_shim
  IMPLICIT NONE

  PRIVATE
  PUBLIC cbm_expl, cbm_impl, cbm_gpu_state_to_host, cbm_gpu_finalize

CONTAINS

  ! The met fields of this call and the radiation call's canopy%vlaiw, in
  ! the caller's tile order.
  SUBROUTINE upload_call_inputs(met, canopy)
    USE cable_def_types_mod
    TYPE(met_type), INTENT(IN) :: met
    TYPE(canopy_type), INTENT(IN) :: canopy
    REAL(c_float), ALLOCATABLE, TARGET :: r4(:, :)

    forc(:, 1) = met%fsd(:, 1)
    forc(:, 2) = met%fsd(:, 2)
    forc(:, 3) = met%fld
    forc(:, 4) = met%precip
    forc(:, 5) = met%precip_sn
    forc(:, 6) = met%tk
    forc(:, 7) = met%pmb
    forc(:, 8) = met%ua
    forc(:, 9) = met%qv
    forc(:, 10) = met%ca
    forc(:, 11) = met%coszen
    forc(:, 12) = met%doy
    forc(:, 13) = met%hod
    CALL check(cablegpu_set_forcing(ctx, C_LOC(forc)), 'set_forcing')
    ALLOCATE(r4(mp, 1))
    r4(:, 1) = canopy%vlaiw; CALL put('vlaiw', C_LOC(r4))
    DEALLOCATE(r4)
  END SUBROUTINE upload_call_inputs

  ! The call's fluxes back into the derived types (waits for the call; its
  ! errors surface here).
  SUBROUTINE download_outputs(canopy, rad)
    USE cable_def_types_mod
    TYPE(canopy_type), INTENT(INOUT) :: canopy
    TYPE(radiation_type), INTENT(INOUT) :: rad

    CALL check(cablegpu_synchronize(ctx), 'synchronize')
    CALL get('out', C_LOC(outb))
    canopy%fe = outb(:, 1)
    canopy%fh = outb(:, 2)
    canopy%fgpp = outb(:, 3)
    canopy%frday = outb(:, 4)
    canopy%tv = outb(:, 5)
    canopy%rnet = outb(:, 6)
    canopy%ga = outb(:, 7)
    rad%trad = outb(:, 8)
  END SUBROUTINE download_outputs

  SUBROUTINE cbm_expl(mp, nrb, ktau, dels, air, bgc, canopy, met, bal, rad, rough, soil, ssnow, sum_flux, veg, &
                      climate)
    USE cable_def_types_mod, ONLY : air_type, bgc_pool_type, canopy_type, met_type, balances_type,         &
                                    radiation_type, roughness_type, soil_snow_type, sum_flux_type,           &
                                    soil_parameter_type, veg_parameter_type, climate_type
    INTEGER, INTENT(IN) :: mp, nrb, ktau
    REAL, INTENT(IN) :: dels
    TYPE(air_type), INTENT(INOUT) :: air
    TYPE(bgc_pool_type), INTENT(INOUT) :: bgc
    TYPE(canopy_type), INTENT(INOUT) :: canopy
    TYPE(met_type), INTENT(INOUT) :: met
    TYPE(balances_type), INTENT(INOUT) :: bal
    TYPE(radiation_type), INTENT(INOUT) :: rad
    TYPE(roughness_type), INTENT(INOUT) :: rough
    TYPE(soil_parameter_type), INTENT(INOUT) :: soil
    TYPE(soil_snow_type), INTENT(INOUT) :: ssnow
    TYPE(sum_flux_type), INTENT(INOUT) :: sum_flux
    TYPE(veg_parameter_type), INTENT(INOUT) :: veg
    TYPE(climate_type) :: climate

    IF (.NOT. C_ASSOCIATED(ctx)) CALL gpu_setup(bal, bgc, canopy, rad, soil, ssnow, veg)
    IF (mp /= mp_gpu) STOP 'cablegpu: mp changed between calls'
    CALL upload_call_inputs(met, canopy)
    ! canopy%vlaiw was uploaded, so no recomputation (lai_refresh = 0)
    CALL check(cablegpu_step_explicit(ctx, INT(ktau, c_int), REAL(dels, c_float), 0_c_int), 'step_explicit')
    CALL download_outputs(canopy, rad)
  END SUBROUTINE cbm_expl

  SUBROUTINE cbm_impl(cycleno, numcycles, mp, nrb, ktau, dels, air, bgc, canopy, met, bal, rad, rough, soil, &
                      ssnow, sum_flux, veg, climate)
    USE cable_def_types_mod, ONLY : air_type, bgc_pool_type, canopy_type, met_type, balances_type,         &
                                    radiation_type, roughness_type, soil_snow_type, sum_flux_type,           &
                                    soil_parameter_type, veg_parameter_type, climate_type
    INTEGER, INTENT(IN) :: cycleno, numcycles, mp, nrb, ktau
    REAL, INTENT(IN) :: dels
    TYPE(air_type), INTENT(INOUT) :: air
    TYPE(bgc_pool_type), INTENT(INOUT) :: bgc
    TYPE(canopy_type), INTENT(INOUT) :: canopy
    TYPE(met_type), INTENT(INOUT) :: met
    TYPE(balances_type), INTENT(INOUT) :: bal
    TYPE(radiation_type), INTENT(INOUT) :: rad
    TYPE(roughness_type), INTENT(INOUT) :: rough
    TYPE(soil_parameter_type), INTENT(INOUT) :: soil
    TYPE(soil_snow_type), INTENT(INOUT) :: ssnow
    TYPE(sum_flux_type), INTENT(INOUT) :: sum_flux
    TYPE(veg_parameter_type), INTENT(INOUT) :: veg
    TYPE(climate_type) :: climate

    IF (.NOT. C_ASSOCIATED(ctx)) CALL gpu_setup(bal, bgc, canopy, rad, soil, ssnow, veg)
    IF (mp /= mp_gpu) STOP 'cablegpu: mp changed between calls'
    CALL upload_call_inputs(met, canopy)
    CALL check(cablegpu_step_implicit(ctx, INT(ktau, c_int), REAL(dels, c_float), INT(cycleno, c_int), &
                                      INT(numcycles, c_int)), 'step_implicit')
    CALL download_outputs(canopy, rad)
  END SUBROUTINE cbm_impl

END MODULE cable_cbm_module
