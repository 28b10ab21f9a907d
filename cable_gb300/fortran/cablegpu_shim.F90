!==============================================================================
! cablegpu_shim.F90 - what the offline and the coupled replacements of
! cable_cbm_module share: the device context, the first-call set-up (tiles,
! science switches, the driver's initial prognostic state), the copy of the
! device state back into the derived types, and the clean-up.
!==============================================================================

MODULE cablegpu_shim
  USE, INTRINSIC :: iso_c_binding
  USE cablegpu_c
  IMPLICIT NONE

  PUBLIC

  TYPE(c_ptr), SAVE :: ctx = c_null_ptr
  INTEGER, SAVE :: mp_gpu = 0
  REAL(c_float), ALLOCATABLE, TARGET, SAVE :: forc(:, :)   ! (mp, 13)
  REAL(c_float), ALLOCATABLE, TARGET, SAVE :: outb(:, :)   ! (mp, 8)
  ! caller tile (1-based) of each device slot: the per-step forcing and
  ! outputs move in device order (cablegpu_set_host_layout), gathered and
  ! scattered through this index on the host
  INTEGER(c_int), ALLOCATABLE, TARGET, SAVE :: slot_tile(:)

CONTAINS

  SUBROUTINE check(rc, what)
    INTEGER(c_int), INTENT(IN) :: rc
    CHARACTER(LEN=*), INTENT(IN) :: what
    CHARACTER(KIND=c_char), POINTER :: msg(:)
    INTEGER :: n
    IF (rc == 0) RETURN
    WRITE(*, *) 'cablegpu: ', what, ' failed with code ', rc
    IF (C_ASSOCIATED(ctx)) THEN
      CALL C_F_POINTER(cablegpu_last_error(ctx), msg, [512])
      n = 0
      DO WHILE (n < 512)
        IF (msg(n + 1) == c_null_char) EXIT
        n = n + 1
      END DO
      WRITE(*, *) 'cablegpu: ', msg(1:n)
    END IF
    STOP 'cablegpu error'
  END SUBROUTINE check

  SUBROUTINE put(name, p)
    CHARACTER(LEN=*), INTENT(IN) :: name
    TYPE(c_ptr), INTENT(IN) :: p
    CALL check(cablegpu_set_field(ctx, fid(name), p), 'set_field ' // name)
  END SUBROUTINE put

  SUBROUTINE get(name, p)
    CHARACTER(LEN=*), INTENT(IN) :: name
    TYPE(c_ptr), INTENT(IN) :: p
    CALL check(cablegpu_get_field(ctx, fid(name), p), 'get_field ' // name)
  END SUBROUTINE get

  ! First call: context, tile description and the driver's initial state.
  SUBROUTINE gpu_setup(bal, bgc, canopy, rad, soil, ssnow, veg)
    USE cable_def_types_mod
    USE cable_runtime_opts_mod, ONLY : cable_user
    TYPE(balances_type), INTENT(IN) :: bal
    TYPE(bgc_pool_type), INTENT(IN) :: bgc
    TYPE(canopy_type), INTENT(IN) :: canopy
    TYPE(radiation_type), INTENT(IN) :: rad
    TYPE(soil_parameter_type), INTENT(IN) :: soil
    TYPE(soil_snow_type), INTENT(IN) :: ssnow
    TYPE(veg_parameter_type), INTENT(IN) :: veg
    TYPE(cablegpu_tiles) :: tiles
    INTEGER(c_int), ALLOCATABLE, TARGET :: iveg(:), isoilm(:), flags(:)
    REAL(c_float), ALLOCATABLE, TARGET :: vlai(:), lat(:), r4(:, :)
    REAL(c_double), ALLOCATABLE, TARGET :: r8(:, :)
    INTEGER(c_int) :: switches

    mp_gpu = mp
    ALLOCATE(iveg(mp), isoilm(mp), vlai(mp), lat(mp), flags(mp))
    iveg = veg%iveg
    isoilm = soil%isoilm
    vlai = veg%vlai
    lat = rad%latitude
    tiles%mp = mp
    tiles%iveg = C_LOC(iveg)
    tiles%isoilm = C_LOC(isoilm)
    tiles%vlai = C_LOC(vlai)
    tiles%lat = C_LOC(lat)
    tiles%lonphase = c_null_ptr
    tiles%tbase = c_null_ptr
    tiles%swscale = c_null_ptr
    tiles%order = 0
    CALL check(cablegpu_create(tiles, 0_c_int, ctx), 'create')
    ! science switch bits (CABLEGPU_SW_* in cablegpu.h)
    switches = 0
    IF (TRIM(cable_user%gs_switch) == 'medlyn') switches = switches + 1
    IF (cable_user%soil_thermal_fix) switches = switches + 2
    IF (cable_user%litter) switches = switches + 4
    IF (cable_user%l_rev_corr) switches = switches + 8
    IF (TRIM(cable_user%fwsoil_switch) == 'non-linear extrapolation') switches = switches + 16
    IF (TRIM(cable_user%fwsoil_switch) == 'Lai and Ktaul 2000') switches = switches + 32
    IF (TRIM(cable_user%ssnow_potev) == 'P-M') switches = switches + 64
    IF (cable_user%l_new_reduce_soilevp) switches = switches + 128
    IF (cable_user%l_new_runoff_speed) switches = switches + 256
    IF (TRIM(cable_user%diag_soil_resp) == 'OFF' .OR. TRIM(cable_user%diag_soil_resp) == 'off') &
      switches = switches + 512
    CALL check(cablegpu_set_options(ctx, switches, 0_c_int, 0_c_int), 'set_options')
    CALL check(cablegpu_set_host_layout(ctx, 1_c_int), 'set_host_layout')
    ALLOCATE(slot_tile(mp))
    CALL check(cablegpu_tile_order(ctx, C_LOC(slot_tile)), 'tile_order')
    slot_tile = slot_tile + 1

    ! prognostic state (soil_snow_type, canopy, bgc, bal)
    ALLOCATE(r8(mp, ms), r4(mp, ms))
    r8 = ssnow%wb;    CALL put('wb', C_LOC(r8))
    r8 = ssnow%wbice; CALL put('wbice', C_LOC(r8))
    r4 = ssnow%tgg;   CALL put('tgg', C_LOC(r4))
    r8(:, 1) = ssnow%gammzz(:, 1); CALL put('gammzz1', C_LOC(r8))
    r4(:, 1:msn) = ssnow%tggsn;  CALL put('tggsn', C_LOC(r4))
    r4(:, 1:msn) = ssnow%ssdn;   CALL put('ssdn', C_LOC(r4))
    r4(:, 1:msn) = ssnow%smass;  CALL put('smass', C_LOC(r4))
    r4(:, 1:msn) = ssnow%sdepth; CALL put('sdepth', C_LOC(r4))
    ! bit 0: isflag; bit 1: soil_snow's first call of the run is pending
    ! (its SAVEd call counter, cbl_soilsnow_main.F90:60-62, 92-96)
    flags = ssnow%isflag + 2
    CALL put('flags', C_LOC(flags))
    r4(:, 1) = ssnow%snowd;   CALL put('snowd', C_LOC(r4))
    r4(:, 1) = ssnow%ssdnn;   CALL put('ssdnn', C_LOC(r4))
    r4(:, 1) = ssnow%snage;   CALL put('snage', C_LOC(r4))
    r4(:, 1) = ssnow%pudsto;  CALL put('pudsto', C_LOC(r4))
    r4(:, 1) = ssnow%owetfac; CALL put('owetfac', C_LOC(r4))
    r4(:, 1) = ssnow%rtsoil;  CALL put('rtsoil', C_LOC(r4))
    r4(:, 1) = ssnow%tss;     CALL put('tss', C_LOC(r4))
    r4(:, 1) = ssnow%wb_lake; CALL put('wb_lake', C_LOC(r4))
    r4(:, 1) = ssnow%wbtot1;  CALL put('wbtot1', C_LOC(r4))
    r4(:, 1) = ssnow%wbtot2;  CALL put('wbtot2', C_LOC(r4))
    r4(:, 1) = canopy%cansto; CALL put('cansto', C_LOC(r4))
    r4(:, 1:3) = bgc%cplant;  CALL put('cplant', C_LOC(r4))
    r4(:, 1:2) = bgc%csoil;   CALL put('csoil', C_LOC(r4))
    r8(:, 1) = bal%ebal_tot;  CALL put('ebal_tot', C_LOC(r8))
    r8(:, 1) = bal%wbal_tot;  CALL put('wbal_tot', C_LOC(r8))
    ! mass_balance's SAVEd previous total (cable_checks.F90:496-513) is
    ! re-initialised by the step at ktau = 1; zero otherwise
    r8(:, 1) = 0.0_c_double;  CALL put('owb', C_LOC(r8))

    ALLOCATE(forc(mp, CABLEGPU_NFORCING), outb(mp, 8))
    DEALLOCATE(iveg, isoilm, vlai, lat, flags, r8, r4)
  END SUBROUTINE gpu_setup

  ! Copies the device-resident prognostic state back into the derived types
  ! (before a restart write, cable_output.F90 / create_restart).
  SUBROUTINE cbm_gpu_state_to_host(bal, bgc, canopy, ssnow)
    USE cable_def_types_mod
    TYPE(balances_type), INTENT(INOUT) :: bal
    TYPE(bgc_pool_type), INTENT(INOUT) :: bgc
    TYPE(canopy_type), INTENT(INOUT) :: canopy
    TYPE(soil_snow_type), INTENT(INOUT) :: ssnow
    REAL(c_float), ALLOCATABLE, TARGET :: r4(:, :)
    REAL(c_double), ALLOCATABLE, TARGET :: r8(:, :)
    INTEGER(c_int), ALLOCATABLE, TARGET :: flags(:)

    IF (.NOT. C_ASSOCIATED(ctx)) RETURN
    CALL check(cablegpu_synchronize(ctx), 'synchronize')
    ALLOCATE(r8(mp, ms), r4(mp, ms), flags(mp))
    CALL get('wb', C_LOC(r8));    ssnow%wb = r8
    CALL get('wbice', C_LOC(r8)); ssnow%wbice = r8
    CALL get('tgg', C_LOC(r4));   ssnow%tgg = r4
    CALL get('gammzz1', C_LOC(r8)); ssnow%gammzz(:, 1) = r8(:, 1)
    CALL get('tggsn', C_LOC(r4));  ssnow%tggsn = r4(:, 1:msn)
    CALL get('ssdn', C_LOC(r4));   ssnow%ssdn = r4(:, 1:msn)
    CALL get('smass', C_LOC(r4));  ssnow%smass = r4(:, 1:msn)
    CALL get('sdepth', C_LOC(r4)); ssnow%sdepth = r4(:, 1:msn)
    CALL get('flags', C_LOC(flags)); ssnow%isflag = IAND(flags, 1)
    CALL get('snowd', C_LOC(r4));   ssnow%snowd = r4(:, 1)
    CALL get('ssdnn', C_LOC(r4));   ssnow%ssdnn = r4(:, 1)
    CALL get('snage', C_LOC(r4));   ssnow%snage = r4(:, 1)
    CALL get('pudsto', C_LOC(r4));  ssnow%pudsto = r4(:, 1)
    CALL get('owetfac', C_LOC(r4)); ssnow%owetfac = r4(:, 1)
    CALL get('rtsoil', C_LOC(r4));  ssnow%rtsoil = r4(:, 1)
    CALL get('tss', C_LOC(r4));     ssnow%tss = r4(:, 1)
    CALL get('wb_lake', C_LOC(r4)); ssnow%wb_lake = r4(:, 1)
    CALL get('cansto', C_LOC(r4));  canopy%cansto = r4(:, 1)
    CALL get('cplant', C_LOC(r4));  bgc%cplant = r4(:, 1:3)
    CALL get('csoil', C_LOC(r4));   bgc%csoil = r4(:, 1:2)
    CALL get('ebal_tot', C_LOC(r8)); bal%ebal_tot = REAL(r8(:, 1))
    CALL get('wbal_tot', C_LOC(r8)); bal%wbal_tot = REAL(r8(:, 1))
    DEALLOCATE(r8, r4, flags)
  END SUBROUTINE cbm_gpu_state_to_host

  SUBROUTINE cbm_gpu_finalize()
    IF (C_ASSOCIATED(ctx)) CALL check(cablegpu_destroy(ctx), 'destroy')
    ctx = c_null_ptr
    IF (ALLOCATED(forc)) DEALLOCATE(forc)
    IF (ALLOCATED(outb)) DEALLOCATE(outb)
    IF (ALLOCATED(slot_tile)) DEALLOCATE(slot_tile)
  END SUBROUTINE cbm_gpu_finalize

END MODULE cablegpu_shim
