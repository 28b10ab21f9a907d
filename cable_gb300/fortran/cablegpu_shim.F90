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
  ! Copy-back after each step: .TRUE. (default) copies every field the
  ! offline driver reads; a driver may set it to .FALSE. on steps where it
  ! neither writes output nor runs its own mass / energy balance checks,
  ! and then only the fields it uses every step come back (runoff and melt,
  ! screen temperature and humidity, the carbon fluxes, the balances).
  LOGICAL, SAVE :: cbm_gpu_copy_all = .TRUE.
  INTEGER, SAVE :: mp_gpu = 0
  ! the per-step forcing and output buffers, in page-locked host memory
  ! from cablegpu_host_alloc (the CUDA driver's pinned allocator: steadier
  ! end-to-end steps than registering ALLOCATE-d arrays)
  REAL(c_float), POINTER, SAVE :: forc(:, :) => NULL()   ! (mp, 13)
  REAL(c_float), POINTER, SAVE :: outb(:, :) => NULL()   ! (mp, 8)
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
    TYPE(c_ptr) :: pbuf
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
    ! diagnostics on: the fields the driver reads after cbm() beyond the
    ! eight output fluxes (driver_fields_to_host) are diagnostics fields
    CALL check(cablegpu_set_options(ctx, switches, 1_c_int, 0_c_int), 'set_options')
    ! the kernels take the veg and soil parameters from per-type tables:
    ! refuse per-tile values that differ from them
    CALL check_params(soil, veg)
    CALL check(cablegpu_set_host_layout(ctx, 1_c_int), 'set_host_layout')
    ALLOCATE(slot_tile(mp))
    CALL check(cablegpu_tile_order(ctx, C_LOC(slot_tile)), 'tile_order')
    slot_tile = slot_tile + 1

    ! prognostic state (soil_snow_type, canopy, bgc, bal)
    ALLOCATE(r8(mp, ms), r4(mp, ms))
    ! the per-tile bare-soil albedo (VIS, soil%albsoil(:,1)) of the gridded
    ! soil file
    r4(:, 1) = soil%albsoil(:, 1); CALL put('albsoil', C_LOC(r4))
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

    ! page-locked, so that each step's forcing upload and flux download are
    ! asynchronous copies at full speed
    CALL check(cablegpu_host_alloc(INT(4, c_size_t) * mp * CABLEGPU_NFORCING, pbuf), 'host_alloc forc')
    CALL C_F_POINTER(pbuf, forc, [mp, CABLEGPU_NFORCING])
    CALL check(cablegpu_host_alloc(INT(4, c_size_t) * mp * 8, pbuf), 'host_alloc outb')
    CALL C_F_POINTER(pbuf, outb, [mp, 8])
    DEALLOCATE(iveg, isoilm, vlai, lat, flags, r8, r4)
  END SUBROUTINE gpu_setup

  ! One per-tile parameter against the library's per-type tables.
  SUBROUTINE check_one(name, values)
    CHARACTER(LEN=*), INTENT(IN) :: name
    REAL, INTENT(IN) :: values(:)
    REAL(c_float), ALLOCATABLE, TARGET :: v(:)
    ALLOCATE(v(SIZE(values)))
    v = values
    CALL check(cablegpu_check_tile_param(ctx, TRIM(name) // c_null_char, C_LOC(v)), 'check_tile_param ' // name)
    DEALLOCATE(v)
  END SUBROUTINE check_one

  ! The veg and soil parameters the kernels take from per-type tables
  ! (init_veg_from_vegin and derived_parameters fill them per tile,
  ! cable_parameters.F90:3277-3345, :1759-2343): each must equal its type's
  ! table value, or the run stops with the tile that differs.
  SUBROUTINE check_params(soil, veg)
    USE cable_def_types_mod
    TYPE(soil_parameter_type), INTENT(IN) :: soil
    TYPE(veg_parameter_type), INTENT(IN) :: veg
    INTEGER :: k
    CALL check_one('canst1', veg%canst1); CALL check_one('dleaf', veg%dleaf); CALL check_one('ejmax', veg%ejmax)
    CALL check_one('frac4', veg%frac4);   CALL check_one('hc', veg%hc);       CALL check_one('vbeta', veg%vbeta)
    CALL check_one('rp20', veg%rp20);     CALL check_one('vegcf', veg%vegcf); CALL check_one('extkn', veg%extkn)
    CALL check_one('a1gs', veg%a1gs);     CALL check_one('d0gs', veg%d0gs);   CALL check_one('alpha', veg%alpha)
    CALL check_one('convex', veg%convex); CALL check_one('cfrd', veg%cfrd);   CALL check_one('gswmin', veg%gswmin)
    CALL check_one('conkc0', veg%conkc0); CALL check_one('conko0', veg%conko0); CALL check_one('ekc', veg%ekc)
    CALL check_one('eko', veg%eko);       CALL check_one('g0', veg%g0);       CALL check_one('g1', veg%g1)
    CALL check_one('vcmax', veg%vcmax);   CALL check_one('xfang', veg%xfang); CALL check_one('shelrb', veg%shelrb)
    CALL check_one('refl1', veg%refl(:, 1)); CALL check_one('refl2', veg%refl(:, 2))
    CALL check_one('taul1', veg%taul(:, 1)); CALL check_one('taul2', veg%taul(:, 2))
    CALL check_one('froot', [(veg%froot(:, k), k = 1, ms)])
    CALL check_one('bch', soil%bch);     CALL check_one('css', soil%css);     CALL check_one('hyds', soil%hyds)
    CALL check_one('rhosoil', soil%rhosoil); CALL check_one('sfc', soil%sfc); CALL check_one('ssat', soil%ssat)
    CALL check_one('sucs', soil%sucs);   CALL check_one('swilt', soil%swilt); CALL check_one('cnsd', soil%cnsd)
    CALL check_one('hsbh', soil%hsbh);   CALL check_one('ibp2', soil%ibp2);   CALL check_one('i2bp3', soil%i2bp3)
    CALL check_one('pwb_min', soil%pwb_min)
  END SUBROUTINE check_params

  ! After each step: every field the offline driver reads from the derived
  ! types before its next cbm() call (cable_serial.F90:594-740): the runoff
  ! and melt rates it rescales by dels (:602-605), the screen temperature
  ! and humidity (:607-608), the carbon fluxes of sumcflux (:713), the
  ! energy and water fluxes, stores and balances of mass_balance /
  ! energy_balance (:725-728; the device runs both checks, so bal%ebal,
  ! wbal and their totals come back and check%mass_bal / check%energy_bal can
  ! stay off) and what the output writer accumulates (:734-738): fluxes,
  ! temperatures, the soil profiles and the snow.  The diagnostics fields hold
  ! amounts of the step (mm) where the reference holds rates (mm/s).
  SUBROUTINE driver_fields_to_host(dels, bal, canopy, rad, ssnow)
    USE cable_def_types_mod
    REAL, INTENT(IN) :: dels
    TYPE(balances_type), INTENT(INOUT) :: bal
    TYPE(canopy_type), INTENT(INOUT) :: canopy
    TYPE(radiation_type), INTENT(INOUT) :: rad
    TYPE(soil_snow_type), INTENT(INOUT) :: ssnow
    REAL(c_float), ALLOCATABLE, TARGET :: r4(:, :)
    REAL(c_double), ALLOCATABLE, TARGET :: r8(:, :)
    INTEGER(c_int), ALLOCATABLE, TARGET :: flags(:)
    ALLOCATE(r8(mp, ms), r4(mp, ms), flags(mp))
    ! every step: the rates the driver rescales, the screen temperature of
    ! its daily extremes, sumcflux's carbon fluxes and the balances
    CALL get('runoff', C_LOC(r4)); ssnow%runoff = r4(:, 1) / dels
    CALL get('rnof1', C_LOC(r4));  ssnow%rnof1 = r4(:, 1) / dels
    CALL get('rnof2', C_LOC(r4));  ssnow%rnof2 = r4(:, 1) / dels
    CALL get('smelt', C_LOC(r4));  ssnow%smelt = r4(:, 1) / dels
    CALL get('tscrn', C_LOC(r4));  canopy%tscrn = r4(:, 1)
    CALL get('qscrn', C_LOC(r4));  canopy%qscrn = r4(:, 1)
    CALL get('fpn', C_LOC(r4));    canopy%fpn = r4(:, 1)
    CALL get('fnpp', C_LOC(r4));   canopy%fnpp = r4(:, 1)
    CALL get('fnee', C_LOC(r4));   canopy%fnee = r4(:, 1)
    CALL get('fra', C_LOC(r4));    canopy%fra = r4(:, 1)
    CALL get('frp', C_LOC(r4));    canopy%frp = r4(:, 1)
    CALL get('frpw', C_LOC(r4));   canopy%frpw = r4(:, 1)
    CALL get('frpr', C_LOC(r4));   canopy%frpr = r4(:, 1)
    CALL get('frs', C_LOC(r4));    canopy%frs = r4(:, 1)
    CALL get('ebal', C_LOC(r4));   bal%ebal = r4(:, 1)
    CALL get('wbal', C_LOC(r4));   bal%wbal = r4(:, 1)
    CALL get('ebal_tot', C_LOC(r8)); bal%ebal_tot = REAL(r8(:, 1))
    CALL get('wbal_tot', C_LOC(r8)); bal%wbal_tot = REAL(r8(:, 1))
    IF (.NOT. cbm_gpu_copy_all) THEN
      DEALLOCATE(r8, r4, flags)
      RETURN
    END IF
    ! output steps and the driver's own balance checks: their inputs and
    ! what the output writer accumulates
    CALL get('fev', C_LOC(r4));    canopy%fev = r4(:, 1)
    CALL get('fhv', C_LOC(r4));    canopy%fhv = r4(:, 1)
    CALL get('fhs', C_LOC(r4));    canopy%fhs = r4(:, 1)
    CALL get('fns', C_LOC(r4));    canopy%fns = r4(:, 1)
    CALL get('fnv', C_LOC(r4));    canopy%fnv = r4(:, 1)
    CALL get('fes', C_LOC(r4));    canopy%fes = r4(:, 1)
    CALL get('fevc', C_LOC(r4));   canopy%fevc = r4(:, 1)
    CALL get('fevw', C_LOC(r4));   canopy%fevw = r4(:, 1)
    CALL get('us', C_LOC(r4));     canopy%us = r4(:, 1)
    CALL get('cduv', C_LOC(r4));   canopy%cduv = r4(:, 1)
    CALL get('epot', C_LOC(r4));   canopy%epot = r4(:, 1)
    CALL get('dgdtg', C_LOC(r4));  canopy%dgdtg = r4(:, 1)
    CALL get('delwc', C_LOC(r4));  canopy%delwc = r4(:, 1)
    CALL get('through', C_LOC(r4)); canopy%through = r4(:, 1)
    CALL get('precis', C_LOC(r4)); canopy%precis = r4(:, 1)
    CALL get('fwet', C_LOC(r4));   canopy%fwet = r4(:, 1)
    CALL get('ghflux', C_LOC(r4)); canopy%ghflux = r4(:, 1)
    CALL get('sghflux', C_LOC(r4)); canopy%sghflux = r4(:, 1)
    CALL get('cansto', C_LOC(r4)); canopy%cansto = r4(:, 1)
    CALL get('wetfac', C_LOC(r4)); ssnow%wetfac = r4(:, 1)
    CALL get('potev', C_LOC(r4));  ssnow%potev = r4(:, 1)
    CALL get('cls', C_LOC(r4));    ssnow%cls = r4(:, 1)
    CALL get('wbtot', C_LOC(r4));  ssnow%wbtot = r4(:, 1)
    CALL get('albedo_vis', C_LOC(r4)); rad%albedo(:, 1) = r4(:, 1)
    CALL get('albedo_nir', C_LOC(r4)); rad%albedo(:, 2) = r4(:, 1)
    CALL get('transd', C_LOC(r4)); rad%transd = r4(:, 1)
    CALL get('qssabs', C_LOC(r4)); rad%qssabs = r4(:, 1)
    ! soil and snow profiles, snow and surface temperature
    CALL get('wb', C_LOC(r8));     ssnow%wb = r8
    CALL get('wbice', C_LOC(r8));  ssnow%wbice = r8
    CALL get('tgg', C_LOC(r4));    ssnow%tgg = r4
    CALL get('tggsn', C_LOC(r4));  ssnow%tggsn = r4(:, 1:msn)
    CALL get('sdepth', C_LOC(r4)); ssnow%sdepth = r4(:, 1:msn)
    CALL get('flags', C_LOC(flags)); ssnow%isflag = IAND(flags, 1)
    CALL get('snowd', C_LOC(r4));  ssnow%snowd = r4(:, 1)
    CALL get('ssdnn', C_LOC(r4));  ssnow%ssdnn = r4(:, 1)
    CALL get('tss', C_LOC(r4));    ssnow%tss = r4(:, 1)
    DEALLOCATE(r8, r4, flags)
  END SUBROUTINE driver_fields_to_host

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
    IF (ASSOCIATED(forc)) THEN
      CALL check(cablegpu_host_free(C_LOC(forc)), 'host_free forc')
      NULLIFY(forc)
    END IF
    IF (ASSOCIATED(outb)) THEN
      CALL check(cablegpu_host_free(C_LOC(outb)), 'host_free outb')
      NULLIFY(outb)
    END IF
    IF (ALLOCATED(slot_tile)) DEALLOCATE(slot_tile)
  END SUBROUTINE cbm_gpu_finalize

END MODULE cablegpu_shim
