!==============================================================================
! cablegpu_c.F90 - ISO_C_BINDING interfaces of the C ABI declared in
! include/cablegpu.h, shared by the offline (cable_cbm_gpu.F90) and the
! coupled (cable_cbm_coupled_gpu.F90) replacements of cable_cbm_module.
!==============================================================================

MODULE cablegpu_c
  USE, INTRINSIC :: iso_c_binding
  IMPLICIT NONE

  ! struct cablegpu_tiles (include/cablegpu.h)
  TYPE, BIND(C) :: cablegpu_tiles
    INTEGER(c_int) :: mp
    TYPE(c_ptr) :: iveg, isoilm, vlai, lat, lonphase, tbase, swscale
    INTEGER(c_int) :: order
  END TYPE cablegpu_tiles

  INTEGER(c_int), PARAMETER :: CABLEGPU_NFORCING = 13

  INTERFACE
    INTEGER(c_int) FUNCTION cablegpu_create(tiles, device, ctx) BIND(C, name="cablegpu_create")
      IMPORT :: c_int, c_ptr, cablegpu_tiles
      TYPE(cablegpu_tiles), INTENT(IN) :: tiles
      INTEGER(c_int), VALUE :: device
      TYPE(c_ptr), INTENT(OUT) :: ctx
    END FUNCTION cablegpu_create

    INTEGER(c_int) FUNCTION cablegpu_destroy(ctx) BIND(C, name="cablegpu_destroy")
      IMPORT :: c_int, c_ptr
      TYPE(c_ptr), VALUE :: ctx
    END FUNCTION cablegpu_destroy

    INTEGER(c_int) FUNCTION cablegpu_field_id(name) BIND(C, name="cablegpu_field_id")
      IMPORT :: c_int, c_char
      CHARACTER(KIND=c_char), DIMENSION(*), INTENT(IN) :: name
    END FUNCTION cablegpu_field_id

    INTEGER(c_int) FUNCTION cablegpu_set_field(ctx, id, host) BIND(C, name="cablegpu_set_field")
      IMPORT :: c_int, c_ptr
      TYPE(c_ptr), VALUE :: ctx
      INTEGER(c_int), VALUE :: id
      TYPE(c_ptr), VALUE :: host
    END FUNCTION cablegpu_set_field

    INTEGER(c_int) FUNCTION cablegpu_get_field(ctx, id, host) BIND(C, name="cablegpu_get_field")
      IMPORT :: c_int, c_ptr
      TYPE(c_ptr), VALUE :: ctx
      INTEGER(c_int), VALUE :: id
      TYPE(c_ptr), VALUE :: host
    END FUNCTION cablegpu_get_field

    INTEGER(c_int) FUNCTION cablegpu_set_forcing(ctx, host) BIND(C, name="cablegpu_set_forcing")
      IMPORT :: c_int, c_ptr
      TYPE(c_ptr), VALUE :: ctx
      TYPE(c_ptr), VALUE :: host
    END FUNCTION cablegpu_set_forcing

    INTEGER(c_int) FUNCTION cablegpu_set_options(ctx, switches, diag, capture) BIND(C, name="cablegpu_set_options")
      IMPORT :: c_int, c_ptr
      TYPE(c_ptr), VALUE :: ctx
      INTEGER(c_int), VALUE :: switches, diag, capture
    END FUNCTION cablegpu_set_options

    INTEGER(c_int) FUNCTION cablegpu_step(ctx, ktau, dels) BIND(C, name="cablegpu_step")
      IMPORT :: c_int, c_ptr, c_float
      TYPE(c_ptr), VALUE :: ctx
      INTEGER(c_int), VALUE :: ktau
      REAL(c_float), VALUE :: dels
    END FUNCTION cablegpu_step

    INTEGER(c_int) FUNCTION cablegpu_synchronize(ctx) BIND(C, name="cablegpu_synchronize")
      IMPORT :: c_int, c_ptr
      TYPE(c_ptr), VALUE :: ctx
    END FUNCTION cablegpu_synchronize

    INTEGER(c_int) FUNCTION cablegpu_check_tile_param(ctx, name, host) BIND(C, name="cablegpu_check_tile_param")
      IMPORT :: c_int, c_ptr, c_char
      TYPE(c_ptr), VALUE :: ctx
      CHARACTER(KIND=c_char), DIMENSION(*), INTENT(IN) :: name
      TYPE(c_ptr), VALUE :: host
    END FUNCTION cablegpu_check_tile_param

    TYPE(c_ptr) FUNCTION cablegpu_last_error(ctx) BIND(C, name="cablegpu_last_error")
      IMPORT :: c_ptr
      TYPE(c_ptr), VALUE :: ctx
    END FUNCTION cablegpu_last_error

    INTEGER(c_int) FUNCTION cablegpu_step_host(ctx, ktau, dels, forcing, out) BIND(C, name="cablegpu_step_host")
      IMPORT :: c_int, c_float, c_ptr
      TYPE(c_ptr), VALUE :: ctx
      INTEGER(c_int), VALUE :: ktau
      REAL(c_float), VALUE :: dels
      TYPE(c_ptr), VALUE :: forcing, out
    END FUNCTION cablegpu_step_host

    INTEGER(c_int) FUNCTION cablegpu_set_host_layout(ctx, layout) BIND(C, name="cablegpu_set_host_layout")
      IMPORT :: c_int, c_ptr
      TYPE(c_ptr), VALUE :: ctx
      INTEGER(c_int), VALUE :: layout
    END FUNCTION cablegpu_set_host_layout

    INTEGER(c_int) FUNCTION cablegpu_tile_order(ctx, order) BIND(C, name="cablegpu_tile_order")
      IMPORT :: c_int, c_ptr
      TYPE(c_ptr), VALUE :: ctx
      TYPE(c_ptr), VALUE :: order
    END FUNCTION cablegpu_tile_order
    INTEGER(c_int) FUNCTION cablegpu_step_explicit(ctx, ktau, dels, lai_refresh) &
        BIND(C, name="cablegpu_step_explicit")
      IMPORT :: c_int, c_ptr, c_float
      TYPE(c_ptr), VALUE :: ctx
      INTEGER(c_int), VALUE :: ktau, lai_refresh
      REAL(c_float), VALUE :: dels
    END FUNCTION cablegpu_step_explicit

    INTEGER(c_int) FUNCTION cablegpu_step_implicit(ctx, ktau, dels, cycleno, numcycles) &
        BIND(C, name="cablegpu_step_implicit")
      IMPORT :: c_int, c_ptr, c_float
      TYPE(c_ptr), VALUE :: ctx
      INTEGER(c_int), VALUE :: ktau, cycleno, numcycles
      REAL(c_float), VALUE :: dels
    END FUNCTION cablegpu_step_implicit
    INTEGER(c_int) FUNCTION cablegpu_get_fields(ctx, n, ids, host) BIND(C, name="cablegpu_get_fields")
      IMPORT :: c_int, c_ptr
      TYPE(c_ptr), VALUE :: ctx
      INTEGER(c_int), VALUE :: n
      INTEGER(c_int), INTENT(IN) :: ids(*)
      TYPE(c_ptr), INTENT(IN) :: host(*)
    END FUNCTION cablegpu_get_fields

    INTEGER(c_int) FUNCTION cablegpu_host_register(ptr, bytes) BIND(C, name="cablegpu_host_register")
      IMPORT :: c_int, c_ptr, c_size_t
      TYPE(c_ptr), VALUE :: ptr
      INTEGER(c_size_t), VALUE :: bytes
    END FUNCTION cablegpu_host_register

    INTEGER(c_int) FUNCTION cablegpu_host_unregister(ptr) BIND(C, name="cablegpu_host_unregister")
      IMPORT :: c_int, c_ptr
      TYPE(c_ptr), VALUE :: ptr
    END FUNCTION cablegpu_host_unregister

    ! page-locked host memory (cudaHostAlloc), for the per-step buffers
    INTEGER(c_int) FUNCTION cablegpu_host_alloc(bytes, out) BIND(C, name="cablegpu_host_alloc")
      IMPORT :: c_int, c_ptr, c_size_t
      INTEGER(c_size_t), VALUE :: bytes
      TYPE(c_ptr) :: out
    END FUNCTION cablegpu_host_alloc

    INTEGER(c_int) FUNCTION cablegpu_host_free(ptr) BIND(C, name="cablegpu_host_free")
      IMPORT :: c_int, c_ptr
      TYPE(c_ptr), VALUE :: ptr
    END FUNCTION cablegpu_host_free
  END INTERFACE

CONTAINS

  ! Field id of a registry name; stops the run on an unknown name.
  INTEGER(c_int) FUNCTION fid(name)
    CHARACTER(LEN=*), INTENT(IN) :: name
    fid = cablegpu_field_id(TRIM(name) // c_null_char)
    IF (fid < 0) THEN
      WRITE(*, *) 'cablegpu: unknown field ', TRIM(name)
      STOP 'cablegpu: field registry mismatch'
    END IF
  END FUNCTION fid

END MODULE cablegpu_c
