!-----------------------------------------------------------------------
! mg_filtering_gpu: ISO_C_BINDING shim over libmgbf for Fortran callers.
!
! Drop-in for the filtering path of the reference's modules:
!   mg_initialize            (mg_entrymod.f90:36)   -> mg_initialize_gpu
!   filtering_procedure(mg_filt) (mg_filtering.f90:67) -> filtering_procedure
!   anal_to_filt_all2 / filt_to_anal_all2 (mg_transfer.f90:154-203)
!                                                   -> anal_to_filt_all2 / filt_to_anal_all2
!   mg_finalize              (mg_entrymod.f90:222)  -> mg_finalize_gpu
! A caller such as RBETA_TEST keeps `call filtering_procedure(mgbf_proc)`
! and passes its VALL array (km_all, 1-hx:im+hx, 1-hy:jm+hy) in real(8),
! laid out over the whole filter grid (im = nxPE*im_filt, jm = nyPE*jm_filt).
! The array stays in host memory; libmgbf copies it to the GPU and back.
! The namelist is read from 'mgbeta.nml', the file name the reference uses
! (mg_parameter.f90:210).
!
! Not compiled in this project's build: no Fortran compiler is available
! on the build and test machines.  The C-ABI it binds is tested from C and
! Python.
!-----------------------------------------------------------------------
module mg_filtering_gpu
  use iso_c_binding
  implicit none
  private
  public :: mg_initialize_gpu, filtering_procedure, filtering_procedure_adjoint, mg_finalize_gpu
  public :: anal_to_filt_all2, filt_to_anal_all2
  public :: mgbf_ok

  integer(c_int), parameter :: mgbf_ok = 0
  integer(c_int), parameter :: mgbf_f64 = 0, mgbf_mem_host = 1

  type(c_ptr), save :: handle = c_null_ptr

  interface
    integer(c_int) function mgbf_create_from_namelist(path, out) bind(C, name="mgbf_create_from_namelist")
      import :: c_int, c_char, c_ptr
      character(kind=c_char), dimension(*), intent(in) :: path
      type(c_ptr), intent(out) :: out
    end function
    integer(c_int) function mgbf_filtering_procedure(h, mg_filt, vall, dtype, mem, stream) &
        bind(C, name="mgbf_filtering_procedure")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
      integer(c_int), value :: mg_filt, dtype, mem
      type(c_ptr), value :: vall, stream
    end function
    integer(c_int) function mgbf_filtering_procedure_adjoint(h, mg_filt, vall, dtype, mem, stream) &
        bind(C, name="mgbf_filtering_procedure_adjoint")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
      integer(c_int), value :: mg_filt, dtype, mem
      type(c_ptr), value :: vall, stream
    end function
    integer(c_int) function mgbf_anal_to_filt(h, worka, vall, dtype, mem, stream) bind(C, name="mgbf_anal_to_filt")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
      type(c_ptr), value :: worka, vall, stream
      integer(c_int), value :: dtype, mem
    end function
    integer(c_int) function mgbf_filt_to_anal(h, vall, worka, dtype, mem, stream) bind(C, name="mgbf_filt_to_anal")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
      type(c_ptr), value :: vall, worka, stream
      integer(c_int), value :: dtype, mem
    end function
    integer(c_int) function mgbf_destroy(h) bind(C, name="mgbf_destroy")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
    end function
    type(c_ptr) function mgbf_last_error() bind(C, name="mgbf_last_error")
      import :: c_ptr
    end function
  end interface

contains

  subroutine fail(rc, what)
    integer(c_int), intent(in) :: rc
    character(*), intent(in) :: what
    print '(a,a,i4)', what, ': libmgbf error ', rc
    stop 'mg_filtering_gpu'
  end subroutine

  ! Replaces mg_initialize for the filtering path: reads mgbeta.nml and
  ! builds the filter tables.
  subroutine mg_initialize_gpu()
    integer(c_int) :: rc
    rc = mgbf_create_from_namelist('mgbeta.nml'//c_null_char, handle)
    if (rc /= mgbf_ok) call fail(rc, 'mg_initialize_gpu')
  end subroutine

  ! filtering_procedure(mg_filt) on VALL in place.
  subroutine filtering_procedure(mg_filt, vall)
    integer, intent(in) :: mg_filt
    real(c_double), dimension(:,:,:), contiguous, target, intent(inout) :: vall
    integer(c_int) :: rc
    rc = mgbf_filtering_procedure(handle, int(mg_filt, c_int), c_loc(vall), mgbf_f64, mgbf_mem_host, c_null_ptr)
    if (rc /= mgbf_ok) call fail(rc, 'filtering_procedure')
  end subroutine

  subroutine filtering_procedure_adjoint(mg_filt, vall)
    integer, intent(in) :: mg_filt
    real(c_double), dimension(:,:,:), contiguous, target, intent(inout) :: vall
    integer(c_int) :: rc
    rc = mgbf_filtering_procedure_adjoint(handle, int(mg_filt, c_int), c_loc(vall), mgbf_f64, mgbf_mem_host, &
                                          c_null_ptr)
    if (rc /= mgbf_ok) call fail(rc, 'filtering_procedure_adjoint')
  end subroutine

  ! anal_to_filt_all2: WORKA(km_a_all, nm0, mm0) -> VALL (overwritten).
  subroutine anal_to_filt_all2(worka, vall)
    real(c_double), dimension(:,:,:), contiguous, target, intent(in) :: worka
    real(c_double), dimension(:,:,:), contiguous, target, intent(inout) :: vall
    integer(c_int) :: rc
    rc = mgbf_anal_to_filt(handle, c_loc(worka), c_loc(vall), mgbf_f64, mgbf_mem_host, c_null_ptr)
    if (rc /= mgbf_ok) call fail(rc, 'anal_to_filt_all2')
  end subroutine

  ! filt_to_anal_all2: VALL -> WORKA; VALL's interpolation halo is filled,
  ! as boco_2d does in the reference.
  subroutine filt_to_anal_all2(vall, worka)
    real(c_double), dimension(:,:,:), contiguous, target, intent(inout) :: vall
    real(c_double), dimension(:,:,:), contiguous, target, intent(inout) :: worka
    integer(c_int) :: rc
    rc = mgbf_filt_to_anal(handle, c_loc(vall), c_loc(worka), mgbf_f64, mgbf_mem_host, c_null_ptr)
    if (rc /= mgbf_ok) call fail(rc, 'filt_to_anal_all2')
  end subroutine

  subroutine mg_finalize_gpu()
    integer(c_int) :: rc
    rc = mgbf_destroy(handle)
    handle = c_null_ptr
  end subroutine

end module mg_filtering_gpu
