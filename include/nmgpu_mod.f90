! nmgpu_mod.f90 -- Fortran 2003 ISO_C_BINDING interface to libnmgpu
! (include/nmgpu.h).  This is the binding a NormalModes build would use to
! hand its operators to the GPU and to keep pEVSL's callback registration
! shape (src/mod_pevsl.f90:69-80): nm_amv / nm_bmv / nm_bsolve take
! (ctx, v, w) like sparsefsAV / sparseBV / solveBV take (v, w, mymv).
!
! Derived types mirror the C structs field by field (bind(C) keeps the C
! layout).  Pointers to arrays are passed as type(c_ptr) from c_loc().
module nmgpu_mod
  use iso_c_binding
  implicit none

  integer(c_int), parameter :: NM_OK = 0, NM_ERR_ARG = -1, NM_ERR_CUDA = -2, NM_ERR_OOM = -3, &
                               NM_ERR_NOCONV = -4, NM_ERR_TIMEOUT = -5, NM_ERR_NUMERIC = -6
  integer(c_int), parameter :: NM_PREC_FP64 = 0, NM_PREC_MIXED = 1
  ! phases of the progress callback, subroutine progress(data, phase, done, total) bind(C)
  integer(c_int), parameter :: NM_PHASE_BOUNDS = 0, NM_PHASE_LANCZOS = 1, NM_PHASE_RITZ = 2, &
                               NM_PHASE_REFINE = 3, NM_PHASE_DONE = 4

  type, bind(C) :: nm_csr
    integer(c_int) :: nrows, ncols
    type(c_ptr) :: rowptr   ! int32, 0-based, nrows+1
    type(c_ptr) :: col      ! int32, 0-based (the reference passes col-1)
    type(c_ptr) :: val      ! real(c_double)
  end type nm_csr

  type, bind(C) :: nm_opts
    integer(c_int) :: porder, device, b_cheb_deg, ap_cheb_deg
    real(c_double) :: b_bounds(2), ap_bounds(2)
    integer(c_int) :: precision, verbose
    integer(c_int) :: filter_form, orth
    real(c_double) :: inner_tol
    integer(c_int) :: autotune
  end type nm_opts

  type, bind(C) :: nm_solve_opts
    integer(c_int) :: maxit
    real(c_double) :: tol, thresh_int, thresh_ext
    integer(c_int) :: mlan_bounds
    real(c_double) :: ab_bounds(2)
    integer(c_int) :: damping, want_vectors, unscale, use_graph, block, polish
    real(c_double) :: resid_tol
    integer(c_int) :: refine_sweeps, refine_maxdeg
    real(c_double) :: refine_band
    integer(c_int) :: refine_purge
    type(c_funptr) :: progress
    type(c_ptr) :: progress_data
    real(c_double) :: refine_guard, refine_near, refine_growth
  end type nm_solve_opts

  type, bind(C) :: nm_result
    integer(c_int) :: nev, n
    type(c_ptr) :: lam, vec, err_ref, res2
    real(c_double) :: xintv(4)
    integer(c_int) :: pol_deg
    real(c_double) :: pol_gam, pol_bar
    integer(c_int) :: lanczos_steps, nritz_above_bar
    real(c_double) :: t_bounds, t_filter_design, t_lanczos, t_ritz, t_total
    integer(c_long_long) :: n_amv, n_bsolve, n_spmv, n_kernels
    real(c_double) :: t_filter, t_orth, t_eig
    integer(c_int) :: refine_passes, refine_blocks, refine_maxdeg
    integer(c_long_long) :: refine_steps
    real(c_double) :: res2_before_refine
    integer(c_int) :: refine_guards
  end type nm_result

  type, bind(C) :: nm_slice
    real(c_double) :: f_lo_mhz, f_hi_mhz
  end type nm_slice

  type, bind(C) :: nm_kpm_opts
    integer(c_int) :: degree, nvec
    integer(c_long_long) :: seed          ! unsigned long long in C
    real(c_double) :: ab_bounds(2)
  end type nm_kpm_opts

  interface
    integer(c_int) function nm_create(ctx, A, B, Ap, E, ET, opts) bind(C, name="nm_create")
      import :: c_int, c_ptr, nm_csr, nm_opts
      type(c_ptr), intent(out) :: ctx
      type(nm_csr), intent(in) :: A, B
      type(c_ptr), value :: Ap, E, ET          ! c_loc(nm_csr) or c_null_ptr (solid model)
      type(nm_opts), intent(in) :: opts
    end function nm_create

    subroutine nm_destroy(ctx) bind(C, name="nm_destroy")
      import :: c_ptr
      type(c_ptr), value :: ctx
    end subroutine nm_destroy

    subroutine nm_default_opts(o) bind(C, name="nm_default_opts")
      import :: nm_opts
      type(nm_opts), intent(out) :: o
    end subroutine nm_default_opts

    subroutine nm_default_solve_opts(o) bind(C, name="nm_default_solve_opts")
      import :: nm_solve_opts
      type(nm_solve_opts), intent(out) :: o
    end subroutine nm_default_solve_opts

    ! sparseAV / sparsefsAV (src/mod_matvec.f90:445-458,498-520)
    integer(c_int) function nm_amv(ctx, v, w) bind(C, name="nm_amv")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(in) :: v(*)
      real(c_double), intent(out) :: w(*)
    end function nm_amv

    ! sparseBV (src/mod_matvec.f90:461-472)
    integer(c_int) function nm_bmv(ctx, v, w) bind(C, name="nm_bmv")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(in) :: v(*)
      real(c_double), intent(out) :: w(*)
    end function nm_bmv

    ! solveBV (src/mod_matvec.f90:475-483)
    integer(c_int) function nm_bsolve(ctx, v, w) bind(C, name="nm_bsolve")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(in) :: v(*)
      real(c_double), intent(out) :: w(*)
    end function nm_bsolve

    ! pnm_apply_pevsl (src/mod_pevsl.f90:16-222)
    integer(c_int) function nm_solve(ctx, f_lo_mhz, f_hi_mhz, opts, res) bind(C, name="nm_solve")
      import :: c_int, c_ptr, c_double, nm_solve_opts, nm_result
      type(c_ptr), value :: ctx
      real(c_double), value :: f_lo_mhz, f_hi_mhz
      type(nm_solve_opts), intent(in) :: opts
      type(nm_result), intent(inout) :: res
    end function nm_solve

    ! several intervals on one context (no counterpart in the reference)
    integer(c_int) function nm_solve_batched(ctx, slices, nslices, opts, results) &
        bind(C, name="nm_solve_batched")
      import :: c_int, c_ptr, nm_slice, nm_solve_opts, nm_result
      type(c_ptr), value :: ctx
      type(nm_slice), intent(in) :: slices(*)
      integer(c_int), value :: nslices
      type(nm_solve_opts), intent(in) :: opts
      type(nm_result), intent(inout) :: results(*)
    end function nm_solve_batched

    subroutine nm_default_kpm_opts(o) bind(C, name="nm_default_kpm_opts")
      import :: nm_kpm_opts
      type(nm_kpm_opts), intent(out) :: o
    end subroutine nm_default_kpm_opts

    ! equal-count slices of [f_lo, f_hi] for nm_solve_batched (KPM estimate)
    integer(c_int) function nm_slice_spectrum(ctx, f_lo_mhz, f_hi_mhz, nslices, opts, slices, counts) &
        bind(C, name="nm_slice_spectrum")
      import :: c_int, c_ptr, c_double, nm_kpm_opts, nm_slice
      type(c_ptr), value :: ctx
      real(c_double), value :: f_lo_mhz, f_hi_mhz
      integer(c_int), value :: nslices
      type(nm_kpm_opts), intent(in) :: opts
      type(nm_slice), intent(out) :: slices(*)
      real(c_double), intent(out) :: counts(*)
    end function nm_slice_spectrum

    subroutine nm_result_free(res) bind(C, name="nm_result_free")
      import :: nm_result
      type(nm_result), intent(inout) :: res
    end subroutine nm_result_free

    type(c_ptr) function nm_last_error(ctx) bind(C, name="nm_last_error")
      import :: c_ptr
      type(c_ptr), value :: ctx
    end function nm_last_error
  end interface
end module nmgpu_mod
