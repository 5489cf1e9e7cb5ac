! vlm_gb300.f90 -- ISO_C_BINDING interfaces of libvlm_gb300.so (include/vlm.h)
! for a Fortran host of the reference (VOLCANOR).  A maintainer compiles this
! module with the host program and links the shared library:
!   gfortran -O2 vlm_gb300.f90 main.f90 -L<repo>/volcanor_gb300/_build -lvlm_gb300 \
!            -Wl,-rpath,<repo>/volcanor_gb300/_build
! Every interface binds one C symbol by name with the header's argument list;
! arrays of shape (3, m) pass without repacking (xyz fastest).
module vlm_gb300
  use, intrinsic :: iso_c_binding
  implicit none
  integer(c_int), parameter :: VLM_OK = 0, VLM_PREC_FP64 = 0, VLM_PREC_FP32 = 1, VLM_PREC_FP32_NEAR64 = 2

  type, bind(c) :: vlm_options
    integer(c_int) :: precision
    integer(c_int) :: sum_chunk
    real(c_double) :: near_factor
    integer(c_int) :: device
    integer(c_int) :: use_graph
    integer(c_int) :: solve_mode
    integer(c_int) :: nbody_slots
    integer(c_int) :: lattice
    integer(c_int) :: incremental
  end type

  interface
    subroutine vlm_default_options(opt) bind(c, name='vlm_default_options')
      import :: vlm_options
      type(vlm_options), intent(out) :: opt
    end subroutine
    integer(c_int) function vlm_last_error(buf, len) bind(c, name='vlm_last_error')
      import :: c_int, c_char, c_size_t
      character(kind=c_char), intent(out) :: buf(*)
      integer(c_size_t), value :: len
    end function
    integer(c_int) function vlm_case_create_from_dir(dir, opt, cs) bind(c, name='vlm_case_create_from_dir')
      import :: c_int, c_char, c_ptr, vlm_options
      character(kind=c_char), intent(in) :: dir(*)
      type(vlm_options), intent(in) :: opt
      type(c_ptr), intent(out) :: cs
    end function
    integer(c_int) function vlm_case_create(cfg, geo, base, opt, cs) bind(c, name='vlm_case_create')
      import :: c_int, c_char, c_ptr, vlm_options
      character(kind=c_char), intent(in) :: cfg(*), geo(*), base(*)
      type(vlm_options), intent(in) :: opt
      type(c_ptr), intent(out) :: cs
    end function
    integer(c_int) function vlm_case_destroy(cs) bind(c, name='vlm_case_destroy')
      import :: c_int, c_ptr
      type(c_ptr), value :: cs
    end function
    integer(c_int) function vlm_case_start(cs) bind(c, name='vlm_case_start')
      import :: c_int, c_ptr
      type(c_ptr), value :: cs
    end function
    integer(c_int) function vlm_case_step(cs, nsteps, ct_rows) bind(c, name='vlm_case_step')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: cs
      integer(c_int), value :: nsteps
      real(c_double), intent(out) :: ct_rows(10, *)
    end function
    ! coupled rotors (nr > 1): config.nml + geom01.nml .. geomNN.nml of a case
    ! directory; rotor handles (0-based ir) serve vlm_case_get / _get_int
    integer(c_int) function vlm_system_create_from_dir(dir, opt, ys) bind(c, name='vlm_system_create_from_dir')
      import :: c_int, c_char, c_ptr, vlm_options
      character(kind=c_char), intent(in) :: dir(*)
      type(vlm_options), intent(in) :: opt
      type(c_ptr), intent(out) :: ys
    end function
    integer(c_int) function vlm_system_rotor(ys, ir, cs) bind(c, name='vlm_system_rotor')
      import :: c_int, c_ptr
      type(c_ptr), value :: ys
      integer(c_int), value :: ir
      type(c_ptr), intent(out) :: cs
    end function
    integer(c_int) function vlm_system_start(ys) bind(c, name='vlm_system_start')
      import :: c_int, c_ptr
      type(c_ptr), value :: ys
    end function
    integer(c_int) function vlm_system_step(ys, nsteps, ct_rows) bind(c, name='vlm_system_step')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ys
      integer(c_int), value :: nsteps
      real(c_double), intent(out) :: ct_rows(10, *)
    end function
    integer(c_int) function vlm_system_destroy(ys) bind(c, name='vlm_system_destroy')
      import :: c_int, c_ptr
      type(c_ptr), value :: ys
    end function
    integer(c_int) function vlm_case_get_int(cs, name, val) bind(c, name='vlm_case_get_int')
      import :: c_int, c_ptr, c_char, c_int64_t
      type(c_ptr), value :: cs
      character(kind=c_char), intent(in) :: name(*)
      integer(c_int64_t), intent(out) :: val
    end function
    integer(c_int64_t) function vlm_case_get(cs, name, blade, out, cap) bind(c, name='vlm_case_get')
      import :: c_int, c_ptr, c_char, c_int64_t, c_double
      type(c_ptr), value :: cs
      character(kind=c_char), intent(in) :: name(*)
      integer(c_int), value :: blade
      real(c_double), intent(out) :: out(*)
      integer(c_int64_t), value :: cap
    end function
    integer(c_int) function vlm_biot_savart_filaments(fc, rvc, gam, n, P, m, V, prec) &
        bind(c, name='vlm_biot_savart_filaments')
      import :: c_int, c_int64_t, c_double
      real(c_double), intent(in) :: fc(3, 2, *), rvc(*), gam(*), P(3, *)
      integer(c_int64_t), value :: n, m
      real(c_double), intent(out) :: V(3, *)
      integer(c_int), value :: prec
    end function
    integer(c_int64_t) function vlm_wing_kinematics(cfg, geo, base, iter, name, blade, out, cap) &
        bind(c, name='vlm_wing_kinematics')
      import :: c_int, c_int64_t, c_char, c_double
      character(kind=c_char), intent(in) :: cfg(*), geo(*), base(*), name(*)
      integer(c_int), value :: iter, blade
      real(c_double), intent(out) :: out(*)
      integer(c_int64_t), value :: cap
    end function
    integer(c_int64_t) function vlm_case_params_json(cs, buf, cap) bind(c, name='vlm_case_params_json')
      import :: c_ptr, c_char, c_int64_t
      type(c_ptr), value :: cs
      character(kind=c_char), intent(out) :: buf(*)
      integer(c_int64_t), value :: cap
    end function
    integer(c_int) function vlm_case_vind_points(cs, P, m, V) bind(c, name='vlm_case_vind_points')
      import :: c_int, c_ptr, c_int64_t, c_double
      type(c_ptr), value :: cs
      real(c_double), intent(in) :: P(3, *)
      integer(c_int64_t), value :: m
      real(c_double), intent(out) :: V(3, *)
    end function
    integer(c_int) function vlm_biot_savart_rings(corners, rvc, gam, n, P, m, V, prec) &
        bind(c, name='vlm_biot_savart_rings')
      import :: c_int, c_int64_t, c_double
      real(c_double), intent(in) :: corners(3, 4, *), rvc(4, *), gam(*), P(3, *)
      integer(c_int64_t), value :: n, m
      real(c_double), intent(out) :: V(3, *)
      integer(c_int), value :: prec
    end function
    ! the time step as separate calls (include/vlm.h): a host that keeps its
    ! own loop replaces calcAIC + inv2, the RHS loop + matmulAX + map_gam,
    ! calc_force, and the wake update one by one
    integer(c_int) function vlm_case_aic_factor(cs) bind(c, name='vlm_case_aic_factor')
      import :: c_int, c_ptr
      type(c_ptr), value :: cs
    end function
    integer(c_int) function vlm_case_solve_circulation(cs, kinematic_vel, gam_out) &
        bind(c, name='vlm_case_solve_circulation')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: cs
      ! absent optional arguments pass NULL (Fortran 2018 interoperability)
      real(c_double), intent(in), optional :: kinematic_vel(3, *)
      real(c_double), intent(out), optional :: gam_out(*)
    end function
    integer(c_int) function vlm_case_loads(cs, ct_row) bind(c, name='vlm_case_loads')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: cs
      real(c_double), intent(out), optional :: ct_row(10)
    end function
    integer(c_int) function vlm_case_wake_step(cs) bind(c, name='vlm_case_wake_step')
      import :: c_int, c_ptr
      type(c_ptr), value :: cs
    end function
    integer(c_int) function vlm_case_get_wake(cs, blade, waN, waN_gam, waF, waF_gam) &
        bind(c, name='vlm_case_get_wake')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: cs
      integer(c_int), value :: blade
      real(c_double), intent(out) :: waN(3, 4, *), waN_gam(*), waF(3, 2, *), waF_gam(*)
    end function
    integer(c_int) function vlm_case_checkpoint_save(cs, path) bind(c, name='vlm_case_checkpoint_save')
      import :: c_int, c_ptr, c_char
      type(c_ptr), value :: cs
      character(kind=c_char), intent(in) :: path(*)
    end function
    integer(c_int) function vlm_case_checkpoint_load(cs, path) bind(c, name='vlm_case_checkpoint_load')
      import :: c_int, c_ptr, c_char
      type(c_ptr), value :: cs
      character(kind=c_char), intent(in) :: path(*)
    end function
  end interface

contains

  subroutine vlm_check(stat)
    integer(c_int), intent(in) :: stat
    character(kind=c_char) :: buf(512)
    integer :: i, ierr
    if (stat == VLM_OK) return
    ierr = vlm_last_error(buf, int(size(buf), c_size_t))
    do i = 1, size(buf)
      if (buf(i) == c_null_char) exit
      write(*, '(a)', advance='no') buf(i)
    end do
    write(*, *)
    error stop 'libvlm_gb300 error'
  end subroutine

end module vlm_gb300
