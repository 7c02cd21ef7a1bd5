!*************************************************************************
! mwf_gpu_c: Fortran (iso_c_binding) binding of the GB300 timestep library,
! mirroring the C header include/mwf_gpu.h entry point by entry point.
!
! Every function returns 0 (MWF_OK) or a negative MWF_ERR_* code.  Arrays
! are passed by reference in the reference's own layouts: a type(mpt) state
! as its Re and Im arrays (K, 0:M-1, 0:NN-1), a type(spec) as its Re and Im
! arrays (KK, 0:M-1, 0:NN-1), a type(phys) as its Re array
! (KK, 0:3NN-1, 0:3MM-1).  mwf_check stops the program with the library's
! message, as the reference stops on I/O errors (io.f90:135,177,195).
!*************************************************************************
module mwf_gpu_c
  use iso_c_binding
  implicit none

  integer(c_int), parameter :: MWF_FP64 = 0, MWF_FP32 = 1
  integer(c_int), parameter :: MWF_OK = 0

  ! one run: the run-time copy of the compile-time constants of parameters.f90
  type, bind(c) :: mwf_run_desc
     integer(c_int) :: K0, MM, NN, precision
     real(c_double) :: alpha, gamma, Re, dt, drag, vdrag, hypo
     integer(c_int) :: dragall, reflect, uvreflect, wreflect
     real(c_double) :: theta
     integer(c_int) :: xf_cols = 0, xi_cols = 0, z_lines = 0, x_radix = 0, z_radix = 0
  end type mwf_run_desc

  interface
     integer(c_int) function mwf_create(runs, n_runs, device, h) bind(c, name='mwf_create')
       import :: c_int, c_ptr, mwf_run_desc
       type(mwf_run_desc), intent(in) :: runs(*)
       integer(c_int), value :: n_runs, device
       type(c_ptr), intent(out) :: h
     end function mwf_create

     integer(c_int) function mwf_destroy(h) bind(c, name='mwf_destroy')
       import :: c_int, c_ptr
       type(c_ptr), value :: h
     end function mwf_destroy

     integer(c_int) function mwf_set_state(h, run, re, im) bind(c, name='mwf_set_state')
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: h
       integer(c_int), value :: run
       real(c_double), intent(in) :: re(*), im(*)
     end function mwf_set_state

     integer(c_int) function mwf_get_state(h, run, re, im) bind(c, name='mwf_get_state')
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: h
       integer(c_int), value :: run
       real(c_double), intent(out) :: re(*), im(*)
     end function mwf_get_state

     integer(c_int) function mwf_step(h, nsteps) bind(c, name='mwf_step')
       import :: c_int, c_ptr
       type(c_ptr), value :: h
       integer(c_int), value :: nsteps
     end function mwf_step

     integer(c_int) function mwf_reset_history(h, run) bind(c, name='mwf_reset_history')
       import :: c_int, c_ptr
       type(c_ptr), value :: h
       integer(c_int), value :: run
     end function mwf_reset_history

     integer(c_int) function mwf_energy(h, run, e) bind(c, name='mwf_energy')
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: h
       integer(c_int), value :: run
       real(c_double), intent(out) :: e
     end function mwf_energy

     integer(c_int) function mwf_phys_diagnostics(h, run, threshold, count_above, energy) &
          bind(c, name='mwf_phys_diagnostics')
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: h
       integer(c_int), value :: run
       real(c_double), value :: threshold
       real(c_double), intent(out) :: count_above, energy
     end function mwf_phys_diagnostics

     integer(c_int) function mwf_get_phys(h, run, p) bind(c, name='mwf_get_phys')
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: h
       integer(c_int), value :: run
       real(c_double), intent(out) :: p(*)
     end function mwf_get_phys

     integer(c_int) function mwf_spectrum_maxima(h, run, m_max, n_max) bind(c, name='mwf_spectrum_maxima')
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: h
       integer(c_int), value :: run
       real(c_double), intent(out) :: m_max(*), n_max(*)
     end function mwf_spectrum_maxima

     integer(c_int) function mwf_history(h, run, y, n_probes, hist) bind(c, name='mwf_history')
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: h
       integer(c_int), value :: run, n_probes
       real(c_double), value :: y
       real(c_double), intent(out) :: hist(*)
     end function mwf_history

     integer(c_int) function mwf_remap_x(h, run, factor) bind(c, name='mwf_remap_x')
       import :: c_int, c_ptr
       type(c_ptr), value :: h
       integer(c_int), value :: run, factor
     end function mwf_remap_x

     integer(c_int) function mwf_blend_state(h, run, other, d) bind(c, name='mwf_blend_state')
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: h
       integer(c_int), value :: run, other
       real(c_double), value :: d
     end function mwf_blend_state

     integer(c_int) function mwf_add_noise(h, run, scale, seed) bind(c, name='mwf_add_noise')
       import :: c_int, c_ptr, c_double, c_long_long
       type(c_ptr), value :: h
       integer(c_int), value :: run
       real(c_double), value :: scale
       integer(c_long_long), value :: seed
     end function mwf_add_noise

     integer(c_int) function mwf_spec2phys(d, s_re, s_im, p) bind(c, name='mwf_spec2phys')
       import :: c_int, c_double, mwf_run_desc
       type(mwf_run_desc), intent(in) :: d
       real(c_double), intent(in) :: s_re(*), s_im(*)
       real(c_double), intent(out) :: p(*)
     end function mwf_spec2phys

     integer(c_int) function mwf_phys2spec(d, p, s_re, s_im) bind(c, name='mwf_phys2spec')
       import :: c_int, c_double, mwf_run_desc
       type(mwf_run_desc), intent(in) :: d
       real(c_double), intent(in) :: p(*)
       real(c_double), intent(out) :: s_re(*), s_im(*)
     end function mwf_phys2spec

     integer(c_int) function mwf_last_error(buf, len) bind(c, name='mwf_last_error')
       import :: c_int, c_char, c_size_t
       character(kind=c_char), intent(out) :: buf(*)
       integer(c_size_t), value :: len
     end function mwf_last_error
  end interface

contains

  ! stop with the library's message when a call failed
  subroutine mwf_check(rc, what)
    integer(c_int), intent(in) :: rc
    character(*), intent(in) :: what
    character(kind=c_char) :: buf(512)
    character(len=512) :: msg
    integer(c_int) :: n
    integer :: i
    if (rc == MWF_OK) return
    n = mwf_last_error(buf, int(size(buf), c_size_t))
    msg = ' '
    do i = 1, min(int(n), len(msg))
       msg(i:i) = buf(i)
    end do
    print*, what, ' failed (', rc, '): ', trim(msg)
    stop 'mwf_gpu: library call failed'
  end subroutine mwf_check

end module mwf_gpu_c
