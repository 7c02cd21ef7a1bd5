!*************************************************************************
! velocity (GPU): the reference's velocity module (program/velocity.f90)
! with the time step on one GB300 through the C library (mwf_gpu_c).
!
! It keeps the reference's public names, so main.f90, io.f90, turb.f90 and
! the utilities compile unchanged against it:
!   module variables  vel_p, vel_c, vel_c2, vel_onl, vel_nl, lhs, rhs, nst
!                     (velocity.f90:15-17)
!   vel_TS            velocity.f90:21-41      vel_precompute  velocity.f90:43-50
!   vel_clk_time      velocity.f90:53-64      vel_imposesym   velocity.f90:68-74
!   vel_addlam        velocity.f90:76-82      vel_mpt2phys    velocity.f90:84-90
!   epos, eposC       velocity.f90:115-142    vel_energy      velocity.f90:144-162
!   vel_history       velocity.f90:164-180
! vel_nonlinear (velocity.f90:92-113) has no caller outside vel_TS; its work
! is fused into the library's step and it is not exported.
!
! Where the state lives.  The run's MPT state and its AB2 history are kept on
! the device between steps.  vel_c on the host is refreshed from the device
! after every step (every vel_sync_every steps, see below), so io.f90 reads it
! as before; a state written into vel_c on the host (io_load_state, the
! utilities) is uploaded before the next step or transform.  vel_nl and
! vel_onl stay on the device: their host arrays are not updated.  nst keeps
! its meaning: .true. makes the next step an Euler step (velocity.f90:24-27).
! The symmetry masks of vel_imposesym are applied to the host copy (so
! io.f90 sees the masked state, as in the reference) and by the library at
! the start of every step.  One process drives one GPU: build with _Np = 1.
!*************************************************************************
#include "../parallel.h"
module velocity
  use iso_c_binding
  use mpif
  use variables
  use modes
  use mwf_gpu_c
  implicit none
  save

  type (phys) :: vel_p
  type (mpt), target :: vel_c
  type (mpt)  :: vel_c2,vel_onl,vel_nl,lhs,rhs
  logical :: nst

  ! steps between refreshes of vel_c on the host (1: after every step, so a
  ! stop at any step saves the current state; the refresh also happens
  ! whenever the next io_write2files or the step limit needs vel_c)
  integer :: vel_sync_every = 1
  type(c_ptr), private :: vel_h = c_null_ptr     ! library handle of the run
  logical, private :: vel_host_newer = .true.    ! vel_c was set on the host

contains

  subroutine vel_precompute()
    type(mwf_run_desc) :: d
    call var_mpt_init(vel_c)
    call var_mpt_init(vel_nl)
    call var_LHSRHS(lhs,rhs)
    nst = .true.
    if (_Np /= 1) stop 'velocity (GPU): one process drives one GPU; build with _Np = 1'
    d%K0 = i_K0
    d%MM = i_MM
    d%NN = i_NN
    d%precision = MWF_FP64
    d%alpha = d_alpha
    d%gamma = d_gamma
    d%Re = d_Re
    d%dt = d_dt
    d%drag = d_drag
    d%vdrag = d_vdrag
    d%hypo = d_HYPO
    d%dragall = merge(1, 0, s_dragall)
    d%reflect = merge(1, 0, s_reflect)
    d%uvreflect = merge(1, 0, s_uvreflect)
    d%wreflect = merge(1, 0, s_wreflect)
    d%theta = d_theta
    if (c_associated(vel_h)) call mwf_check(mwf_destroy(vel_h), 'mwf_destroy')
    call mwf_check(mwf_create([d], 1_c_int, 0_c_int, vel_h), 'mwf_create')
    vel_host_newer = .true.
  end subroutine vel_precompute

  ! the host state vel_c replaces the device state
  subroutine vel_upload()
    call mwf_check(mwf_set_state(vel_h, 0_c_int, vel_c%Re, vel_c%Im), 'mwf_set_state')
    vel_host_newer = .false.
  end subroutine vel_upload

  subroutine vel_TS()
    logical :: refresh
    if (vel_host_newer) call vel_upload()
    if (nst) then
       call mwf_check(mwf_reset_history(vel_h, 0_c_int), 'mwf_reset_history')
       nst = .false.
    end if
    call mwf_check(mwf_step(vel_h, 1_c_int), 'mwf_step')
    ! main.f90 advances tim_step after this call; io_write2files then runs at tim_step + 1
    refresh = modulo(tim_step + 1, vel_sync_every) == 0            &
         .or. modulo(tim_step + 1, i_save_rate1) == 0               &
         .or. modulo(tim_step + 1, i_save_rate2) == 0               &
         .or. tim_step + 1 >= i_maxtstep                            &
         .or. (d_maxt > 0d0 .and. tim_t + d_dt >= d_maxt)
    if (refresh) &
         call mwf_check(mwf_get_state(vel_h, 0_c_int, vel_c%Re, vel_c%Im), 'mwf_get_state')
  end subroutine vel_TS

   !-------------------------------------------------------------------------
   ! seconds of CPU time (_CPUTIME) or of wall-clock time; the 64-bit counter of
   ! system_clock does not wrap within a run
   subroutine vel_clk_time(t)
     real, intent(out) :: t
#ifdef _CPUTIME
     call cpu_time(t)
#else
     integer(kind=8) :: count, rate
     call system_clock(count, rate)
     t = real(dble(count) / dble(rate))
#endif
   end subroutine vel_clk_time

!-------------------------------------------------------------------------

  subroutine vel_imposesym()
    if (s_reflect)   call var_reflect(vel_c)
    if (s_uvreflect) call var_uvreflect(vel_c)
    if (s_wreflect)  call var_wreflect(vel_c)
  end subroutine vel_imposesym

  subroutine vel_addlam(u)
    type (spec), intent(inout) :: u
    if (var_N%pH0 == 0) then
       u%Re(2,0,0) = u%Re(2,0,0) + dcos(d_theta)
       u%Re(2*i_K0+1,0,0) = u%Re(2*i_K0+1,0,0) + dsin(d_theta)
    end if
  end subroutine vel_addlam

  ! u, v, w of an MPT state on the physical grid, on the device.  u is uploaded
  ! first unless it is vel_c and the device already holds it.
  subroutine vel_mpt2phys(u,p)
    type(mpt), intent(in), target :: u
    type(phys), intent(out) :: p
    logical :: is_vel_c
    is_vel_c = c_associated(c_loc(u%Re), c_loc(vel_c%Re))
    if (.not. is_vel_c .or. vel_host_newer) then
       call mwf_check(mwf_set_state(vel_h, 0_c_int, u%Re, u%Im), 'mwf_set_state')
       vel_host_newer = .not. is_vel_c        ! the device holds u, not vel_c
    end if
    call mwf_check(mwf_get_phys(vel_h, 0_c_int, p%Re), 'mwf_get_phys')
  end subroutine vel_mpt2phys

  ! y-mean of u.u at one point (velocity.f90:115-126)
  function epos(u) result(e)
    double precision :: e
    double precision,intent(in) :: u(i_KK)
    double precision :: udotu(i_K0)
    udotu = nluw(u(1:i_K0),u(1:i_K0))
    e = udotu(1)
    udotu = nlvv(u(i_K0+1:2*i_K0-1))
    e = e + udotu(1)
    udotu = nluw(u(2*i_K0:i_KK),u(2*i_K0:i_KK))
    e = e + udotu(1)
  end function epos

  ! its three components (velocity.f90:128-142)
  function eposC(u) result(e)
    double precision :: e(3)
    double precision,intent(in) :: u(i_KK)
    double precision :: udotu(i_K0)
    udotu = nluw(u(1:i_K0),u(1:i_K0))
    e(1) = udotu(1)
    udotu = nlvv(u(i_K0+1:2*i_K0-1))
    e(2) = udotu(1)
    udotu = nluw(u(2*i_K0:i_KK),u(2*i_K0:i_KK))
    e(3) = udotu(1)
  end function eposC

  ! mean of epos over the grid points of a physical field (velocity.f90:144-162)
  subroutine vel_energy(a,e)
    type (phys), intent(in) :: a
    double precision, intent(out) :: e
    integer :: m, n
    e = 0d0
    do m = 0, i_3M-1
       do n = 0, i_3N-1
          e = e + epos(a%Re(:,n,m))
       end do
    end do
    e = e / (i_3M * i_3N)
  end subroutine vel_energy

  ! velocity probes at x = 0, height y (velocity.f90:164-180)
  subroutine vel_history(V,y,ans)
    type(phys), intent(in) :: V
    double precision, intent(out) :: ans(4,i_H)
    double precision,intent(in) :: y
    integer :: j,ji
    if(mpi_rnk/=0) return
    do j=1,i_H
       ji=int((j-1)*i_3N/i_H)+1
       ans(1,j)=dble(ji)*d_Lz/i_3N
       ans(2,j)=velU(V%Re(:,ji,0),y)
       ans(3,j)=velV(V%Re(:,ji,0),y)
       ans(4,j)=velW(V%Re(:,ji,0),y)
    end do
  end subroutine vel_history

end module velocity
