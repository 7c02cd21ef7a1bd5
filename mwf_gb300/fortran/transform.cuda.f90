!*************************************************************************
! transform (GPU): the reference's transform module
! (program/transform.fftw5.f90) with the 3/2-dealiased 2D transforms on one
! GB300 through the C library (mwf_gpu_c).  Public names as in the
! reference: tra_precompute (transform.fftw5.f90:33-59), tra_spec2phys
! (64-87) and tra_phys2spec (122-145).  The transforms of the time step itself
! are fused into the library's step (velocity.gpu.f90); these two serve the
! callers that transform fields of their own.  Each call moves its arrays to
! the device and back.  One process drives one GPU: build with _Np = 1.
!*************************************************************************
#include "../parallel.h"
module transform
  use iso_c_binding
  use parameters
  use variables
  use mpif
  use mwf_gpu_c
  implicit none
  save

  type(mwf_run_desc), private :: tra_d

contains

  ! the library plans its transforms per grid size when it is called; this
  ! records the grid the module's transforms use
  subroutine tra_precompute
    if (_Np /= 1) stop 'transform (GPU): one process drives one GPU; build with _Np = 1'
    tra_d%K0 = i_K0
    tra_d%MM = i_MM
    tra_d%NN = i_NN
    tra_d%precision = MWF_FP64
    tra_d%alpha = d_alpha
    tra_d%gamma = d_gamma
    tra_d%Re = d_Re
    tra_d%dt = d_dt
    tra_d%drag = d_drag
    tra_d%vdrag = d_vdrag
    tra_d%hypo = d_HYPO
    tra_d%dragall = merge(1, 0, s_dragall)
    tra_d%reflect = 0
    tra_d%uvreflect = 0
    tra_d%wreflect = 0
    tra_d%theta = d_theta
  end subroutine tra_precompute

  ! spectral u, v, w (KK fields) -> the 3MM x 3NN physical grid, unnormalised
  ! backward transforms with the 3/2-rule padding
  subroutine tra_spec2phys(s, p)
    type (spec), intent(in)  :: s
    type (phys), intent(out) :: p
    call mwf_check(mwf_spec2phys(tra_d, s%Re, s%Im, p%Re), 'mwf_spec2phys')
  end subroutine tra_spec2phys

  ! physical grid -> the retained spectral modes, scaled by 1/(3MM 3NN)
  subroutine tra_phys2spec(p, s)
    type (phys), intent(in)  :: p
    type (spec), intent(out) :: s
    call mwf_check(mwf_phys2spec(tra_d, p%Re, s%Re, s%Im), 'mwf_phys2spec')
  end subroutine tra_phys2spec

end module transform
