! mxll_3D_gpu_mod.f90 -- TMxll_3D_gpu: the reference's 3D Maxwell type (TMxll_3D,
! src/FDTD/mxll_3D_mod.f90) with its time-step procedures replaced by calls into libomx_gpu.so.
! maxwell_factory (src/FDTD/factory_mod.f90:15-30) gains an arm that allocates this type; the
! driver loop (src/FDTD/mxim_mxll.f90:92-132) is unchanged.
!
! Uncompiled: there is no Fortran compiler in the build image of this library.  The calls it
! makes are declared in omx_gpu_mod.f90, which tests/test_fortran_binding.py checks against
! include/omx_gpu.h.
module mxll_3D_gpu_mod
    use iso_c_binding
    use constants_mod
    use mxll_base_mod
    use mxll_3D_mod
    use omx_gpu_mod
    implicit none

    type, extends(TMxll_3D) :: TMxll_3D_gpu
        type(c_ptr) :: ctx = c_null_ptr
    contains
        procedure :: init => init_3Dgrid_gpu
        procedure :: kill => kill_3Dgrid_gpu
        procedure :: td_propagate_H_field => td_propagate_H_3Dfield_gpu
        procedure :: td_propagate_E_field => td_propagate_E_3Dfield_gpu
    end type TMxll_3D_gpu

contains

    subroutine init_3Dgrid_gpu(this, grid_Ndims, npml, boundaries, dt, dr, mode, n_media, mpi_coords, mpi_dims)
        class(TMxll_3D_gpu), intent(inout) :: this
        integer, intent(in)  :: grid_Ndims(3), npml, boundaries(3), mode, n_media, mpi_coords(3), mpi_dims(3)
        real(dp), intent(in) :: dt, dr
        type(omx_grid_desc) :: d
        type(omx_medium), allocatable :: m(:)
        integer :: i, np
        ! host-side state exactly as the CPU type builds it (media, eps, CPML tables)
        call init_3Dgrid(this, grid_Ndims, npml, boundaries, dt, dr, mode, n_media, mpi_coords, mpi_dims)
        d%dimensions = 3
        d%grid_Ndims = grid_Ndims
        d%npml = npml
        d%boundaries = boundaries
        d%mode = mode
        d%precision = OMX_PREC_FP32          ! OMX_PREC_FP64 for the plain, bit-exact path
        d%dt = dt
        d%dr = dr
        call omx_check(omx_create(d, this%ctx))
        allocate(m(max(1, n_media)))
        do i = 1, n_media
            m(i)%medium_type = this%media(i)%medium_type
            m(i)%n_poles = 0
            m(i)%eps_r = this%media(i)%eps_r
            m(i)%A1 = this%media(i)%A1
            m(i)%A2 = this%media(i)%A2
            m(i)%C1 = this%media(i)%C1
            m(i)%C2 = this%media(i)%C2
            m(i)%C3 = this%media(i)%C3
            m(i)%C4 = this%media(i)%C4
            if (allocated(this%media(i)%alpha_k)) then
                np = min(this%media(i)%n_poles, OMX_MAX_POLES)
                m(i)%n_poles = np
                m(i)%alpha_k(1:np) = this%media(i)%alpha_k(1:np)
                m(i)%beta_k(1:np)  = this%media(i)%beta_k(1:np)
                m(i)%gamma_k(1:np) = this%media(i)%gamma_k(1:np)
                m(i)%B1_k(1:np)    = this%media(i)%B1_k(1:np)
                m(i)%B2_k(1:np)    = this%media(i)%B2_k(1:np)
            end if
        end do
        if (n_media > 0) then
            call omx_check(omx_set_media(this%ctx, n_media, m, this%media_map, this%eps_x, this%eps_y, this%eps_z))
        end if
    end subroutine init_3Dgrid_gpu

    ! td_propagate_H_3Dfield (mxll_3D_mod.f90:505-696)
    subroutine td_propagate_H_3Dfield_gpu(this)
        class(TMxll_3D_gpu), intent(inout) :: this
        call omx_check(omx_step_H(this%ctx))
    end subroutine td_propagate_H_3Dfield_gpu

    ! td_propagate_E_3Dfield (mxll_3D_mod.f90:700-923): the driver has set this%time and
    ! this%t_skip for the step (mxim_mxll.f90:93-104); t is the step index
    subroutine td_propagate_E_3Dfield_gpu(this, t)
        class(TMxll_3D_gpu), intent(inout) :: this
        integer, intent(in) :: t
        call omx_check(omx_step_E(this%ctx, real(this%time, c_double), real(this%t_skip, c_double)))
    end subroutine td_propagate_E_3Dfield_gpu

    subroutine kill_3Dgrid_gpu(this)
        class(TMxll_3D_gpu), intent(inout) :: this
        call omx_check(omx_destroy(this%ctx))
        this%ctx = c_null_ptr
        call kill_3Dgrid(this)
    end subroutine kill_3Dgrid_gpu

end module mxll_3D_gpu_mod
