! omx_gpu_mod.f90 -- iso_c_binding interface of libomx_gpu.so (include/omx_gpu.h) for the
! reference's Fortran time loop.  A maintainer adds this module (and mxll_3D_gpu_mod.f90) to
! src/FDTD and links the library.
!
! Uncompiled: there is no Fortran compiler in the build image of this library.  The derived
! types are checked against the C structs (sizes and field offsets) and every bound name and
! argument count against the C prototypes by tests/test_fortran_binding.py.
module omx_gpu_mod
    use iso_c_binding
    implicit none

    integer(c_int), parameter :: OMX_PREC_FP64 = 0, OMX_PREC_FP32 = 1
    integer(c_int), parameter :: OMX_MAX_POLES = 8

    ! TMxll%init arguments (mxll_base_mod.f90:41-57) plus the precision of the GPU path
    type, bind(C) :: omx_grid_desc
        integer(c_int) :: dimensions
        integer(c_int) :: grid_Ndims(3)
        integer(c_int) :: npml
        integer(c_int) :: boundaries(3)
        integer(c_int) :: mode
        integer(c_int) :: precision
        real(c_double) :: dt
        real(c_double) :: dr
    end type omx_grid_desc

    ! TClassicalMedium coefficients (classical_medium_mod.f90:6-37)
    type, bind(C) :: omx_medium
        integer(c_int) :: medium_type
        integer(c_int) :: n_poles
        real(c_double) :: eps_r
        real(c_double) :: A1, A2, C1, C2, C3, C4
        real(c_double) :: alpha_k(8), beta_k(8), gamma_k(8)
        real(c_double) :: B1_k(8), B2_k(8)
    end type omx_medium

    ! TSource (source_mod.f90:7-27), values in a.u.
    type, bind(C) :: omx_source_desc
        character(kind=c_char) :: dir
        real(c_double) :: j_amp, w0, t0, tau, t_init, t_final, phase
        real(c_double) :: r0(3)
        real(c_double) :: radius
        real(c_double) :: chirp
    end type omx_source_desc

    ! plane-wave soft source (no counterpart in the reference)
    type, bind(C) :: omx_plane_source_desc
        integer(c_int) :: comp
        integer(c_int) :: plane_axis
        integer(c_int) :: plane_index
        real(c_double) :: j_amp, w0, t0, tau, t_init, t_final, phase, chirp
    end type omx_plane_source_desc

    ! TQ_group (q_group_mod.f90:12-28) with a few-level emitter model
    type, bind(C) :: omx_qgroup_desc
        integer(c_int) :: group_type
        integer(c_int) :: model
        integer(c_int) :: n_systems
        real(c_double) :: density
        real(c_double) :: dt
    end type omx_qgroup_desc

    interface
        integer(c_int) function omx_select_device(device) bind(C, name="omx_select_device")
            import
            integer(c_int), value :: device
        end function
        integer(c_int) function omx_create(desc, ctx) bind(C, name="omx_create")
            import
            type(omx_grid_desc), intent(in) :: desc
            type(c_ptr) :: ctx
        end function
        integer(c_int) function omx_destroy(ctx) bind(C, name="omx_destroy")
            import
            type(c_ptr), value :: ctx
        end function
        integer(c_int) function omx_synchronize(ctx) bind(C, name="omx_synchronize")
            import
            type(c_ptr), value :: ctx
        end function
        type(c_ptr) function omx_last_error(ctx) bind(C, name="omx_last_error")
            import
            type(c_ptr), value :: ctx
        end function
        integer(c_int) function omx_set_cpml_tables(ctx, be, ce, bh, ch, den_ex, den_ey, den_ez, den_hx, &
                                                    den_hy, den_hz) bind(C, name="omx_set_cpml_tables")
            import
            type(c_ptr), value :: ctx
            real(c_double), intent(in) :: be(*), ce(*), bh(*), ch(*)
            real(c_double), intent(in) :: den_ex(*), den_ey(*), den_ez(*), den_hx(*), den_hy(*), den_hz(*)
        end function
        integer(c_int) function omx_set_media(ctx, n_media, media, media_map, eps_x, eps_y, eps_z) &
                bind(C, name="omx_set_media")
            import
            type(c_ptr), value :: ctx
            integer(c_int), value :: n_media
            type(omx_medium), intent(in) :: media(*)
            integer(c_int32_t), intent(in) :: media_map(*)
            real(c_double), intent(in) :: eps_x(*), eps_y(*), eps_z(*)
        end function
        integer(c_int) function omx_step_H(ctx) bind(C, name="omx_step_H")
            import
            type(c_ptr), value :: ctx
        end function
        integer(c_int) function omx_step_E(ctx, time, t_skip) bind(C, name="omx_step_E")
            import
            type(c_ptr), value :: ctx
            real(c_double), value :: time, t_skip
        end function
        integer(c_int) function omx_source_add(ctx, d, id) bind(C, name="omx_source_add")
            import
            type(c_ptr), value :: ctx
            type(omx_source_desc), intent(in) :: d
            integer(c_int) :: id
        end function
        integer(c_int) function omx_plane_source_add(ctx, d, id) bind(C, name="omx_plane_source_add")
            import
            type(c_ptr), value :: ctx
            type(omx_plane_source_desc), intent(in) :: d
            integer(c_int) :: id
        end function
        integer(c_int) function omx_source_interactions(ctx, time) bind(C, name="omx_source_interactions")
            import
            type(c_ptr), value :: ctx
            real(c_double), value :: time
        end function
        integer(c_int) function omx_qgroup_create(ctx, d, cell, params, id) bind(C, name="omx_qgroup_create")
            import
            type(c_ptr), value :: ctx
            type(omx_qgroup_desc), intent(in) :: d
            integer(c_int32_t), intent(in) :: cell(*)
            real(c_double), intent(in) :: params(*)
            integer(c_int) :: id
        end function
        integer(c_int) function omx_qgroup_step(ctx, id, tq_step) bind(C, name="omx_qgroup_step")
            import
            type(c_ptr), value :: ctx
            integer(c_int), value :: id, tq_step
        end function
        integer(c_int) function omx_qgroup_read(ctx, id, dipole, dpt_dt, efield, rho) bind(C, name="omx_qgroup_read")
            import
            type(c_ptr), value :: ctx
            integer(c_int), value :: id
            real(c_double) :: dipole(*), dpt_dt(*), efield(*), rho(*)
        end function
        integer(c_int) function omx_detector_add(ctx, dtype, field, nd, indx, id) bind(C, name="omx_detector_add")
            import
            type(c_ptr), value :: ctx
            integer(c_int), value :: dtype, field, nd
            integer(c_int32_t), intent(in) :: indx(*)
            integer(c_int) :: id
        end function
        integer(c_int) function omx_detectors_record(ctx, time) bind(C, name="omx_detectors_record")
            import
            type(c_ptr), value :: ctx
            real(c_double), value :: time
        end function
        integer(c_int) function omx_detectors_drain(ctx, times, values, max_rec, n_rec) &
                bind(C, name="omx_detectors_drain")
            import
            type(c_ptr), value :: ctx
            real(c_double) :: times(*), values(*)
            integer(c_int), value :: max_rec
            integer(c_int) :: n_rec
        end function
        integer(c_int) function omx_detectors_drain_async(ctx, ticket) bind(C, name="omx_detectors_drain_async")
            import
            type(c_ptr), value :: ctx
            integer(c_long_long) :: ticket
        end function
        integer(c_int) function omx_detectors_collect(ctx, ticket, times, values, max_rec, n_rec) &
                bind(C, name="omx_detectors_collect")
            import
            type(c_ptr), value :: ctx
            integer(c_long_long), value :: ticket
            real(c_double) :: times(*), values(*)
            integer(c_int), value :: max_rec
            integer(c_int) :: n_rec
        end function
        integer(c_int) function omx_run(ctx, tt0, nsteps, n_skip_steps, t_det_print, use_graph) bind(C, name="omx_run")
            import
            type(c_ptr), value :: ctx
            integer(c_int), value :: tt0, nsteps, n_skip_steps, t_det_print, use_graph
        end function
        integer(c_int) function omx_autotune(ctx, reps, choice) bind(C, name="omx_autotune")
            import
            type(c_ptr), value :: ctx
            integer(c_int), value :: reps
            integer(c_int) :: choice
        end function
        integer(c_int) function omx_read_field(ctx, field, host) bind(C, name="omx_read_field")
            import
            type(c_ptr), value :: ctx
            integer(c_int), value :: field
            real(c_double) :: host(*)
        end function
    end interface

contains

    ! the reference stops on errors; a non-zero status from the library does the same
    subroutine omx_check(rc)
        integer(c_int), intent(in) :: rc
        if (rc /= 0) then
            write(*, *) "omx_gpu error ", rc
            error stop
        end if
    end subroutine omx_check

end module omx_gpu_mod
