! dns3d_gpu -- ISO_C_BINDING interface to libdns3d_gpu.so (include/dns3d_capi.h)
!
! The module a maintainer adds beside DNS_pressure_BC_3D.f90 so that its time
! loop (DNS_pressure_BC_3D.f90:286-361) calls the GB300 step in place of its
! five internal subroutines (3D:314-326), in the style of the reference's own
! C binding to FFTW (fftw3_dns_module.f90:13-16).  Every function returns the
! library's status (0 = DNS3D_OK); the caller keeps the reference's `stop` at
! the call site.  Arrays u(nx,ny,nz) pass as they are: Fortran order is the
! library's layout.
!
! The derived types mirror the C structs field for field; tests/
! test_fortran_module.py checks their order and kinds, and every interface's
! name and argument count, against include/dns3d_capi.h.
!
! Link: gfortran -c fortran/dns3d_gpu.f90; gfortran ... DNS_pressure_BC_3D.f90 \
!       dns3d_gpu.o -Lf90_dns_gb300 -ldns3d_gpu -Wl,-rpath,<dir>
module dns3d_gpu
    use iso_c_binding
    implicit none

    integer(c_int), parameter :: DNS3D_OK = 0
    integer(c_int), parameter :: DNS3D_PREC_FP64 = 0, DNS3D_PREC_MIXED = 1

    ! read_input_3d namelist values (3D:559-603) and the extension keys
    type, bind(C) :: dns3d_config
        integer(c_int) :: nx, ny, nz
        integer(c_int) :: istart, nsteps, nwrt, restart_write_freq
        real(c_double) :: dt
        real(c_double) :: re, xlen, ylen, u_centerline
        integer(c_int) :: use_crank_nicolson
        integer(c_int) :: flow_control_method
        real(c_double) :: target_pressure_gradient, target_bulk_velocity, controller_gain
        integer(c_int) :: controller_update_freq
        integer(c_int) :: enable_perturbations
        real(c_double) :: perturbation_amplitude
        integer(c_int) :: zero_w_perturbations, use_analytical_perturbations
        integer(c_int) :: analytical_mode_x, analytical_mode_y
        integer(c_int) :: use_weak_form_divergence
        integer(c_int) :: use_dealias_23_rule
        integer(c_int) :: lgl_dmatrix_guard
        integer(c_int) :: precision
        integer(c_int) :: device
        integer(c_long_long) :: perturbation_seed
        integer(c_int) :: convection_scheme
        integer(c_int) :: linear_solver
        real(c_double) :: cgstol
        real(c_double) :: noise_amplitude
        integer(c_int) :: poisson_refinement
        integer(c_int) :: pad_
    end type dns3d_config

    ! PI controller globals (3D:75-89)
    type, bind(C) :: dns3d_pi_state
        real(c_double) :: current_pressure_gradient
        real(c_double) :: current_bulk_velocity
        real(c_double) :: bulk_velocity_error
        real(c_double) :: bulk_velocity_error_integral
        real(c_double) :: bulk_velocity_error_prev
        real(c_double) :: pressure_gradient_sum
        real(c_double) :: avg_pressure_gradient
        integer(c_int) :: pressure_gradient_count
        integer(c_int) :: pad_
    end type dns3d_pi_state

    ! output_diagnostics_3d (3D:2094-2146) and check_divergence_3d (3D:2171-2190)
    type, bind(C) :: dns3d_diag
        real(c_double) :: umax, vmax, wmax, energy
        real(c_double) :: u_bulk, dpdx, dpdx_avg
        real(c_double) :: max_div
        real(c_double) :: time
        integer(c_int) :: step
        integer(c_int) :: pad_
    end type dns3d_diag

    interface
        ! read_input_3d defaults (3D:571-603)
        integer(c_int) function dns3d_config_defaults(cfg) bind(C)
            import :: c_int, dns3d_config
            type(dns3d_config), intent(out) :: cfg
        end function

        ! read_input_3d (3D:554-708); path is NUL-terminated
        integer(c_int) function dns3d_config_read_namelist(path, cfg) bind(C)
            import :: c_char, c_int, dns3d_config
            character(kind=c_char), intent(in) :: path(*)
            type(dns3d_config), intent(inout) :: cfg
        end function

        ! setup_grid_3d, setup_spectral_3d, allocate_arrays_3d,
        ! initialize_fields_3d (3D:728-962)
        integer(c_int) function dns3d_create(cfg, h) bind(C)
            import :: c_int, c_ptr, dns3d_config
            type(dns3d_config), intent(in) :: cfg
            type(c_ptr), intent(out) :: h
        end function

        integer(c_int) function dns3d_destroy(h) bind(C)
            import :: c_int, c_ptr
            type(c_ptr), value :: h
        end function

        ! initialize_fields_3d (3D:909-962)
        integer(c_int) function dns3d_initialize_fields(h) bind(C)
            import :: c_int, c_ptr
            type(c_ptr), value :: h
        end function

        ! the globals u, v, w, p_total, grad_p_prev wall planes, PI state
        ! (3D:108-125); pass c_null_ptr (by value) to skip an argument
        integer(c_int) function dns3d_set_state(h, u, v, w, p, gx1, gx2, gy1, gy2, pi) bind(C)
            import :: c_int, c_ptr
            type(c_ptr), value :: h, u, v, w, p, gx1, gx2, gy1, gy2, pi
        end function

        integer(c_int) function dns3d_get_state(h, u, v, w, p, gx1, gx2, gy1, gy2, pi) bind(C)
            import :: c_int, c_ptr
            type(c_ptr), value :: h, u, v, w, p, gx1, gx2, gy1, gy2, pi
        end function

        integer(c_int) function dns3d_set_clock(h, step, time) bind(C)
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: h
            integer(c_int), value :: step
            real(c_double), value :: time
        end function

        ! the five subroutines of the time loop (3D:314-326), in order
        integer(c_int) function dns3d_compute_source_terms(h) bind(C)
            import :: c_int, c_ptr
            type(c_ptr), value :: h
        end function

        integer(c_int) function dns3d_viscous_step(h) bind(C)
            import :: c_int, c_ptr
            type(c_ptr), value :: h
        end function

        integer(c_int) function dns3d_solve_pressure(h) bind(C)
            import :: c_int, c_ptr
            type(c_ptr), value :: h
        end function

        integer(c_int) function dns3d_pressure_correction(h) bind(C)
            import :: c_int, c_ptr
            type(c_ptr), value :: h
        end function

        integer(c_int) function dns3d_apply_boundary_conditions(h) bind(C)
            import :: c_int, c_ptr
            type(c_ptr), value :: h
        end function

        ! nsteps loop bodies (3D:286-361 without IO), one graph replay each
        integer(c_int) function dns3d_step(h, nsteps) bind(C)
            import :: c_int, c_ptr
            type(c_ptr), value :: h
            integer(c_int), value :: nsteps
        end function

        integer(c_int) function dns3d_synchronize(h) bind(C)
            import :: c_int, c_ptr
            type(c_ptr), value :: h
        end function

        integer(c_int) function dns3d_diagnostics(h, d) bind(C)
            import :: c_int, c_ptr, dns3d_diag
            type(c_ptr), value :: h
            type(dns3d_diag), intent(out) :: d
        end function

        ! output_diagnostics_3d (3D:2094-2146)
        integer(c_int) function dns3d_output_diagnostics(h, d) bind(C)
            import :: c_int, c_ptr, dns3d_diag
            type(c_ptr), value :: h
            type(dns3d_diag), intent(out) :: d
        end function

        ! check_divergence_3d (3D:2171-2190)
        integer(c_int) function dns3d_check_divergence(h, max_div) bind(C)
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: h
            real(c_double), intent(out) :: max_div
        end function

        ! write_restart_file_3d / read_restart_file_3d (3D:2976-3209)
        integer(c_int) function dns3d_save_restart(h, path, istep, time) bind(C)
            import :: c_int, c_ptr, c_char, c_double
            type(c_ptr), value :: h
            character(kind=c_char), intent(in) :: path(*)
            integer(c_int), value :: istep
            real(c_double), value :: time
        end function

        integer(c_int) function dns3d_load_restart(h, path, istep, time) bind(C)
            import :: c_int, c_ptr, c_char, c_double
            type(c_ptr), value :: h
            character(kind=c_char), intent(in) :: path(*)
            integer(c_int), intent(out) :: istep
            real(c_double), intent(out) :: time
        end function

        ! write_time_series_data, write_flow_statistics,
        ! write_spanwise_averaged_profile, write_velocity_field_snapshot
        ! (3D:2702-2952) into the directory `dir`
        integer(c_int) function dns3d_write_time_series_data(h, dir) bind(C)
            import :: c_int, c_ptr, c_char
            type(c_ptr), value :: h
            character(kind=c_char), intent(in) :: dir(*)
        end function

        integer(c_int) function dns3d_write_flow_statistics(h, dir) bind(C)
            import :: c_int, c_ptr, c_char
            type(c_ptr), value :: h
            character(kind=c_char), intent(in) :: dir(*)
        end function

        integer(c_int) function dns3d_write_spanwise_averaged_profile(h, dir) bind(C)
            import :: c_int, c_ptr, c_char
            type(c_ptr), value :: h
            character(kind=c_char), intent(in) :: dir(*)
        end function

        integer(c_int) function dns3d_write_velocity_field_snapshot(h, dir) bind(C)
            import :: c_int, c_ptr, c_char
            type(c_ptr), value :: h
            character(kind=c_char), intent(in) :: dir(*)
        end function

        ! message of a status code (static C string)
        type(c_ptr) function dns3d_strerror(code) bind(C)
            import :: c_int, c_ptr
            integer(c_int), value :: code
        end function
    end interface
end module dns3d_gpu
