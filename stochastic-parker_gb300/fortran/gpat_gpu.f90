!*******************************************************************************
!< ISO_C_BINDING interface to the GB300 particle-mover engine
!< (include/gpat_engine.h).  Compiled into GPAT's own build, it lets
!< solve_transport_equation call the engine in place of the particle_module
!< and mhd_data_parallel procedures on the mover path; procedure names carry a
!< gpu_ prefix and the reference's argument lists.
!<
!< Particle records cross the boundary as structure-of-arrays: gpu_put_ptls /
!< gpu_get_ptls copy ptls(1:nptl_current) field by field.
!*******************************************************************************
module gpat_gpu
    use, intrinsic :: iso_c_binding
    implicit none
    private
    public gpat_mhd_config_t, gpat_params_t, gpat_local_dist_t
    public gpu_init, gpu_free, gpu_read_particle_params, gpu_calc_tstamps_mhd, &
        gpu_set_tstamps, gpu_read_field_data, gpu_calc_fields_gradients, &
        gpu_copy_fields, gpu_inject_particles_spatial_uniform, &
        gpu_inject_particles_at_x, gpu_particle_mover, gpu_split_particle, &
        gpu_global_distribution, gpu_pbins_edges, gpu_quick_check, &
        gpu_put_ptls, gpu_get_ptls, gpu_nptl_current, &
        gpu_inject_particles_at_large_jz, gpu_inject_particles_at_large_absj, &
        gpu_inject_particles_at_large_divv, gpu_inject_particles_at_large_rho, &
        gpu_inject_particles_at_large_db2, gpu_read_magnetic_fluctuation, &
        gpu_read_grid_positions, gpu_init_acc_surface, gpu_read_acc_surface, &
        gpu_read_correlation_length, &
        gpu_calc_escaped_distributions, gpu_reset_escaped_particles, &
        gpu_init_particle_tracking, gpu_read_particle_tracking, gpu_tracking_dims, &
        gpu_get_tracked_particles, gpu_free_particle_tracking, &
        gpu_load_tstamps_mhd, gpu_get_pmax_global, gpu_global_distribution_mu, &
        gpu_escaped_distribution_mu, gpu_local_distribution, gpu_local_escaped_distribution, &
        gpu_get_escaped_ptls, gpu_get_counters, gpu_set_counters, gpat_counters_t, &
        gpu_inject_particles_at_shock

    integer(c_int), parameter :: GPAT_OK = 0

    type, bind(c) :: gpat_mhd_config_t
        real(c_double) :: dx, dy, dz, xmin, ymin, zmin, xmax, ymax, zmax
        real(c_double) :: lx, ly, lz, dt_out
        integer(c_int32_t) :: nx, ny, nz, nxs, nys, nzs, topox, topoy, topoz
        integer(c_int32_t) :: nvar, bcx, bcy, bcz
    end type gpat_mhd_config_t

    type, bind(c) :: gpat_params_t
        real(c_double) :: b0, p0, pmin, pmax
        real(c_double) :: gamma_turb, pindex, kpara0, kret, dt_min_rel, dt_max_rel
        real(c_double) :: acc_region(6)
        real(c_double) :: drift1, drift2
        integer(c_int32_t) :: momentum_dependency, mag_dependency, acc_region_flag, charge
        integer(c_int32_t) :: check_drift_2d, ndim, pbcx, pbcy, pbcz, npp_global
        integer(c_int64_t) :: seed
        integer(c_int32_t) :: noise, precision
        integer(c_int64_t) :: nptl_max
        integer(c_int32_t) :: time_interp
        integer(c_int32_t) :: dpp_wave, dpp_shear, deltab_flag, correlation_flag
        integer(c_int32_t) :: include_3rd_dim, spherical_coord, nonuniform_grid
        integer(c_int32_t) :: bin_interval, weak_scattering
        real(c_double) :: duu0, tau0
    end type gpat_params_t

    type, bind(c) :: gpat_particles_t
        type(c_ptr) :: x, y, z, p, v, mu, weight, t, dt
        type(c_ptr) :: split_times, count_flag
        type(c_ptr) :: origin, nsteps_tracked, nsteps_pushed, tag_injected, tag_splitted
        type(c_ptr) :: rng_ctr
    end type gpat_particles_t

    !< One parameter set of the local distributions (pminK, pmaxK, npbinsK,
    !< nmuK, rxK, ryK, rzK of read_diagnostics_params).
    type, bind(c) :: gpat_local_dist_t
        real(c_double) :: pmin, pmax
        integer(c_int32_t) :: npbins, nmu, rx, ry, rz, reserved
    end type gpat_local_dist_t

    type, bind(c) :: gpat_counters_t
        integer(c_int64_t) :: nptl_current, nptl_split, nptl_escaped, tag_max
        real(c_double) :: leak, leak_negp
        integer(c_int64_t) :: leak_hi, leak_lo, leak_negp_hi, leak_negp_lo
        integer(c_int64_t) :: steps
        real(c_double) :: last_mover_ms
        integer(c_int64_t) :: last_mover_steps
        integer(c_int64_t) :: last_mover_launches
    end type gpat_counters_t

    interface
        integer(c_int) function c_read_particle_params(path, params) &
                bind(c, name="gpat_read_particle_params")
            import :: c_int, c_char, gpat_params_t
            character(kind=c_char), dimension(*), intent(in) :: path
            type(gpat_params_t), intent(inout) :: params
        end function
        integer(c_int) function c_create(params, cfg, device, handle) bind(c, name="gpat_create")
            import :: c_int, c_ptr, gpat_params_t, gpat_mhd_config_t
            type(gpat_params_t), intent(in) :: params
            type(gpat_mhd_config_t), intent(in) :: cfg
            integer(c_int), value :: device
            type(c_ptr), intent(out) :: handle
        end function
        integer(c_int) function c_destroy(handle) bind(c, name="gpat_destroy")
            import :: c_int, c_ptr
            type(c_ptr), value :: handle
        end function
        type(c_ptr) function c_last_error(handle) bind(c, name="gpat_last_error")
            import :: c_ptr
            type(c_ptr), value :: handle
        end function
        integer(c_int) function c_set_tstamps(handle, tstamps, n) bind(c, name="gpat_set_tstamps")
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: handle
            real(c_double), dimension(*), intent(in) :: tstamps
            integer(c_int), value :: n
        end function
        integer(c_int) function c_calc_tstamps_mhd(handle, t_start, t_end) &
                bind(c, name="gpat_calc_tstamps_mhd")
            import :: c_int, c_ptr
            type(c_ptr), value :: handle
            integer(c_int), value :: t_start, t_end
        end function
        integer(c_int) function c_read_field_data(handle, filename, var_flag) &
                bind(c, name="gpat_read_field_data")
            import :: c_int, c_ptr, c_char
            type(c_ptr), value :: handle
            character(kind=c_char), dimension(*), intent(in) :: filename
            integer(c_int), value :: var_flag
        end function
        integer(c_int) function c_init_acc_surface(handle, norm1, norm2, is_intersection) &
                bind(c, name="gpat_init_acc_surface")
            import :: c_int, c_ptr, c_char
            type(c_ptr), value :: handle
            character(kind=c_char), dimension(*), intent(in) :: norm1
            type(c_ptr), value :: norm2
            integer(c_int), value :: is_intersection
        end function
        integer(c_int) function c_read_acc_surface(handle, var_flag, file1, file2) &
                bind(c, name="gpat_read_acc_surface")
            import :: c_int, c_ptr, c_char
            type(c_ptr), value :: handle
            integer(c_int), value :: var_flag
            character(kind=c_char), dimension(*), intent(in) :: file1
            type(c_ptr), value :: file2
        end function
        integer(c_int) function c_read_grid_positions(handle, dirname) &
                bind(c, name="gpat_read_grid_positions")
            import :: c_int, c_ptr, c_char
            type(c_ptr), value :: handle
            character(kind=c_char), dimension(*), intent(in) :: dirname
        end function
        integer(c_int) function c_read_magnetic_fluctuation(handle, filename, var_flag) &
                bind(c, name="gpat_read_magnetic_fluctuation")
            import :: c_int, c_ptr, c_char
            type(c_ptr), value :: handle
            character(kind=c_char), dimension(*), intent(in) :: filename
            integer(c_int), value :: var_flag
        end function
        integer(c_int) function c_read_correlation_length(handle, filename, var_flag) &
                bind(c, name="gpat_read_correlation_length")
            import :: c_int, c_ptr, c_char
            type(c_ptr), value :: handle
            character(kind=c_char), dimension(*), intent(in) :: filename
            integer(c_int), value :: var_flag
        end function
        integer(c_int) function c_calc_fields_gradients(handle, var_flag) &
                bind(c, name="gpat_calc_fields_gradients")
            import :: c_int, c_ptr
            type(c_ptr), value :: handle
            integer(c_int), value :: var_flag
        end function
        integer(c_int) function c_copy_fields(handle) bind(c, name="gpat_copy_fields")
            import :: c_int, c_ptr
            type(c_ptr), value :: handle
        end function
        integer(c_int) function c_inject_uniform(handle, nptl, dt, dist_flag, particle_v0, &
                ct_mhd, part_box, power_index) bind(c, name="gpat_inject_particles_spatial_uniform")
            import :: c_int, c_ptr, c_double, c_int64_t
            type(c_ptr), value :: handle
            integer(c_int64_t), value :: nptl
            real(c_double), value :: dt, particle_v0, power_index
            integer(c_int), value :: dist_flag, ct_mhd
            real(c_double), dimension(6), intent(in) :: part_box
        end function
        integer(c_int) function c_inject_at_x(handle, nptl, xpos, dt, dist_flag, particle_v0, &
                ct_mhd, power_index) bind(c, name="gpat_inject_particles_at_x")
            import :: c_int, c_ptr, c_double, c_int64_t
            type(c_ptr), value :: handle
            integer(c_int64_t), value :: nptl
            real(c_double), value :: xpos, dt, particle_v0, power_index
            integer(c_int), value :: dist_flag, ct_mhd
        end function
        integer(c_int) function c_inject_at_large(handle, quantity, nptl, dt, dist_flag, &
                particle_v0, ct_mhd, inject_same_nptl, qmin, ncells_norm, part_box, &
                power_index, ninjected) bind(c, name="gpat_inject_particles_at_large")
            import :: c_int, c_ptr, c_double, c_int64_t
            type(c_ptr), value :: handle
            integer(c_int), value :: quantity, dist_flag, ct_mhd, inject_same_nptl
            integer(c_int64_t), value :: nptl, ncells_norm
            real(c_double), value :: dt, particle_v0, qmin, power_index
            real(c_double), dimension(6), intent(in) :: part_box
            integer(c_int64_t), intent(out) :: ninjected
        end function
        integer(c_int) function c_escaped_distributions(handle, fescaped, counts) &
                bind(c, name="gpat_calc_escaped_distributions")
            import :: c_int, c_ptr, c_double, c_int64_t
            type(c_ptr), value :: handle
            real(c_double), dimension(*), intent(out) :: fescaped
            integer(c_int64_t), dimension(*), intent(out) :: counts
        end function
        integer(c_int) function c_reset_escaped(handle) bind(c, name="gpat_reset_escaped_particles")
            import :: c_int, c_ptr
            type(c_ptr), value :: handle
        end function
        integer(c_int) function c_particle_mover(handle, focused_transport, nlgc, kperp_kpara, &
                nsteps_interval, mhd_tframe, num_fine_steps, dump_escaped_dist) &
                bind(c, name="gpat_particle_mover")
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: handle
            integer(c_int), value :: focused_transport, nlgc, nsteps_interval, mhd_tframe
            integer(c_int), value :: num_fine_steps, dump_escaped_dist
            real(c_double), value :: kperp_kpara
        end function
        integer(c_int) function c_split_particle(handle, split_ratio, pmin_split, &
                nsteps_interval) bind(c, name="gpat_split_particle")
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: handle
            real(c_double), value :: split_ratio, pmin_split
            integer(c_int), value :: nsteps_interval
        end function
        integer(c_int) function c_distributions(handle, fglobal, counts) &
                bind(c, name="gpat_calc_particle_distributions")
            import :: c_int, c_ptr, c_double, c_int64_t
            type(c_ptr), value :: handle
            real(c_double), dimension(*), intent(out) :: fglobal
            integer(c_int64_t), dimension(*), intent(out) :: counts
        end function
        integer(c_int) function c_pbins_edges(handle, edges) bind(c, name="gpat_pbins_edges")
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: handle
            real(c_double), dimension(*), intent(out) :: edges
        end function
        integer(c_int) function c_quick_check(handle, out) bind(c, name="gpat_quick_check")
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: handle
            real(c_double), dimension(8), intent(out) :: out
        end function
        integer(c_int) function c_put_particles(handle, src, n) bind(c, name="gpat_put_particles")
            import :: c_int, c_ptr, c_int64_t, gpat_particles_t
            type(c_ptr), value :: handle
            type(gpat_particles_t), intent(in) :: src
            integer(c_int64_t), value :: n
        end function
        integer(c_int) function c_get_particles(handle, dst, capacity, n) &
                bind(c, name="gpat_get_particles")
            import :: c_int, c_ptr, c_int64_t, gpat_particles_t
            type(c_ptr), value :: handle
            type(gpat_particles_t), intent(inout) :: dst
            integer(c_int64_t), value :: capacity
            integer(c_int64_t), intent(out) :: n
        end function
        integer(c_int) function c_get_counters(handle, out) bind(c, name="gpat_get_counters")
            import :: c_int, c_ptr, gpat_counters_t
            type(c_ptr), value :: handle
            type(gpat_counters_t), intent(out) :: out
        end function
        integer(c_int) function c_init_tracking(handle, tags, nrows, nptl_tracking, &
                nsteps_interval) bind(c, name="gpat_init_particle_tracking")
            import :: c_int, c_ptr, c_int32_t
            type(c_ptr), value :: handle
            integer(c_int32_t), dimension(*), intent(in) :: tags
            integer(c_int32_t), value :: nrows, nptl_tracking, nsteps_interval
        end function
        integer(c_int) function c_read_tracking(handle, filename, nsteps_interval) &
                bind(c, name="gpat_read_particle_tracking")
            import :: c_int, c_ptr, c_char, c_int32_t
            type(c_ptr), value :: handle
            character(kind=c_char), dimension(*), intent(in) :: filename
            integer(c_int32_t), value :: nsteps_interval
        end function
        integer(c_int) function c_tracking_dims(handle, nsteps, nptl_tracking, dropped) &
                bind(c, name="gpat_tracking_dims")
            import :: c_int, c_ptr, c_int32_t, c_int64_t
            type(c_ptr), value :: handle
            integer(c_int64_t), intent(out) :: nsteps, dropped
            integer(c_int32_t), intent(out) :: nptl_tracking
        end function
        integer(c_int) function c_get_tracked(handle, dst) &
                bind(c, name="gpat_get_tracked_particles")
            import :: c_int, c_ptr, gpat_particles_t
            type(c_ptr), value :: handle
            type(gpat_particles_t), intent(inout) :: dst
        end function
        integer(c_int) function c_free_tracking(handle) bind(c, name="gpat_free_particle_tracking")
            import :: c_int, c_ptr
            type(c_ptr), value :: handle
        end function
        integer(c_int) function c_load_tstamps(handle, t_start, t_end, tmax_mhd, dirname) &
                bind(c, name="gpat_load_tstamps_mhd")
            import :: c_int, c_ptr, c_char
            type(c_ptr), value :: handle
            integer(c_int), value :: t_start, t_end, tmax_mhd
            character(kind=c_char), dimension(*), intent(in) :: dirname
        end function
        integer(c_int) function c_pmax(handle, pmax) bind(c, name="gpat_get_pmax_global")
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: handle
            real(c_double), intent(out) :: pmax
        end function
        integer(c_int) function c_distributions_mu(handle, nmu, f, counts) &
                bind(c, name="gpat_calc_particle_distributions_mu")
            import :: c_int, c_ptr, c_int32_t, c_double, c_int64_t
            type(c_ptr), value :: handle
            integer(c_int32_t), value :: nmu
            real(c_double), dimension(*), intent(out) :: f
            integer(c_int64_t), dimension(*), intent(out) :: counts
        end function
        integer(c_int) function c_escaped_mu(handle, nmu, f, counts) &
                bind(c, name="gpat_calc_escaped_distributions_mu")
            import :: c_int, c_ptr, c_int32_t, c_double, c_int64_t
            type(c_ptr), value :: handle
            integer(c_int32_t), value :: nmu
            real(c_double), dimension(*), intent(out) :: f
            integer(c_int64_t), dimension(*), intent(out) :: counts
        end function
        integer(c_int) function c_local_dist(handle, spec, flocal, counts) &
                bind(c, name="gpat_calc_local_distribution")
            import :: c_int, c_ptr, c_double, c_int64_t, gpat_local_dist_t
            type(c_ptr), value :: handle
            type(gpat_local_dist_t), intent(in) :: spec
            real(c_double), dimension(*), intent(out) :: flocal
            integer(c_int64_t), dimension(*), intent(out) :: counts
        end function
        integer(c_int) function c_local_escaped(handle, spec, fx, fy, fz, cx, cy, cz) &
                bind(c, name="gpat_calc_local_escaped_distribution")
            import :: c_int, c_ptr, gpat_local_dist_t
            type(c_ptr), value :: handle
            type(gpat_local_dist_t), intent(in) :: spec
            type(c_ptr), value :: fx, fy, fz, cx, cy, cz
        end function
        integer(c_int) function c_get_escaped(handle, dst, capacity, n) &
                bind(c, name="gpat_get_escaped_particles")
            import :: c_int, c_ptr, c_int64_t, gpat_particles_t
            type(c_ptr), value :: handle
            type(gpat_particles_t), intent(inout) :: dst
            integer(c_int64_t), value :: capacity
            integer(c_int64_t), intent(out) :: n
        end function
        integer(c_int) function c_inject_at_shock(handle, nptl, dt, dist_flag, particle_v0, &
                ct_mhd, power_index) bind(c, name="gpat_inject_particles_at_shock")
            import :: c_int, c_ptr, c_int64_t, c_double
            type(c_ptr), value :: handle
            integer(c_int64_t), value :: nptl
            real(c_double), value :: dt, particle_v0, power_index
            integer(c_int), value :: dist_flag, ct_mhd
        end function
        integer(c_int) function c_set_counters(handle, in) bind(c, name="gpat_set_counters")
            import :: c_int, c_ptr, gpat_counters_t
            type(c_ptr), value :: handle
            type(gpat_counters_t), intent(in) :: in
        end function
    end interface

    type(c_ptr), save :: h = c_null_ptr

    contains

    subroutine check(rc, what)
        integer(c_int), intent(in) :: rc
        character(*), intent(in) :: what
        character(kind=c_char), pointer :: msg(:)
        integer :: i
        if (rc == GPAT_OK) return
        call c_f_pointer(c_last_error(h), msg, [256])
        write(*, "(A,A,I0)", advance="no") "gpat_gpu: ", what//" failed, code ", rc
        write(*, "(A)", advance="no") ": "
        do i = 1, 256
            if (msg(i) == c_null_char) exit
            write(*, "(A)", advance="no") msg(i)
        enddo
        write(*, *)
        stop 1
    end subroutine check

    !< init_particles + init_field_data + init_particle_distributions
    subroutine gpu_init(params, cfg, device)
        type(gpat_params_t), intent(in) :: params
        type(gpat_mhd_config_t), intent(in) :: cfg
        integer, intent(in) :: device
        call check(c_create(params, cfg, int(device, c_int), h), "gpat_create")
    end subroutine gpu_init

    subroutine gpu_free
        integer(c_int) :: rc
        if (c_associated(h)) rc = c_destroy(h)
        h = c_null_ptr
    end subroutine gpu_free

    !< read_particle_params (particle_module.f90:2778-2878)
    subroutine gpu_read_particle_params(conf_file, params)
        character(*), intent(in) :: conf_file
        type(gpat_params_t), intent(inout) :: params
        call check(c_read_particle_params(trim(conf_file)//c_null_char, params), &
            "read_particle_params")
    end subroutine gpu_read_particle_params

    !< calc_tstamps_mhd (mhd_config.f90:263-271)
    subroutine gpu_calc_tstamps_mhd(t_start, t_end)
        integer, intent(in) :: t_start, t_end
        call check(c_calc_tstamps_mhd(h, int(t_start, c_int), int(t_end, c_int)), "calc_tstamps")
    end subroutine gpu_calc_tstamps_mhd

    !< tstamps_mhd from load_tstamps_mhd (mhd_config.f90:218-255)
    subroutine gpu_set_tstamps(tstamps)
        real(c_double), dimension(:), intent(in) :: tstamps
        call check(c_set_tstamps(h, tstamps, int(size(tstamps), c_int)), "set_tstamps")
    end subroutine gpu_set_tstamps

    !< read_field_data_parallel (mhd_data_parallel.f90:224-300)
    subroutine gpu_read_field_data(filename, var_flag)
        character(*), intent(in) :: filename
        integer, intent(in) :: var_flag
        call check(c_read_field_data(h, trim(filename)//c_null_char, int(var_flag, c_int)), &
            "read_field_data")
    end subroutine gpu_read_field_data

    !< set_local_grid_positions for uniform_grid = 0 (mhd_data_parallel.f90:
    !< 2087-2190): xpos.dat, ypos.dat, zpos.dat in dir_mhd_data
    subroutine gpu_read_grid_positions(dir_mhd_data)
        character(*), intent(in) :: dir_mhd_data
        call check(c_read_grid_positions(h, trim(dir_mhd_data)//c_null_char), &
            "read_grid_positions")
    end subroutine gpu_read_grid_positions

    !< init_acc_surface (acc_region_surface.f90:27-93): norm2 and
    !< is_intersection only for a second surface
    subroutine gpu_init_acc_surface(surface_norm1, surface_norm2, is_intersection)
        character(*), intent(in) :: surface_norm1
        character(*), intent(in), optional :: surface_norm2
        logical, intent(in), optional :: is_intersection
        character(kind=c_char, len=3), target :: n2
        type(c_ptr) :: p2
        integer(c_int) :: inter
        p2 = c_null_ptr
        inter = 1
        if (present(surface_norm2)) then
            n2 = surface_norm2(1:2)//c_null_char
            p2 = c_loc(n2)
        endif
        if (present(is_intersection)) inter = merge(1_c_int, 0_c_int, is_intersection)
        call check(c_init_acc_surface(h, surface_norm1(1:2)//c_null_char, p2, inter), &
            "init_acc_surface")
    end subroutine gpu_init_acc_surface

    !< read_acc_surface (acc_region_surface.f90:112-249)
    subroutine gpu_read_acc_surface(var_flag, filename1, filename2)
        integer, intent(in) :: var_flag
        character(*), intent(in) :: filename1
        character(*), intent(in), optional :: filename2
        character(kind=c_char, len=:), allocatable, target :: f2
        type(c_ptr) :: p2
        p2 = c_null_ptr
        if (present(filename2)) then
            f2 = trim(filename2)//c_null_char
            p2 = c_loc(f2)
        endif
        call check(c_read_acc_surface(h, int(var_flag, c_int), trim(filename1)//c_null_char, &
            p2), "read_acc_surface")
    end subroutine gpu_read_acc_surface

    !< read_magnetic_fluctuation + calc_grad_sigma2_slab/_2d
    !< (mhd_data_parallel.f90:306-397, stochastic-mhd.f90:337-361)
    subroutine gpu_read_magnetic_fluctuation(filename, var_flag)
        character(*), intent(in) :: filename
        integer, intent(in) :: var_flag
        call check(c_read_magnetic_fluctuation(h, trim(filename)//c_null_char, &
            int(var_flag, c_int)), "read_magnetic_fluctuation")
    end subroutine gpu_read_magnetic_fluctuation

    !< read_correlation_length + calc_grad_lc_slab/_2d
    !< (mhd_data_parallel.f90:406-497, stochastic-mhd.f90:342-371)
    subroutine gpu_read_correlation_length(filename, var_flag)
        character(*), intent(in) :: filename
        integer, intent(in) :: var_flag
        call check(c_read_correlation_length(h, trim(filename)//c_null_char, &
            int(var_flag, c_int)), "read_correlation_length")
    end subroutine gpu_read_correlation_length

    !< calc_fields_gradients (mhd_data_parallel.f90:504-610)
    subroutine gpu_calc_fields_gradients(var_flag)
        integer, intent(in) :: var_flag
        call check(c_calc_fields_gradients(h, int(var_flag, c_int)), "calc_fields_gradients")
    end subroutine gpu_calc_fields_gradients

    !< copy_fields (mhd_data_parallel.f90:1920-1926)
    subroutine gpu_copy_fields
        call check(c_copy_fields(h), "copy_fields")
    end subroutine gpu_copy_fields

    !< inject_particles_spatial_uniform (particle_module.f90:454-530)
    subroutine gpu_inject_particles_spatial_uniform(nptl, dt, dist_flag, particle_v0, &
            ct_mhd, part_box, power_index)
        integer, intent(in) :: nptl, dist_flag, ct_mhd
        real(8), intent(in) :: dt, particle_v0, power_index
        real(8), dimension(6), intent(in) :: part_box
        call check(c_inject_uniform(h, int(nptl, c_int64_t), dt, int(dist_flag, c_int), &
            particle_v0, int(ct_mhd, c_int), part_box, power_index), "inject_uniform")
    end subroutine gpu_inject_particles_spatial_uniform

    !< Injection on the plane x = xpos (inject_particles_at_shock draw order)
    subroutine gpu_inject_particles_at_x(nptl, xpos, dt, dist_flag, particle_v0, ct_mhd, &
            power_index)
        integer, intent(in) :: nptl, dist_flag, ct_mhd
        real(8), intent(in) :: xpos, dt, particle_v0, power_index
        call check(c_inject_at_x(h, int(nptl, c_int64_t), xpos, dt, int(dist_flag, c_int), &
            particle_v0, int(ct_mhd, c_int), power_index), "inject_at_x")
    end subroutine gpu_inject_particles_at_x

    !< inject_particles_at_large_jz / _absj / _divv / _rho / _db2
    !< (particle_module.f90:785-1468), same arguments
    subroutine inject_large(quantity, nptl, dt, dist_flag, particle_v0, ct_mhd, &
            inject_same_nptl, qmin, ncells_norm, part_box, power_index)
        integer, intent(in) :: quantity, nptl, dist_flag, ct_mhd, ncells_norm
        logical, intent(in) :: inject_same_nptl
        real(8), intent(in) :: dt, particle_v0, qmin, power_index
        real(8), dimension(6), intent(in) :: part_box
        integer(c_int64_t) :: ninjected
        call check(c_inject_at_large(h, int(quantity, c_int), int(nptl, c_int64_t), dt, &
            int(dist_flag, c_int), particle_v0, int(ct_mhd, c_int), &
            merge(1_c_int, 0_c_int, inject_same_nptl), qmin, int(ncells_norm, c_int64_t), &
            part_box, power_index, ninjected), "inject_particles_at_large")
    end subroutine inject_large

    subroutine gpu_inject_particles_at_large_jz(nptl, dt, dist_flag, particle_v0, ct_mhd, &
            inject_same_nptl, jz_min, ncells_large_jz_norm, part_box, power_index)
        integer, intent(in) :: nptl, dist_flag, ct_mhd, ncells_large_jz_norm
        logical, intent(in) :: inject_same_nptl
        real(8), intent(in) :: dt, particle_v0, jz_min, power_index
        real(8), dimension(6), intent(in) :: part_box
        call inject_large(0, nptl, dt, dist_flag, particle_v0, ct_mhd, inject_same_nptl, &
            jz_min, ncells_large_jz_norm, part_box, power_index)
    end subroutine gpu_inject_particles_at_large_jz

    subroutine gpu_inject_particles_at_large_absj(nptl, dt, dist_flag, particle_v0, ct_mhd, &
            inject_same_nptl, absj_min, ncells_large_absj_norm, part_box, power_index)
        integer, intent(in) :: nptl, dist_flag, ct_mhd, ncells_large_absj_norm
        logical, intent(in) :: inject_same_nptl
        real(8), intent(in) :: dt, particle_v0, absj_min, power_index
        real(8), dimension(6), intent(in) :: part_box
        call inject_large(1, nptl, dt, dist_flag, particle_v0, ct_mhd, inject_same_nptl, &
            absj_min, ncells_large_absj_norm, part_box, power_index)
    end subroutine gpu_inject_particles_at_large_absj

    subroutine gpu_inject_particles_at_large_divv(nptl, dt, dist_flag, particle_v0, ct_mhd, &
            inject_same_nptl, divv_min, ncells_large_divv_norm, part_box, power_index)
        integer, intent(in) :: nptl, dist_flag, ct_mhd, ncells_large_divv_norm
        logical, intent(in) :: inject_same_nptl
        real(8), intent(in) :: dt, particle_v0, divv_min, power_index
        real(8), dimension(6), intent(in) :: part_box
        call inject_large(2, nptl, dt, dist_flag, particle_v0, ct_mhd, inject_same_nptl, &
            divv_min, ncells_large_divv_norm, part_box, power_index)
    end subroutine gpu_inject_particles_at_large_divv

    subroutine gpu_inject_particles_at_large_rho(nptl, dt, dist_flag, particle_v0, ct_mhd, &
            inject_same_nptl, rho_min, ncells_large_rho_norm, part_box, power_index)
        integer, intent(in) :: nptl, dist_flag, ct_mhd, ncells_large_rho_norm
        logical, intent(in) :: inject_same_nptl
        real(8), intent(in) :: dt, particle_v0, rho_min, power_index
        real(8), dimension(6), intent(in) :: part_box
        call inject_large(3, nptl, dt, dist_flag, particle_v0, ct_mhd, inject_same_nptl, &
            rho_min, ncells_large_rho_norm, part_box, power_index)
    end subroutine gpu_inject_particles_at_large_rho

    subroutine gpu_inject_particles_at_large_db2(nptl, dt, dist_flag, particle_v0, ct_mhd, &
            inject_same_nptl, db2_min, ncells_large_db2_norm, part_box, power_index)
        integer, intent(in) :: nptl, dist_flag, ct_mhd, ncells_large_db2_norm
        logical, intent(in) :: inject_same_nptl
        real(8), intent(in) :: dt, particle_v0, db2_min, power_index
        real(8), dimension(6), intent(in) :: part_box
        call inject_large(4, nptl, dt, dist_flag, particle_v0, ct_mhd, inject_same_nptl, &
            db2_min, ncells_large_db2_norm, part_box, power_index)
    end subroutine gpu_inject_particles_at_large_db2

    !< calc_escaped_distributions (diagnostics.f90:913-960): fescaped(npp, 2*ndim)
    subroutine gpu_calc_escaped_distributions(fescaped, counts)
        real(8), dimension(:, :), intent(out) :: fescaped
        integer(8), dimension(:, :), intent(out) :: counts
        call check(c_escaped_distributions(h, fescaped, counts), "calc_escaped_distributions")
    end subroutine gpu_calc_escaped_distributions

    !< reset_escaped_particles
    subroutine gpu_reset_escaped_particles
        call check(c_reset_escaped(h), "reset_escaped_particles")
    end subroutine gpu_reset_escaped_particles

    !< particle_mover (particle_module.f90:1846-1974), same arguments
    subroutine gpu_particle_mover(focused_transport, nlgc, kperp_kpara, nsteps_interval, &
            mhd_tframe, num_fine_steps, dump_escaped_dist)
        logical, intent(in) :: focused_transport, nlgc, dump_escaped_dist
        real(8), intent(in) :: kperp_kpara
        integer, intent(in) :: nsteps_interval, mhd_tframe, num_fine_steps
        call check(c_particle_mover(h, merge(1_c_int, 0_c_int, focused_transport), &
            merge(1_c_int, 0_c_int, nlgc), kperp_kpara, int(nsteps_interval, c_int), &
            int(mhd_tframe, c_int), int(num_fine_steps, c_int), &
            merge(1_c_int, 0_c_int, dump_escaped_dist)), "particle_mover")
    end subroutine gpu_particle_mover

    !< split_particle (particle_module.f90:5430-5480), same arguments
    subroutine gpu_split_particle(split_ratio, pmin_split, nsteps_interval)
        real(8), intent(in) :: split_ratio, pmin_split
        integer, intent(in) :: nsteps_interval
        call check(c_split_particle(h, split_ratio, pmin_split, int(nsteps_interval, c_int)), &
            "split_particle")
    end subroutine gpu_split_particle

    !< fglobal(1, :) of calc_particle_distributions (diagnostics.f90:738-780)
    subroutine gpu_global_distribution(fglobal, counts)
        real(c_double), dimension(:), intent(out) :: fglobal
        integer(c_int64_t), dimension(:), intent(out) :: counts
        call check(c_distributions(h, fglobal, counts), "calc_particle_distributions")
    end subroutine gpu_global_distribution

    !< pbins_edges_global (diagnostics.f90:194-204)
    subroutine gpu_pbins_edges(edges)
        real(c_double), dimension(:), intent(out) :: edges
        call check(c_pbins_edges(h, edges), "pbins_edges")
    end subroutine gpu_pbins_edges

    !< quick_check sums (diagnostics.f90:116-170)
    subroutine gpu_quick_check(out)
        real(c_double), dimension(8), intent(out) :: out
        call check(c_quick_check(h, out), "quick_check")
    end subroutine gpu_quick_check

    integer function gpu_nptl_current()
        type(gpat_counters_t) :: c
        call check(c_get_counters(h, c), "get_counters")
        gpu_nptl_current = int(c%nptl_current)
    end function gpu_nptl_current

    !< Copies particle arrays (structure of arrays, length n) to the engine.
    subroutine gpu_put_ptls(n, x, y, z, p, v, mu, weight, t, dt, split_times, count_flag, &
            origin, nsteps_tracked, nsteps_pushed, tag_injected, tag_splitted, rng_ctr)
        integer, intent(in) :: n
        real(c_double), dimension(n), intent(in), target :: x, y, z, p, v, mu, weight, t, dt
        integer(c_int8_t), dimension(n), intent(in), target :: split_times, count_flag
        integer(c_int32_t), dimension(n), intent(in), target :: origin, nsteps_tracked, &
            nsteps_pushed, tag_injected, tag_splitted, rng_ctr
        type(gpat_particles_t) :: s
        s%x = c_loc(x); s%y = c_loc(y); s%z = c_loc(z); s%p = c_loc(p); s%v = c_loc(v)
        s%mu = c_loc(mu); s%weight = c_loc(weight); s%t = c_loc(t); s%dt = c_loc(dt)
        s%split_times = c_loc(split_times); s%count_flag = c_loc(count_flag)
        s%origin = c_loc(origin); s%nsteps_tracked = c_loc(nsteps_tracked)
        s%nsteps_pushed = c_loc(nsteps_pushed); s%tag_injected = c_loc(tag_injected)
        s%tag_splitted = c_loc(tag_splitted); s%rng_ctr = c_loc(rng_ctr)
        call check(c_put_particles(h, s, int(n, c_int64_t)), "put_particles")
    end subroutine gpu_put_ptls

    !< Copies the engine's particles into arrays of length capacity; n on exit.
    subroutine gpu_get_ptls(capacity, n, x, y, z, p, v, mu, weight, t, dt, split_times, &
            count_flag, origin, nsteps_tracked, nsteps_pushed, tag_injected, tag_splitted, rng_ctr)
        integer, intent(in) :: capacity
        integer, intent(out) :: n
        real(c_double), dimension(capacity), intent(out), target :: x, y, z, p, v, mu, weight, &
            t, dt
        integer(c_int8_t), dimension(capacity), intent(out), target :: split_times, count_flag
        integer(c_int32_t), dimension(capacity), intent(out), target :: origin, nsteps_tracked, &
            nsteps_pushed, tag_injected, tag_splitted, rng_ctr
        type(gpat_particles_t) :: s
        integer(c_int64_t) :: got
        s%x = c_loc(x); s%y = c_loc(y); s%z = c_loc(z); s%p = c_loc(p); s%v = c_loc(v)
        s%mu = c_loc(mu); s%weight = c_loc(weight); s%t = c_loc(t); s%dt = c_loc(dt)
        s%split_times = c_loc(split_times); s%count_flag = c_loc(count_flag)
        s%origin = c_loc(origin); s%nsteps_tracked = c_loc(nsteps_tracked)
        s%nsteps_pushed = c_loc(nsteps_pushed); s%tag_injected = c_loc(tag_injected)
        s%tag_splitted = c_loc(tag_splitted); s%rng_ctr = c_loc(rng_ctr)
        call check(c_get_particles(h, s, int(capacity, c_int64_t), got), "get_particles")
        n = int(got)
    end subroutine gpu_get_ptls

    !< init_particle_tracking (particle_module.f90:5825-5877) from the
    !< tags_tracking table itself, (split_times_max + 2, nptl_tracking)
    subroutine gpu_init_particle_tracking(tags_tracking, nsteps_interval)
        integer(c_int32_t), dimension(:, :), intent(in) :: tags_tracking
        integer, intent(in) :: nsteps_interval
        call check(c_init_tracking(h, tags_tracking, int(size(tags_tracking, 1), c_int32_t), &
            int(size(tags_tracking, 2), c_int32_t), int(nsteps_interval, c_int32_t)), &
            "init_particle_tracking")
    end subroutine gpu_init_particle_tracking

    !< init_particle_tracking from a raw tags file (int32 nrows, int32
    !< nptl_tracking, then the table)
    subroutine gpu_read_particle_tracking(particle_tags_file, nsteps_interval)
        character(*), intent(in) :: particle_tags_file
        integer, intent(in) :: nsteps_interval
        call check(c_read_tracking(h, trim(particle_tags_file)//c_null_char, &
            int(nsteps_interval, c_int32_t)), "init_particle_tracking")
    end subroutine gpu_read_particle_tracking

    !< nsteps_tracking_max and nptl_tracking, the shape of particles_tracked
    subroutine gpu_tracking_dims(nsteps_tracking_max, nptl_tracking)
        integer, intent(out) :: nsteps_tracking_max, nptl_tracking
        integer(c_int64_t) :: nsteps, dropped
        integer(c_int32_t) :: ntrk
        call check(c_tracking_dims(h, nsteps, ntrk, dropped), "tracking_dims")
        nsteps_tracking_max = int(nsteps)
        nptl_tracking = int(ntrk)
    end subroutine gpu_tracking_dims

    !< sync_tracked_particles and the datasets of dump_tracked_particles
    !< (:5994-6030, :6235-6299): particles_tracked(nsteps_tracking_max,
    !< nptl_tracking) field by field
    subroutine gpu_get_tracked_particles(x, y, z, p, v, mu, weight, t, dt, split_times, &
            count_flag, origin, nsteps_tracked, nsteps_pushed, tag_injected, tag_splitted)
        real(c_double), dimension(:, :), intent(out), target, contiguous :: x, y, z, p, v, mu, &
            weight, t, dt
        integer(c_int8_t), dimension(:, :), intent(out), target, contiguous :: split_times, &
            count_flag
        integer(c_int32_t), dimension(:, :), intent(out), target, contiguous :: origin, &
            nsteps_tracked, nsteps_pushed, tag_injected, tag_splitted
        type(gpat_particles_t) :: s
        s%x = c_loc(x); s%y = c_loc(y); s%z = c_loc(z); s%p = c_loc(p); s%v = c_loc(v)
        s%mu = c_loc(mu); s%weight = c_loc(weight); s%t = c_loc(t); s%dt = c_loc(dt)
        s%split_times = c_loc(split_times); s%count_flag = c_loc(count_flag)
        s%origin = c_loc(origin); s%nsteps_tracked = c_loc(nsteps_tracked)
        s%nsteps_pushed = c_loc(nsteps_pushed); s%tag_injected = c_loc(tag_injected)
        s%tag_splitted = c_loc(tag_splitted); s%rng_ctr = c_null_ptr
        call check(c_get_tracked(h, s), "dump_tracked_particles")
    end subroutine gpu_get_tracked_particles

    !< locate_shock_xpos + inject_particles_at_shock (particle_module.f90:
    !< 542-633), same arguments
    subroutine gpu_inject_particles_at_shock(nptl, dt, dist_flag, particle_v0, ct_mhd, &
            power_index)
        integer, intent(in) :: nptl, dist_flag, ct_mhd
        real(8), intent(in) :: dt, particle_v0, power_index
        call check(c_inject_at_shock(h, int(nptl, c_int64_t), dt, int(dist_flag, c_int), &
            particle_v0, int(ct_mhd, c_int), power_index), "inject_particles_at_shock")
    end subroutine gpu_inject_particles_at_shock

    !< load_tstamps_mhd (mhd_config.f90:221-255) for varying_dt_mhd
    subroutine gpu_load_tstamps_mhd(t_start, t_end, tmax_mhd, dir_mhd_data)
        integer, intent(in) :: t_start, t_end, tmax_mhd
        character(*), intent(in) :: dir_mhd_data
        call check(c_load_tstamps(h, int(t_start, c_int), int(t_end, c_int), &
            int(tmax_mhd, c_int), trim(dir_mhd_data)//c_null_char), "load_tstamps_mhd")
    end subroutine gpu_load_tstamps_mhd

    !< get_pmax_global (diagnostics.f90:1691-1721) without the file
    subroutine gpu_get_pmax_global(pmax)
        real(c_double), intent(out) :: pmax
        call check(c_pmax(h, pmax), "get_pmax_global")
    end subroutine gpu_get_pmax_global

    !< fglobal(nmu_global, npp_global) of calc_particle_distributions
    !< (diagnostics.f90:773-779)
    subroutine gpu_global_distribution_mu(fglobal, counts)
        real(c_double), dimension(:, :), intent(out) :: fglobal
        integer(c_int64_t), dimension(:, :), intent(out) :: counts
        call check(c_distributions_mu(h, int(size(fglobal, 1), c_int32_t), fglobal, counts), &
            "calc_particle_distributions")
    end subroutine gpu_global_distribution_mu

    !< fescaped(nmu_global, npp_global, 2 ndim) of calc_escaped_distributions
    !< (:949-957) over the escaped particles kept since the last reset
    subroutine gpu_escaped_distribution_mu(fescaped, counts)
        real(c_double), dimension(:, :, :), intent(out) :: fescaped
        integer(c_int64_t), dimension(:, :, :), intent(out) :: counts
        call check(c_escaped_mu(h, int(size(fescaped, 1), c_int32_t), fescaped, counts), &
            "calc_escaped_distributions")
    end subroutine gpu_escaped_distribution_mu

    !< flocalK(nmu, npbins, nrx, nry, nrz) of calc_particle_distributions
    !< (:782-878) for one parameter set
    subroutine gpu_local_distribution(spec, flocal, counts)
        type(gpat_local_dist_t), intent(in) :: spec
        real(c_double), dimension(:, :, :, :, :), intent(out) :: flocal
        integer(c_int64_t), dimension(:, :, :, :, :), intent(out) :: counts
        call check(c_local_dist(h, spec, flocal, counts), "calc_particle_distributions")
    end subroutine gpu_local_distribution

    !< fescapedK_x / _y / _z of calc_escaped_distributions (:958-1230); the
    !< y and z arrays are left out below 2D and 3D
    subroutine gpu_local_escaped_distribution(spec, fx, cx, fy, cy, fz, cz)
        type(gpat_local_dist_t), intent(in) :: spec
        real(c_double), dimension(:, :, :, :, :), intent(out), target, contiguous :: fx
        integer(c_int64_t), dimension(:, :, :, :, :), intent(out), target, contiguous :: cx
        real(c_double), dimension(:, :, :, :, :), intent(out), target, contiguous, &
            optional :: fy, fz
        integer(c_int64_t), dimension(:, :, :, :, :), intent(out), target, contiguous, &
            optional :: cy, cz
        type(c_ptr) :: pfy, pfz, pcy, pcz
        pfy = c_null_ptr; pfz = c_null_ptr; pcy = c_null_ptr; pcz = c_null_ptr
        if (present(fy)) pfy = c_loc(fy)
        if (present(cy)) pcy = c_loc(cy)
        if (present(fz)) pfz = c_loc(fz)
        if (present(cz)) pcz = c_loc(cz)
        call check(c_local_escaped(h, spec, c_loc(fx), pfy, pfz, c_loc(cx), pcy, pcz), &
            "calc_escaped_distributions")
    end subroutine gpu_local_escaped_distribution

    !< escaped_ptls (dump_escaped_particles, diagnostics.f90:1896-1978) into
    !< arrays of length capacity; n on exit
    subroutine gpu_get_escaped_ptls(capacity, n, x, y, z, p, v, mu, weight, t, dt, &
            split_times, count_flag, origin, nsteps_tracked, nsteps_pushed, tag_injected, &
            tag_splitted, rng_ctr)
        integer, intent(in) :: capacity
        integer, intent(out) :: n
        real(c_double), dimension(capacity), intent(out), target :: x, y, z, p, v, mu, weight, &
            t, dt
        integer(c_int8_t), dimension(capacity), intent(out), target :: split_times, count_flag
        integer(c_int32_t), dimension(capacity), intent(out), target :: origin, nsteps_tracked, &
            nsteps_pushed, tag_injected, tag_splitted, rng_ctr
        type(gpat_particles_t) :: s
        integer(c_int64_t) :: got
        integer(c_int) :: rc
        s%x = c_loc(x); s%y = c_loc(y); s%z = c_loc(z); s%p = c_loc(p); s%v = c_loc(v)
        s%mu = c_loc(mu); s%weight = c_loc(weight); s%t = c_loc(t); s%dt = c_loc(dt)
        s%split_times = c_loc(split_times); s%count_flag = c_loc(count_flag)
        s%origin = c_loc(origin); s%nsteps_tracked = c_loc(nsteps_tracked)
        s%nsteps_pushed = c_loc(nsteps_pushed); s%tag_injected = c_loc(tag_injected)
        s%tag_splitted = c_loc(tag_splitted); s%rng_ctr = c_loc(rng_ctr)
        rc = c_get_escaped(h, s, int(capacity, c_int64_t), got)
        n = int(got)
        call check(rc, "get_escaped_particles")
    end subroutine gpu_get_escaped_ptls

    !< Module state for save_particle_module_state / read_particle_module_state
    !< (particle_module.f90:5532-5660): nptl_split, tag_max and the exact leak
    !< sums travel in gpat_counters_t
    subroutine gpu_get_counters(c)
        type(gpat_counters_t), intent(out) :: c
        call check(c_get_counters(h, c), "get_counters")
    end subroutine gpu_get_counters

    subroutine gpu_set_counters(c)
        type(gpat_counters_t), intent(in) :: c
        call check(c_set_counters(h, c), "set_counters")
    end subroutine gpu_set_counters

    !< free_particle_tracking (:5905-5911)
    subroutine gpu_free_particle_tracking
        call check(c_free_tracking(h), "free_particle_tracking")
    end subroutine gpu_free_particle_tracking

end module gpat_gpu
