! mprw_gpu.f90 -- Fortran 2003 ISO_C_BINDING interface to libmprw_gpu.
!
! The bind(C) derived types mirror the structs of mprw_gpu.h field by field
! (same order, same C types), and every entry point of the C ABI has an
! interface here.  A MODPATH-RW build adds this file to its sources, `use
! mprw_gpu` in MPathRW.F90, and links -lmprw_gpu -lcudart.  The calls replace
! the tracking part of the particle loop (MPathRW.F90:1207-1539) and the
! GPKDE reconstruction (MPathRW.F90:1568-1642); the header mprw_gpu.h states
! each entry point's semantics and the reference routine it replaces.
module mprw_gpu
  use, intrinsic :: iso_c_binding
  implicit none

  integer(c_int), parameter :: MPRW_OK = 0, MPRW_FP64 = 0, MPRW_MIXED = 1
  integer(c_int), parameter :: MPRW_E_INVAL = -1, MPRW_E_CUDA = -2, MPRW_E_OOM = -3, MPRW_E_STATE = -4, &
                               MPRW_E_ABORTED = -5, MPRW_E_SIZE = -6
  integer(c_int32_t), parameter :: MPRW_NOALLOC_MAX_BINS = 2**20

  type, bind(C) :: mprw_grid_desc
    integer(c_int32_t) :: nlay, nrow, ncol
    type(c_ptr) :: delr, delc, top, botm          ! real(c_double) arrays
  end type

  type, bind(C) :: mprw_options
    integer(c_int32_t) :: time_step_kind           ! 1 ADV 2 DISP 3 MIN_ADV_DISP 4 FIXED
    real(c_double)     :: ts_param(2)
    integer(c_int32_t) :: advection_kind           ! 2 EULERIAN
    integer(c_int32_t) :: dim_mask(3)
    integer(c_int32_t) :: dispersion_model
    integer(c_int32_t) :: stop_weak_sinks, stop_weak_sources, backward, stop_zone
    integer(c_int32_t) :: uniform_porosity
    integer(c_int64_t) :: rng_seed                 ! uint64 in C
    integer(c_int32_t) :: precision                ! MPRW_FP64 or MPRW_MIXED
  end type

  type, bind(C) :: mprw_flow_desc
    type(c_ptr)        :: ia, ja                   ! 1-based CSR of the MF6 grid file
    integer(c_int64_t) :: nja
    type(c_ptr)        :: flowja, boundary_flows, porosity, retardation
    type(c_ptr)        :: iboundts, icboundts
    integer(c_int32_t) :: default_icbound
    type(c_ptr)        :: heads, celltype, source_flow, sink_flow, zones
    type(c_ptr)        :: alpha_l, alpha_t, dm_eff
    integer(c_int32_t) :: uniform_dispersion, steady_state
    type(c_ptr)        :: alpha_lv, alpha_tv       ! axisymmetric model, or c_null_ptr
  end type

  type, bind(C) :: mprw_gpkde_options
    real(c_double)     :: origin(3), domain_size(3), bin_size(3)
    integer(c_int32_t) :: n_opt_loops
    real(c_double)     :: min_hover_delta, delta_hover_delta, max_hover_delta
    real(c_double)     :: rel_err_convergence
    integer(c_int32_t) :: skip_error_convergence, unit_volume
    real(c_double)     :: scaling_factor
    integer(c_int32_t) :: precision                ! MPRW_FP64 or MPRW_MIXED
    integer(c_int32_t) :: isotropic                ! gpkdeIsotropicKernels (0 or 1)
  end type

  type, bind(C) :: mprw_gpkde_sums                 ! summable part of a reconstruction
    real(c_double)     :: n_active, sum_w, sum_w2
    real(c_double)     :: sum_dx(3), sum_dx2(3)     ! about the domain centre
  end type

  type, bind(C) :: mprw_adj_options                ! differentiable walk
    integer(c_int32_t) :: nzones, nsteps, checkpoint
    real(c_double)     :: dt, velocity_floor
    integer(c_int64_t) :: seed                     ! uint64 in C
    real(c_double)     :: origin(3), bin_size(3)
    integer(c_int32_t) :: n_bins(3)
    real(c_double)     :: bandwidth(3)
  end type

  type, bind(C) :: mprw_series_options             ! the observation post-process GPKDE
    real(c_double)     :: origin, domain_size, bin_size
    integer(c_int32_t) :: bin_format               ! obs%histogramBinFormat
    real(c_double)     :: bin_size_fraction        ! obs%binSizeFraction
    integer(c_int32_t) :: adapt_grid, exact_point, effective_weight_format
    integer(c_int32_t) :: initial_smoothing_selection
    real(c_double)     :: initial_smoothing_factor ! obs%binSizeFactor
    integer(c_int32_t) :: apply_initial_factor, n_opt_loops
    real(c_double)     :: rel_err_convergence      ! obs%errorConvergence
    integer(c_int32_t) :: skip_error_convergence, only_histogram, compute_raw_density, unit_volume
  end type

  type, bind(C) :: mprw_series_result
    integer(c_int32_t) :: n_bins, delta_bins_origin
    real(c_double)     :: bin_size, grid_origin
    integer(c_int32_t) :: loops_done, active_bins
  end type

  interface
    integer(c_int) function mprw_create(h, grid, opt) bind(C, name="mprw_create")
      import; type(c_ptr) :: h; type(mprw_grid_desc), intent(in) :: grid
      type(mprw_options), intent(in) :: opt
    end function
    integer(c_int) function mprw_load_flow(h, flow) bind(C, name="mprw_load_flow")
      import; type(c_ptr), value :: h; type(mprw_flow_desc), intent(in) :: flow
    end function
    integer(c_int) function mprw_set_particles(h, n, cell, lx, ly, lz, t, status, mass, id, rng_ctr) &
        bind(C, name="mprw_set_particles")
      import; type(c_ptr), value :: h; integer(c_int64_t), value :: n
      integer(c_int32_t), intent(in) :: cell(*), status(*)
      real(c_double), intent(in) :: lx(*), ly(*), lz(*), t(*)
      type(c_ptr), value :: mass, id, rng_ctr        ! c_loc(...) or c_null_ptr
    end function
    integer(c_int) function mprw_advance(h, t_begin, t_end, steps_done) bind(C, name="mprw_advance")
      import; type(c_ptr), value :: h; real(c_double), value :: t_begin, t_end
      integer(c_int64_t) :: steps_done
    end function
    integer(c_int) function mprw_get_particles(h, cell, lx, ly, lz, t, status, rng_ctr, gx, gy, gz) &
        bind(C, name="mprw_get_particles")
      import; type(c_ptr), value :: h
      type(c_ptr), value :: cell, lx, ly, lz, t, status, rng_ctr, gx, gy, gz   ! any may be c_null_ptr
    end function
    integer(c_int) function mprw_histogram(h, origin, bin_size, n_bins, counts, n_binned, eff_mass) &
        bind(C, name="mprw_histogram")
      import; type(c_ptr), value :: h
      real(c_double), intent(in) :: origin(3), bin_size(3); integer(c_int32_t), intent(in) :: n_bins(3)
      real(c_double) :: counts(*); integer(c_int64_t) :: n_binned; real(c_double) :: eff_mass
    end function
    integer(c_int) function mprw_gpkde(h, opt, density, histogram, n_bins_out, loops_done) &
        bind(C, name="mprw_gpkde")
      import; type(c_ptr), value :: h; type(mprw_gpkde_options), intent(in) :: opt
      real(c_double) :: density(*); type(c_ptr), value :: histogram
      integer(c_int32_t) :: n_bins_out(3), loops_done
    end function
    integer(c_int) function mprw_gpkde_partial(h, opt, mass_per_bin, sums) bind(C, name="mprw_gpkde_partial")
      import; type(c_ptr), value :: h; type(mprw_gpkde_options), intent(in) :: opt
      real(c_double) :: mass_per_bin(*); type(mprw_gpkde_sums) :: sums
    end function
    integer(c_int) function mprw_gpkde_from_counts(h, opt, mass_per_bin, sums, density, histogram, n_bins_out, &
        loops_done) bind(C, name="mprw_gpkde_from_counts")
      import; type(c_ptr), value :: h; type(mprw_gpkde_options), intent(in) :: opt
      real(c_double), intent(in) :: mass_per_bin(*); type(mprw_gpkde_sums), intent(in) :: sums
      real(c_double) :: density(*); type(c_ptr), value :: histogram
      integer(c_int32_t) :: n_bins_out(3), loops_done
    end function
    integer(c_int) function mprw_set_observations(h, ncells, cells, obs, nobs, style) &
        bind(C, name="mprw_set_observations")
      import; type(c_ptr), value :: h; integer(c_int32_t), value :: ncells, nobs
      integer(c_int32_t), intent(in) :: cells(*), obs(*), style(*)
    end function
    integer(c_int) function mprw_observe_resident(h, count, mass) bind(C, name="mprw_observe_resident")
      import; type(c_ptr), value :: h; integer(c_int64_t) :: count(*); real(c_double) :: mass(*)
    end function
    integer(c_int) function mprw_observe_sinks(h, capacity, obs, id, time, mass, n_records) &
        bind(C, name="mprw_observe_sinks")
      import; type(c_ptr), value :: h; integer(c_int64_t), value :: capacity
      integer(c_int32_t) :: obs(*); integer(c_int64_t) :: id(*)        ! uint64 in C
      real(c_double) :: time(*), mass(*); integer(c_int64_t) :: n_records
    end function
    integer(c_int) function mprw_gpkde_series(times, weights, n, opt, capacity, counts, wcounts, density, &
        res, stream) bind(C, name="mprw_gpkde_series")
      import; integer(c_int64_t), value :: n; integer(c_int32_t), value :: capacity
      real(c_double), intent(in) :: times(*), weights(*); type(mprw_series_options), intent(in) :: opt
      real(c_double) :: counts(*); type(c_ptr), value :: wcounts, density, stream
      type(mprw_series_result) :: res
    end function
    integer(c_int) function mprw_histogram_noalloc(gx, gy, gz, status, n, origin, bin_size, n_bins, counts, &
        n_binned, stream) bind(C, name="mprw_histogram_noalloc")
      import; type(c_ptr), value :: gx, gy, gz, status  ! device arrays
      integer(c_int64_t), value :: n
      real(c_double), intent(in) :: origin(3), bin_size(3); integer(c_int32_t), intent(in) :: n_bins(3)
      type(c_ptr), value :: counts, n_binned, stream      ! device arrays; cudaStream_t
    end function
    integer(c_int) function mprw_create_batch(h, nmembers, grids, opt) bind(C, name="mprw_create_batch")
      import; type(c_ptr) :: h; integer(c_int32_t), value :: nmembers
      type(mprw_grid_desc), intent(in) :: grids(*); type(mprw_options), intent(in) :: opt
    end function
    integer(c_int) function mprw_batch_member(h, member, view) bind(C, name="mprw_batch_member")
      import; type(c_ptr), value :: h; integer(c_int32_t), value :: member; type(c_ptr) :: view
    end function
    integer(c_int) function mprw_set_particles_batch(h, counts, cell, lx, ly, lz, t, status, mass, id, &
        rng_ctr) bind(C, name="mprw_set_particles_batch")
      import; type(c_ptr), value :: h; integer(c_int64_t), intent(in) :: counts(*)
      integer(c_int32_t), intent(in) :: cell(*), status(*)
      real(c_double), intent(in) :: lx(*), ly(*), lz(*), t(*)
      type(c_ptr), value :: mass, id, rng_ctr
    end function
    integer(c_int) function mprw_gpkde_batch(h, opts, density, histogram, loops_done, concurrency) &
        bind(C, name="mprw_gpkde_batch")
      import; type(c_ptr), value :: h; type(mprw_gpkde_options), intent(in) :: opts(*)
      type(c_ptr), intent(in) :: density(*)          ! c_loc of each member's density array
      type(c_ptr), value :: histogram, loops_done; integer(c_int32_t), value :: concurrency
    end function
    integer(c_int) function mprw_set_tuning(h, blocks_per_sm, sort_interval) bind(C, name="mprw_set_tuning")
      import; type(c_ptr), value :: h; integer(c_int32_t), value :: blocks_per_sm, sort_interval
    end function
    integer(c_int) function mprw_get_tuning(h, blocks_per_sm, sort_interval, max_blocks) &
        bind(C, name="mprw_get_tuning")
      import; type(c_ptr), value :: h; integer(c_int32_t) :: blocks_per_sm, sort_interval, max_blocks
    end function
    integer(c_int) function mprw_autotune(h, t_begin, t_end, blocks_per_sm, sort_interval, rates) &
        bind(C, name="mprw_autotune")
      import; type(c_ptr), value :: h; real(c_double), value :: t_begin, t_end
      integer(c_int32_t) :: blocks_per_sm, sort_interval; type(c_ptr), value :: rates
    end function
    integer(c_int) function mprw_adj_setup(h, zones, opt) bind(C, name="mprw_adj_setup")
      import; type(c_ptr), value :: h; integer(c_int32_t), intent(in) :: zones(*)
      type(mprw_adj_options), intent(in) :: opt
    end function
    integer(c_int) function mprw_adj_forward(h, theta, density) bind(C, name="mprw_adj_forward")
      import; type(c_ptr), value :: h; real(c_double), intent(in) :: theta(*); real(c_double) :: density(*)
    end function
    integer(c_int) function mprw_adj_backward(h, grad_density, grad_theta) bind(C, name="mprw_adj_backward")
      import; type(c_ptr), value :: h; real(c_double), intent(in) :: grad_density(*)
      real(c_double) :: grad_theta(*)
    end function
    integer(c_int) function mprw_set_timeout(h, timeout_ms) bind(C, name="mprw_set_timeout")
      import; type(c_ptr), value :: h; real(c_double), value :: timeout_ms
    end function
    integer(c_int) function mprw_cancel(h) bind(C, name="mprw_cancel")
      import; type(c_ptr), value :: h
    end function
    integer(c_int) function mprw_set_stream(h, stream) bind(C, name="mprw_set_stream")
      import; type(c_ptr), value :: h, stream
    end function
    integer(c_int) function mprw_last_timings(h, step_ms, prep_ms, hist_ms, gpkde_ms, launches) &
        bind(C, name="mprw_last_timings")
      import; type(c_ptr), value :: h; real(c_double) :: step_ms, prep_ms, hist_ms, gpkde_ms
      integer(c_int64_t) :: launches
    end function
    integer(c_int) function mprw_last_gpkde_work(h, madds) bind(C, name="mprw_last_gpkde_work")
      import; type(c_ptr), value :: h; real(c_double) :: madds
    end function
    integer(c_int) function mprw_destroy(h) bind(C, name="mprw_destroy")
      import; type(c_ptr), value :: h
    end function
    type(c_ptr) function mprw_last_error(h) bind(C, name="mprw_last_error")
      import; type(c_ptr), value :: h
    end function
  end interface
end module
