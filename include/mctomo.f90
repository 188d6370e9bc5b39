! ISO_C_BINDING interface to libmctomo_gpu.so (include/mctomo.h), for a
! Fortran host such as MCTomo's sampler. Every C entry point has an
! interface here with the same name; scalars are passed by value, arrays and
! output arguments by reference, device pointers and streams as type(c_ptr).
! Arrays keep Fortran's column-major layout: the C side documents each
! array's shape in Fortran order (e.g. vel(nz, ny, nx) is C vel[nx][ny][nz]).
!
! Example (3D travel times, the fastMarching3D call of
! src/fastMarching_wrapper.f90):
!
!   use mctomo_gb300
!   ierr = mct_fast_marching3d(nx, ny, nz, dx, dy, dz, xmin, ymin, zmin, &
!                              vel, src, rev, nrev, order, ttime, tfield)
!   if (ierr < 0) write(*,*) mct_error_message()
module mctomo_gb300
  use, intrinsic :: iso_c_binding
  implicit none

  integer(c_int), parameter :: MCT_OK = 0
  integer(c_int), parameter :: MCT_MODEL_INVALID = 1
  integer(c_int), parameter :: MCT_ERR_ARG = -1
  integer(c_int), parameter :: MCT_ERR_CUDA = -2
  integer(c_int), parameter :: MCT_ERR_NOMEM = -3
  integer(c_int), parameter :: MCT_ERR_OUTSIDE = -4
  integer(c_int), parameter :: MCT_ERR_UNSUPPORTED = -5
  integer(c_int), parameter :: MCT_ERR_TIMEOUT = -6
  integer(c_int), parameter :: MCT_ERR_INTERNAL = -7
  integer(c_int), parameter :: MCT_LAW_EXPLICIT = 0
  integer(c_int), parameter :: MCT_LAW_REFERENCE = 1
  integer(c_int), parameter :: MCT_LAW_FIXED_RHO = 2
  integer(c_int), parameter :: MCT_EIK3_TILES = 16
  integer(c_int), parameter :: MCT_EIK3_HEAP = 32

  ! T_GRID (src/settings.f90:20-28)
  type, bind(C) :: mct_grid
    integer(c_int) :: nx, ny, nz
    real(c_double) :: xmin, ymin, zmin, dx, dy, dz
    real(c_double) :: scaling, water_depth
  end type mct_grid

  ! surface-wave settings (T_LIKE_SET fields the surface likelihood reads)
  type, bind(C) :: mct_modes_para
    integer(c_int) :: modetype, nmodes, phase_group
    real(c_double) :: tolmin, tolmax, smin_min, smin_max
    real(c_double) :: dc, dcm, dc1, dc2
  end type

  type, bind(C) :: mct_surf_settings
    integer(c_int) :: raylov, phase_group
    real(c_double) :: dphase
    integer(c_int) :: gridx, gridy, sgref, sgdic, sgext, order
    integer(c_int) :: sigdep, material_law
    real(c_double) :: rho_value
    integer(c_int) :: precision, tt_precision, straight
  end type mct_surf_settings

  ! surface-wave data; the pointers are c_loc of the caller's arrays
  type, bind(C) :: mct_surf_data
    integer(c_int) :: nsrc, nrev, np
    type(c_ptr) :: src, rev, freqs, raystat, ttime, sigma
    integer(c_int) :: nrays
  end type mct_surf_data

  type, bind(C) :: mct_body_settings
    integer(c_int) :: order, np, sigdep, solver, dynamic
  end type mct_body_settings

  type, bind(C) :: mct_body_data
    integer(c_int) :: nsrc, nrev, np
    type(c_ptr) :: rev, raystat, ttime, sigma
    integer(c_int) :: nrays
  end type mct_body_data

  type, bind(C) :: mct_tt2d_settings
    integer(c_int) :: gridx, gridy, sgref, sgdic, sgext, order
    integer(c_int) :: sigdep, datatype, straight, precision
  end type mct_tt2d_settings

  type, bind(C) :: mct_tt2d_data
    integer(c_int) :: nsrc, nrev
    type(c_ptr) :: src, rev, raystat, ttime, sigma
    integer(c_int) :: nrays
    type(c_ptr) :: dtime, dcc
    integer(c_int) :: ndtime
  end type mct_tt2d_data

  type, bind(C) :: mct_mcmc_set
    integer(c_int) :: ncell_min, ncell_max, kernel, datatype, sigdep, locate
    real(c_double) :: xmin, xmax, ymin, ymax, zmin, zmax, vpmin, vpmax, vsmin, vsmax
    real(c_double) :: sigma_vp, sigma_vs, sigma_vp2, sigma_vs2, pd, pd2
    real(c_double) :: sigma_bn0, sigma_bn1, bn0_min, bn0_max, bn1_min, bn1_max
    real(c_double) :: sigma_sn0, sigma_sn1, sn0_min, sn0_max, sn1_min, sn1_max
  end type
  type, bind(C) :: mct_mcmc_state
    integer(c_int) :: ncells
    type(c_ptr) :: points, parameters
    integer(c_int) :: nbnoise, nsnoise
    type(c_ptr) :: bnoise0, bnoise1, snoise0, snoise1
  end type
  type, bind(C) :: mct_mcmc_step
    integer(c_int) :: ptype, index, valid
    real(c_double) :: prob, random
  end type
  type, bind(C) :: mct_pt
    integer(c_int) :: nchains, number_of_1s, jump_type
    type(c_ptr) :: values0, values, indices
    integer(c_long_long) :: accepted, total
  end type
  type, bind(C) :: mct_sample
    integer(c_int) :: step, accepted, vindex
    integer(c_long_long) :: ncells
    real(c_double) :: misfit, unweighted_misfit, like
    real(c_double) :: coord(3), values(3)
    real(c_double) :: noise0, noise1
  end type

  interface
    type(c_ptr) function mct_version() bind(C, name="mct_version")
      import :: c_ptr
    end function
    type(c_ptr) function mct_last_error() bind(C, name="mct_last_error")
      import :: c_ptr
    end function

    ! ---- gridding (kdtree_to_grid, src/mcmc_loc2.f90:2002-2082)
    integer(c_int) function mct_kdtree_to_grid(d, n, points, params, nx, ny, nz, grid_lo, grid_step, box, &
        sites_id, vp, vs, rho) bind(C, name="mct_kdtree_to_grid")
      import :: c_int, c_double, c_ptr
      integer(c_int), value :: d, n, nx, ny, nz
      real(c_double), intent(in) :: points(*), params(*), grid_lo(*), grid_step(*)
      type(c_ptr), value :: box
      integer(c_int), intent(inout) :: sites_id(*)
      real(c_double), intent(inout) :: vp(*), vs(*), rho(*)
    end function
    integer(c_int) function mct_grid_nearest_batch_device(d, nchains, ncell_max, ncells, points, params, nx, ny, &
        nz, grid_lo, grid_step, box, sites_id, vp, vs, rho, stream) bind(C, name="mct_grid_nearest_batch_device")
      import :: c_int, c_double, c_ptr
      integer(c_int), value :: d, nchains, ncell_max, nx, ny, nz
      type(c_ptr), value :: ncells, points, params
      real(c_double), intent(in) :: grid_lo(*), grid_step(*)
      type(c_ptr), value :: box, sites_id, vp, vs, rho, stream
    end function
    integer(c_int) function mct_grid_status(stream, status) bind(C, name="mct_grid_status")
      import :: c_int, c_ptr
      type(c_ptr), value :: stream
      integer(c_int), intent(out) :: status
    end function
    integer(c_int) function mct_grid_nearest_batch_device_noalloc(d, nchains, ncell_max, ncells, points, params, &
        nx, ny, nz, grid_lo, grid_step, box, sites_id, vp, vs, rho, stream) &
        bind(C, name="mct_grid_nearest_batch_device_noalloc")
      import :: c_int, c_double, c_ptr
      integer(c_int), value :: d, nchains, ncell_max, nx, ny, nz
      type(c_ptr), value :: ncells, points, params
      real(c_double), intent(in) :: grid_lo(*), grid_step(*)
      type(c_ptr), value :: box, sites_id, vp, vs, rho, stream
    end function

    ! ---- dispersion (surfmodes/surfdisp96.f, surfmodes/surfmodes.f90)
    integer(c_int) function mct_surfdisp96(thkm, vpm, vsm, rhom, nlayer, iflsph, iwave, mode, igr, kmax, t, &
        dphase, cp, cg, ierr) bind(C, name="mct_surfdisp96")
      import :: c_int, c_float, c_double
      real(c_float), intent(in) :: thkm(*), vpm(*), vsm(*), rhom(*)
      integer(c_int), value :: nlayer, iflsph, iwave, mode, igr, kmax
      real(c_double), intent(in) :: t(*)
      real(c_double), value :: dphase
      real(c_double), intent(out) :: cp(*), cg(*)
      integer(c_int), intent(out) :: ierr
    end function
    integer(c_int) function mct_surfdisp_mmodes(thkm, vpm, vsm, rhom, nlayer, iflsph, iwave, mode, igr, kmax, t, &
        dphase, cp, cg, ierr) bind(C, name="mct_surfdisp_mmodes")
      import :: c_int, c_float, c_double
      real(c_float), intent(in) :: thkm(*), vpm(*), vsm(*), rhom(*)
      integer(c_int), value :: nlayer, iflsph, iwave, mode, igr, kmax
      real(c_double), intent(in) :: t(*)
      real(c_double), value :: dphase
      real(c_double), intent(out) :: cp(*), cg(*)
      integer(c_int), intent(out) :: ierr
    end function
    integer(c_int) function mct_surfmodes(thick, vp, vs, rho, nlayers, freqs, np, modetype, phase_group, dc, &
        phase, group, ierr) bind(C, name="mct_surfmodes")
      import :: c_int, c_double
      real(c_double), intent(in) :: thick(*), vp(*), vs(*), rho(*), freqs(*)
      integer(c_int), value :: nlayers, np, modetype, phase_group
      real(c_double), value :: dc
      real(c_double), intent(out) :: phase(*), group(*)
      integer(c_int), intent(out) :: ierr
    end function
    integer(c_int) function mct_surfmodes_para(thick, vp, vs, rho, nlayers, freqs, np, paras, phase, group, &
        ierr) bind(C, name="mct_surfmodes_para")
      import :: c_int, c_double, mct_modes_para
      real(c_double), intent(in) :: thick(*), vp(*), vs(*), rho(*), freqs(*)
      integer(c_int), value :: nlayers, np
      type(mct_modes_para), intent(in) :: paras
      real(c_double), intent(out) :: phase(*), group(*)
      integer(c_int), intent(out) :: ierr
    end function
    integer(c_int) function mct_surfmodes_route(ncol, nl_max, nl, vp, vs, modetype, route) &
        bind(C, name="mct_surfmodes_route")
      import :: c_int, c_double
      integer(c_int), value :: ncol, nl_max, modetype
      integer(c_int), intent(in) :: nl(*)
      real(c_double), intent(in) :: vp(*), vs(*)
      integer(c_int), intent(out) :: route(*)
    end function
    integer(c_int) function mct_grt_batch(ncol, nl_max, nl, thk, vp, vs, rho, np, freqs, paras, phase, group, &
        ierr, nevals) bind(C, name="mct_grt_batch")
      import :: c_int, c_double, c_long_long, mct_modes_para
      integer(c_int), value :: ncol, nl_max, np
      integer(c_int), intent(in) :: nl(*)
      real(c_double), intent(in) :: thk(*), vp(*), vs(*), rho(*), freqs(*)
      type(mct_modes_para), intent(in) :: paras
      real(c_double), intent(out) :: phase(*), group(*)
      integer(c_int), intent(out) :: ierr(*)
      integer(c_long_long), intent(out) :: nevals
    end function
    integer(c_int) function mct_grt_batch_device(ncol, nl_max, nl, thk, vp, vs, rho, np, freqs, paras, phase, &
        group, ierr, nevals, stream) bind(C, name="mct_grt_batch_device")
      import :: c_int, c_ptr, mct_modes_para
      integer(c_int), value :: ncol, nl_max, np
      type(c_ptr), value :: nl, thk, vp, vs, rho, freqs, phase, group, ierr, nevals, stream
      type(mct_modes_para), intent(in) :: paras
    end function
    integer(c_int) function mct_surfdisp_batch(ncol, nl_max, nl, thk, vp, vs, rho, np, periods, iwave, mode, igr, &
        dphase, multimode, precision, cp, cg, ierr, ndltar) bind(C, name="mct_surfdisp_batch")
      import :: c_int, c_float, c_double, c_ptr
      integer(c_int), value :: ncol, nl_max, np, iwave, mode, igr, multimode, precision
      integer(c_int), intent(in) :: nl(*)
      real(c_float), intent(in) :: thk(*), vp(*), vs(*), rho(*)
      real(c_double), intent(in) :: periods(*)
      real(c_double), value :: dphase
      real(c_double), intent(out) :: cp(*), cg(*)
      integer(c_int), intent(out) :: ierr(*)
      type(c_ptr), value :: ndltar
    end function
    integer(c_int) function mct_surfdisp_batch_device(ncol, nl_max, nl, thk, vp, vs, rho, np, periods, iwave, &
        mode, igr, dphase, multimode, precision, cp, cg, ierr, ndltar, stream) &
        bind(C, name="mct_surfdisp_batch_device")
      import :: c_int, c_double, c_ptr
      integer(c_int), value :: ncol, nl_max, np, iwave, mode, igr, multimode, precision
      type(c_ptr), value :: nl, thk, vp, vs, rho, periods
      real(c_double), value :: dphase
      type(c_ptr), value :: cp, cg, ierr, ndltar, stream
    end function

    ! ---- 2D travel times (fm2d/fm2dray_cartesian.f90 modrays)
    integer(c_int) function mct_modrays(nsrc, scx, scz, nrc, rcx, rcz, srsin, wrgf, nvx, nvz, goxd, gozd, dvxd, &
        dvzd, velvin, gdx, gdz, asgr, sgdl, sgs, earth, fom, snb, ttime, uar, crazyray, tfield) &
        bind(C, name="mct_modrays")
      import :: c_int, c_double, c_ptr
      integer(c_int), value :: nsrc, nrc, wrgf, nvx, nvz, gdx, gdz, asgr, sgdl, sgs, fom, uar
      real(c_double), intent(in) :: scx(*), scz(*), rcx(*), rcz(*), velvin(*)
      integer(c_int), intent(in) :: srsin(*)
      real(c_double), value :: goxd, gozd, dvxd, dvzd, earth, snb
      real(c_double), intent(out) :: ttime(*)
      integer(c_int), intent(out) :: crazyray
      type(c_ptr), value :: tfield
    end function
    integer(c_int) function mct_modrays_batch(nmaps, nsrc, scx, scz, nrc, rcx, rcz, srs_nmaps, srs, nvx, nvz, &
        goxd, gozd, dvxd, dvzd, velv, gdx, gdz, asgr, sgdl, sgs, fom, ttime, tfield, precision) &
        bind(C, name="mct_modrays_batch")
      import :: c_int, c_double, c_ptr
      integer(c_int), value :: nmaps, nsrc, nrc, srs_nmaps, nvx, nvz, gdx, gdz, asgr, sgdl, sgs, fom, precision
      real(c_double), intent(in) :: scx(*), scz(*), rcx(*), rcz(*), velv(*)
      integer(c_int), intent(in) :: srs(*)
      real(c_double), value :: goxd, gozd, dvxd, dvzd
      real(c_double), intent(out) :: ttime(*)
      type(c_ptr), value :: tfield
    end function
    integer(c_int) function mct_modrays_group_batch(nmaps, nsrc, scx, scz, nrc, rcx, rcz, srs_nmaps, srs, nvx, &
        nvz, goxd, gozd, dvxd, dvzd, velv, gvel, gdx, gdz, asgr, sgdl, sgs, fom, ttime, gtime, raylen, crazy, &
        precision) bind(C, name="mct_modrays_group_batch")
      import :: c_int, c_double
      integer(c_int), value :: nmaps, nsrc, nrc, srs_nmaps, nvx, nvz, gdx, gdz, asgr, sgdl, sgs, fom, precision
      real(c_double), intent(in) :: scx(*), scz(*), rcx(*), rcz(*), velv(*), gvel(*)
      integer(c_int), intent(in) :: srs(*)
      real(c_double), value :: goxd, gozd, dvxd, dvzd
      real(c_double), intent(out) :: ttime(*), gtime(*), raylen(*)
      integer(c_int), intent(out) :: crazy(*)
    end function

    ! ---- surface-wave likelihood (src/likelihood_surf.F90 surf_likelihood)
    integer(c_int) function mct_surf_create(grid, settings, data, nslots, ncell_max, ctx) &
        bind(C, name="mct_surf_create")
      import :: c_int, c_ptr, mct_grid, mct_surf_settings, mct_surf_data
      type(mct_grid), intent(in) :: grid
      type(mct_surf_settings), intent(in) :: settings
      type(mct_surf_data), intent(in) :: data
      integer(c_int), value :: nslots, ncell_max
      type(c_ptr), intent(out) :: ctx
    end function
    integer(c_int) function mct_surf_destroy(ctx) bind(C, name="mct_surf_destroy")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function mct_surf_forward(ctx, nchains, slots, ncells, points, params, n0, n1, out) &
        bind(C, name="mct_surf_forward")
      import :: c_int, c_double, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: nchains
      integer(c_int), intent(in) :: slots(*), ncells(*)
      real(c_double), intent(in) :: points(*), params(*), n0(*), n1(*)
      real(c_double), intent(out) :: out(*)
    end function
    integer(c_int) function mct_surf_commit(ctx, accept) bind(C, name="mct_surf_commit")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), intent(in) :: accept(*)
    end function
    integer(c_int) function mct_surf_forward_device(ctx, nchains, slots, ncells, points, params, n0, n1, out, &
        stream) bind(C, name="mct_surf_forward_device")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: nchains
      type(c_ptr), value :: slots, ncells, points, params, n0, n1, out, stream
    end function
    integer(c_int) function mct_surf_commit_device(ctx, accept, stream) bind(C, name="mct_surf_commit_device")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx, accept, stream
    end function
    integer(c_int) function mct_surf_noise_likelihood(ctx, nchains, slots, n0, n1, out) &
        bind(C, name="mct_surf_noise_likelihood")
      import :: c_int, c_double, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: nchains
      integer(c_int), intent(in) :: slots(*)
      real(c_double), intent(in) :: n0(*), n1(*)
      real(c_double), intent(out) :: out(*)
    end function
    integer(c_int) function mct_surf_phase_time(ctx, index, phase_time, phase_vel) &
        bind(C, name="mct_surf_phase_time")
      import :: c_int, c_double, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: index
      real(c_double), intent(out) :: phase_time(*), phase_vel(*)
    end function
    integer(c_int) function mct_surf_profile_start(ctx, max_steps) bind(C, name="mct_surf_profile_start")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: max_steps
    end function
    integer(c_int) function mct_surf_profile_read(ctx, stage_ms, steps, launches) &
        bind(C, name="mct_surf_profile_read")
      import :: c_int, c_double, c_long_long, c_ptr
      type(c_ptr), value :: ctx
      real(c_double), intent(out) :: stage_ms(*)
      integer(c_int), intent(out) :: steps
      integer(c_long_long), intent(out) :: launches
    end function
    integer(c_int) function mct_surf_stream(ctx, stream) bind(C, name="mct_surf_stream")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      type(c_ptr), intent(out) :: stream
    end function
    integer(c_int) function mct_surf_device_bytes(grid, settings, data, nslots, ncell_max, bytes) &
        bind(C, name="mct_surf_device_bytes")
      import :: c_int, c_size_t, mct_grid, mct_surf_settings, mct_surf_data
      type(mct_grid), intent(in) :: grid
      type(mct_surf_settings), intent(in) :: settings
      type(mct_surf_data), intent(in) :: data
      integer(c_int), value :: nslots, ncell_max
      integer(c_size_t), intent(out) :: bytes
    end function
    integer(c_int) function mct_surf_admit(ctx, slot) bind(C, name="mct_surf_admit")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), intent(out) :: slot
    end function
    integer(c_int) function mct_surf_evict(ctx, slot) bind(C, name="mct_surf_evict")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: slot
    end function
    integer(c_int) function mct_surf_submit(ctx, nchains, slots, ncells, points, params, n0, n1) &
        bind(C, name="mct_surf_submit")
      import :: c_int, c_double, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: nchains
      integer(c_int), intent(in) :: slots(*), ncells(*)
      real(c_double), intent(in) :: points(*), params(*), n0(*), n1(*)
    end function
    integer(c_int) function mct_surf_poll(ctx, out, done) bind(C, name="mct_surf_poll")
      import :: c_int, c_double, c_ptr
      type(c_ptr), value :: ctx
      real(c_double), intent(out) :: out(*)
      integer(c_int), intent(out) :: done
    end function
    integer(c_int) function mct_surf_stat_add(ctx, nchains, slots) bind(C, name="mct_surf_stat_add")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: nchains
      integer(c_int), intent(in) :: slots(*)
    end function
    integer(c_int) function mct_surf_stat_read(ctx, slot, mean_vp, mean_vs, msq_vp, msq_vs, nthin) &
        bind(C, name="mct_surf_stat_read")
      import :: c_int, c_double, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: slot
      real(c_double), intent(out) :: mean_vp(*), mean_vs(*), msq_vp(*), msq_vs(*)
      integer(c_int), intent(out) :: nthin
    end function
    integer(c_int) function mct_surf_stat_reset(ctx, slot) bind(C, name="mct_surf_stat_reset")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: slot
    end function
    integer(c_int) function mct_body_location_likelihood(ctx, nchains, locations, n0, n1, out, phase_time) &
        bind(C, name="mct_body_location_likelihood")
      import :: c_int, c_double, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: nchains
      real(c_double), intent(in) :: locations(*), n0(*), n1(*)
      real(c_double), intent(out) :: out(*)
      type(c_ptr), value :: phase_time
    end function
    integer(c_int) function mct_body_location_commit(ctx, nchains, accept) bind(C, name="mct_body_location_commit")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: nchains
      integer(c_int), intent(in) :: accept(*)
    end function
    integer(c_int) function mct_body_submit(ctx, nchains, ncells, points, params, locations, n0, n1) &
        bind(C, name="mct_body_submit")
      import :: c_int, c_double, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: nchains
      integer(c_int), intent(in) :: ncells(*)
      real(c_double), intent(in) :: points(*), params(*), locations(*), n0(*), n1(*)
    end function
    integer(c_int) function mct_body_poll(ctx, out, done) bind(C, name="mct_body_poll")
      import :: c_int, c_double, c_ptr
      type(c_ptr), value :: ctx
      real(c_double), intent(out) :: out(*)
      integer(c_int), intent(out) :: done
    end function
    integer(c_int) function mct_tt2d_submit(ctx, nchains, ncells, points, params, n0, n1) &
        bind(C, name="mct_tt2d_submit")
      import :: c_int, c_double, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: nchains
      integer(c_int), intent(in) :: ncells(*)
      real(c_double), intent(in) :: points(*), params(*), n0(*), n1(*)
    end function
    integer(c_int) function mct_tt2d_poll(ctx, out, done) bind(C, name="mct_tt2d_poll")
      import :: c_int, c_double, c_ptr
      type(c_ptr), value :: ctx
      real(c_double), intent(out) :: out(*)
      integer(c_int), intent(out) :: done
    end function

    ! ---- 3D travel times (fastmarching/fastMarching.cpp fastMarching3D)
    integer(c_int) function mct_fast_marching3d(nx, ny, nz, dx, dy, dz, xmin, ymin, zmin, vel, src, rev, nrev, &
        order, ttime, tfield) bind(C, name="mct_fast_marching3d")
      import :: c_int, c_double, c_ptr
      integer(c_int), value :: nx, ny, nz, nrev, order
      real(c_double), value :: dx, dy, dz, xmin, ymin, zmin
      real(c_double), intent(in) :: vel(*), src(*), rev(*)
      real(c_double), intent(out) :: ttime(*)
      type(c_ptr), value :: tfield
    end function
    integer(c_int) function mct_eikonal3d_batch(nsolve, nx, ny, nz, dx, dy, dz, xmin, ymin, zmin, ngrids, vel, &
        solve_grid, src, nrev, rev, order, ttime, tfield, passes) bind(C, name="mct_eikonal3d_batch")
      import :: c_int, c_double, c_ptr
      integer(c_int), value :: nsolve, nx, ny, nz, ngrids, nrev, order
      real(c_double), value :: dx, dy, dz, xmin, ymin, zmin
      real(c_double), intent(in) :: vel(*), src(*), rev(*)
      integer(c_int), intent(in) :: solve_grid(*)
      real(c_double), intent(out) :: ttime(*)
      type(c_ptr), value :: tfield
      integer(c_int), intent(out) :: passes
    end function
    integer(c_int) function mct_eik3_tile_config(cfg, nx, ny, nz, order) bind(C, name="mct_eik3_tile_config")
      import :: c_int
      integer(c_int), value :: cfg, nx, ny, nz, order
    end function

    ! ---- body-wave likelihood (src/likelihood_body.F90 body_likelihood)
    integer(c_int) function mct_body_create(grid, settings, data, nslots, ncell_max, ctx) &
        bind(C, name="mct_body_create")
      import :: c_int, c_ptr, mct_grid, mct_body_settings, mct_body_data
      type(mct_grid), intent(in) :: grid
      type(mct_body_settings), intent(in) :: settings
      type(mct_body_data), intent(in) :: data
      integer(c_int), value :: nslots, ncell_max
      type(c_ptr), intent(out) :: ctx
    end function
    integer(c_int) function mct_body_destroy(ctx) bind(C, name="mct_body_destroy")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function mct_body_forward(ctx, nchains, ncells, points, params, locations, n0, n1, out) &
        bind(C, name="mct_body_forward")
      import :: c_int, c_double, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: nchains
      integer(c_int), intent(in) :: ncells(*)
      real(c_double), intent(in) :: points(*), params(*), locations(*), n0(*), n1(*)
      real(c_double), intent(out) :: out(*)
    end function
    integer(c_int) function mct_body_commit(ctx, nchains, accept) bind(C, name="mct_body_commit")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: nchains
      integer(c_int), intent(in) :: accept(*)
    end function
    integer(c_int) function mct_body_noise_likelihood(ctx, nchains, locations, n0, n1, out) &
        bind(C, name="mct_body_noise_likelihood")
      import :: c_int, c_double, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: nchains
      real(c_double), intent(in) :: locations(*), n0(*), n1(*)
      real(c_double), intent(out) :: out(*)
    end function
    integer(c_int) function mct_body_phase_time(ctx, index, phase_time, passes) bind(C, name="mct_body_phase_time")
      import :: c_int, c_double, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: index
      real(c_double), intent(out) :: phase_time(*)
      integer(c_int), intent(out) :: passes
    end function

    ! ---- 2D travel-time likelihood (mcmc2d/likelihood_dd.F90)
    integer(c_int) function mct_tt2d_create(grid, settings, data, nslots, ncell_max, ctx) &
        bind(C, name="mct_tt2d_create")
      import :: c_int, c_ptr, mct_grid, mct_tt2d_settings, mct_tt2d_data
      type(mct_grid), intent(in) :: grid
      type(mct_tt2d_settings), intent(in) :: settings
      type(mct_tt2d_data), intent(in) :: data
      integer(c_int), value :: nslots, ncell_max
      type(c_ptr), intent(out) :: ctx
    end function
    integer(c_int) function mct_tt2d_destroy(ctx) bind(C, name="mct_tt2d_destroy")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function mct_tt2d_forward(ctx, nchains, ncells, points, params, n0, n1, out) &
        bind(C, name="mct_tt2d_forward")
      import :: c_int, c_double, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: nchains
      integer(c_int), intent(in) :: ncells(*)
      real(c_double), intent(in) :: points(*), params(*), n0(*), n1(*)
      real(c_double), intent(out) :: out(*)
    end function
    integer(c_int) function mct_tt2d_commit(ctx, nchains, accept) bind(C, name="mct_tt2d_commit")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: nchains
      integer(c_int), intent(in) :: accept(*)
    end function
    integer(c_int) function mct_tt2d_noise_likelihood(ctx, nchains, n0, n1, out) &
        bind(C, name="mct_tt2d_noise_likelihood")
      import :: c_int, c_double, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: nchains
      real(c_double), intent(in) :: n0(*), n1(*)
      real(c_double), intent(out) :: out(*)
    end function
    integer(c_int) function mct_tt2d_phase_time(ctx, index, phase_time) bind(C, name="mct_tt2d_phase_time")
      import :: c_int, c_double, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: index
      real(c_double), intent(out) :: phase_time(*)
    end function
  end interface

contains

  ! The last error message of this thread as a Fortran string.
  function mct_error_message() result(msg)
    character(len=:), allocatable :: msg
    character(kind=c_char), pointer :: s(:)
    type(c_ptr) :: p
    integer :: n
    interface
      integer(c_size_t) function c_strlen(str) bind(C, name="strlen")
        import :: c_size_t, c_ptr
        type(c_ptr), value :: str
      end function
  
    ! ---- the sampler's random number stream (src/mt19937.f90)
    integer(c_int) function mct_rng_create(seed, rng) bind(C, name="mct_rng_create")
      import :: c_int, c_ptr
      integer(c_int), value :: seed
      type(c_ptr), intent(out) :: rng
    end function
    subroutine mct_rng_destroy(rng) bind(C, name="mct_rng_destroy")
      import :: c_ptr
      type(c_ptr), value :: rng
    end subroutine
    integer(c_int) function mct_rng_seed(rng, seed) bind(C, name="mct_rng_seed")
      import :: c_int, c_ptr
      type(c_ptr), value :: rng
      integer(c_int), value :: seed
    end function
    real(c_double) function mct_rng_unirand(rng) bind(C, name="mct_rng_unirand")
      import :: c_double, c_ptr
      type(c_ptr), value :: rng
    end function
    real(c_double) function mct_rng_gasdev(rng) bind(C, name="mct_rng_gasdev")
      import :: c_double, c_ptr
      type(c_ptr), value :: rng
    end function
    integer(c_int) function mct_rng_u32(rng) bind(C, name="mct_rng_u32")
      import :: c_int, c_ptr
      type(c_ptr), value :: rng
    end function
    integer(c_long_long) function mct_rng_count(rng) bind(C, name="mct_rng_count")
      import :: c_long_long, c_ptr
      type(c_ptr), value :: rng
    end function
    integer(c_int) function mct_surf_set_priority(ctx, high) bind(C, name="mct_surf_set_priority")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: high
    end function
    integer(c_int) function mct_body_set_priority(ctx, high) bind(C, name="mct_body_set_priority")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: high
    end function
    integer(c_int) function mct_tt2d_set_priority(ctx, high) bind(C, name="mct_tt2d_set_priority")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: high
    end function
    integer(c_int) function mct_surf_set_sm_share(ctx, share) bind(C, name="mct_surf_set_sm_share")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), value :: share
    end function
    integer(c_int) function mct_tt2d_set_sm_share(ctx, share) bind(C, name="mct_tt2d_set_sm_share")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), value :: share
    end function
    integer(c_int) function mct_mcmc_propose(set, rng, iter, redo, state, step) bind(C, name="mct_mcmc_propose")
      import :: c_int, c_ptr, mct_mcmc_set, mct_mcmc_state, mct_mcmc_step
      type(mct_mcmc_set), intent(in) :: set
      type(c_ptr), value :: rng
      integer(c_int), value :: iter, redo
      type(mct_mcmc_state), intent(inout) :: state
      type(mct_mcmc_step), intent(inout) :: step
    end function
    integer(c_int) function mct_mcmc_accept(set, step, like_new, like_old) bind(C, name="mct_mcmc_accept")
      import :: c_int, c_double, mct_mcmc_set, mct_mcmc_step
      type(mct_mcmc_set), intent(in) :: set
      type(mct_mcmc_step), intent(in) :: step
      real(c_double), value :: like_new, like_old
    end function
    integer(c_int) function mct_mcmc_accept_tempered(set, step, like_new, like_old, temperature) &
        bind(C, name="mct_mcmc_accept_tempered")
      import :: c_int, c_double, mct_mcmc_set, mct_mcmc_step
      type(mct_mcmc_set), intent(in) :: set
      type(mct_mcmc_step), intent(in) :: step
      real(c_double), value :: like_new, like_old, temperature
    end function
    integer(c_int) function mct_mcmc_record(state, step, accepted, like, misfit, unweighted_misfit, sample) &
        bind(C, name="mct_mcmc_record")
      import :: c_int, c_double, mct_mcmc_state, mct_mcmc_step, mct_sample
      type(mct_mcmc_state), intent(in) :: state
      type(mct_mcmc_step), intent(in) :: step
      integer(c_int), value :: accepted
      real(c_double), value :: like, misfit, unweighted_misfit
      type(mct_sample), intent(out) :: sample
    end function
    integer(c_int) function mct_samples_write(filename, dim, samples, n) bind(C, name="mct_samples_write")
      import :: c_int, c_char, mct_sample
      character(kind=c_char), intent(in) :: filename(*)
      integer(c_int), value :: dim, n
      type(mct_sample), intent(in) :: samples(*)
    end function
    integer(c_int) function mct_samples_read(filename, dim, samples, n) bind(C, name="mct_samples_read")
      import :: c_int, c_char, mct_sample
      character(kind=c_char), intent(in) :: filename(*)
      integer(c_int), value :: dim, n
      type(mct_sample), intent(out) :: samples(*)
    end function
    integer(c_int) function mct_pt_init(pt) bind(C, name="mct_pt_init")
      import :: c_int, mct_pt
      type(mct_pt), intent(inout) :: pt
    end function
    integer(c_int) function mct_pt_choose(pt, rng, t1_chain, t2_chain) bind(C, name="mct_pt_choose")
      import :: c_int, c_ptr, mct_pt
      type(mct_pt), intent(inout) :: pt
      type(c_ptr), value :: rng
      integer(c_int), intent(out) :: t1_chain, t2_chain
    end function
    integer(c_int) function mct_pt_swap(pt, rng, t1_chain, t2_chain, like_t1, like_t2) bind(C, name="mct_pt_swap")
      import :: c_int, c_double, c_ptr, mct_pt
      type(mct_pt), intent(inout) :: pt
      type(c_ptr), value :: rng
      integer(c_int), value :: t1_chain, t2_chain
      real(c_double), value :: like_t1, like_t2
    end function
  end interface
    p = mct_last_error()
    if (.not. c_associated(p)) then
      msg = ""
      return
    end if
    n = int(c_strlen(p))
    call c_f_pointer(p, s, [n])
    allocate(character(len=n) :: msg)
    msg = transfer(s(1:n), msg)
  end function mct_error_message
end module mctomo_gb300
