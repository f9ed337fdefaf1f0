! fdtd_gpu_mod -- ISO_C_BINDING interface of libfdtd_gb300.so for Fortran 90/2003
! host programs (the declarations of include/fdtd_gb300.h, one for one).
!
! The reference's programs call type-bound procedures from their time loop
! (FDTDsimulations/3D/air-AuAntennasSiO2-Si/program.f90:382-607); a program
! that moves its loop to the GPU uses this module (directly, or through the
! type-bound wrappers of fdtd_gpu_types.f90) and keeps its set-up and output.
!
! Conventions, the same for every entry point:
!   * every function returns an integer(c_int) status, 0 on success; the
!     message of a failure comes from fdtd_last_error;
!   * handles (fdtd_job, fdtd_server) are type(c_ptr), passed by value;
!   * descriptors are bind(c) derived types passed by reference, their
!     components in the C order; C int32_t[3][2] is a Fortran (2,3) array;
!   * cell indices are 0-based (a reference index i is i-1 here);
!   * field and spectrum buffers are real(c_double) host arrays, x fastest,
!     which is a Fortran array's own order.
module fdtd_gpu_mod
  use iso_c_binding
  implicit none

  ! ---- status codes, layouts, precisions, components -----------------------
  integer(c_int), parameter :: FDTD_OK = 0, FDTD_EINVAL = 1, FDTD_ENOMEM = 2, FDTD_ECUDA = 3, &
       FDTD_ESTATE = 4, FDTD_ERANGE = 5, FDTD_ENODEV = 6
  integer(c_int32_t), parameter :: FDTD_LAYOUT_1D = 1, FDTD_LAYOUT_2D_TE = 2, FDTD_LAYOUT_2D_TM = 3, &
       FDTD_LAYOUT_3D = 4
  integer(c_int32_t), parameter :: FDTD_F32 = 1, FDTD_F64 = 2
  integer(c_int32_t), parameter :: FDTD_EX = 0, FDTD_EY = 1, FDTD_EZ = 2, FDTD_HX = 3, FDTD_HY = 4, &
       FDTD_HZ = 5, FDTD_EX_INC = 6, FDTD_HZ_INC = 7, FDTD_E_INC = 6, FDTD_H_INC = 7
  integer(c_int32_t), parameter :: FDTD_REGION_BOX = 0, FDTD_REGION_SPHERES = 1, FDTD_REGION_MASK = 2
  integer(c_int32_t), parameter :: FDTD_LORENTZ_JP = 0, FDTD_LORENTZ_S = 1, FDTD_LORENTZ_MAX_POLES = 4
  integer(c_int32_t), parameter :: FDTD_RAMAN_EXACT = 0, FDTD_RAMAN_CENTRAL = 1
  integer(c_int32_t), parameter :: FDTD_PML_REFERENCE = 1, FDTD_PML_SPLIT = 2
  integer(c_int32_t), parameter :: FDTD_MONITOR_CELLS = 0, FDTD_MONITOR_MEAN = 1
  integer(c_int32_t), parameter :: FDTD_KERNEL_E = 0, FDTD_KERNEL_H = 1, FDTD_KERNEL_DFT = 2, &
       FDTD_KERNEL_LINE1D = 3, FDTD_KERNEL_EDGE = 4, FDTD_KERNEL_ADE = 5, FDTD_KERNEL_STEP = 6, &
       FDTD_KERNEL_COUNT = 7
  integer(c_int32_t), parameter :: FDTD_REQ_QUEUED = 0, FDTD_REQ_RUNNING = 1, FDTD_REQ_DONE = 2, &
       FDTD_REQ_FAILED = 3
  integer(c_int32_t), parameter :: FDTD_NOALLOC_RING = 32, FDTD_NOALLOC_MAX_CELLS = 262144

  ! ---- descriptors ----------------------------------------------------------
  type, bind(c) :: fdtd_grid_desc
     integer(c_int32_t) :: layout, precision
     integer(c_int32_t) :: n(3), periodic(3), main_lo(3), main_hi(3)
     real(c_double) :: ku, dt, ds
  end type fdtd_grid_desc

  type, bind(c) :: fdtd_region
     integer(c_int32_t) :: kind
     integer(c_int32_t) :: lo(3), hi(3)
     integer(c_int32_t) :: count
     type(c_ptr) :: centers_radii = c_null_ptr    ! real(c_double) (4, count): cx, cy, cz, r
     type(c_ptr) :: mask = c_null_ptr             ! integer(c_int8_t) per cell, x fastest
  end type fdtd_region

  type, bind(c) :: fdtd_drude2cp                  ! Gold (3D/gold_mod.f90:28-34)
     real(c_double) :: eps_inf
     real(c_double) :: omega_d, gamma_d           ! wD, dnur
     real(c_double) :: amp(2), phi(2), omega(2), gamma(2)
  end type fdtd_drude2cp

  type, bind(c) :: fdtd_graphene_desc             ! graphene sheet from E_F, tau, T
     real(c_double) :: fermi_ev, tau, temperature, chi3, raman_frac, raman_freq, raman_tau
     real(c_double) :: thickness, e_scale
  end type fdtd_graphene_desc

  type, bind(c) :: fdtd_lorentz_desc              ! *LorentzJp modules (form 0), si_mod (form 1)
     integer(c_int32_t) :: form, npoles
     real(c_double) :: eps_inf
     real(c_double) :: delta_eps(4), omega(4), gamma(4)
     integer(c_int32_t) :: sheet = 0              ! 1: SLG_* sheet, normal = thin axis
     integer(c_int32_t) :: ez_uses_x_current = 0  ! 1: SLG_LJp's Ez line (JpxT)
     real(c_double) :: chi3 = 0.d0                ! xi3
     real(c_double) :: w_nl = 0.d0, gamma_nl = 0.d0   ! wNL, dnuNL
     real(c_double) :: e_scale = 1.d0             ! z0
  end type fdtd_lorentz_desc

  type, bind(c) :: fdtd_graphene_nk_desc          ! graphene633
     real(c_double) :: n, k, wavelength, scale, chi3, alpha, w_nl, gamma_nl
  end type fdtd_graphene_nk_desc

  type, bind(c) :: fdtd_graphene_cp_desc          ! the reference's Graphene
     real(c_double) :: eps_inf, drude_omega, drude_gamma   ! graphene_epinf, _wD, _dnur
     real(c_double) :: amp(4), phi(4)                      ! ap, phip
     real(c_double) :: omega(4), gamma(4)                  ! omp, rp
     real(c_double) :: width, chi3                         ! Graphenewidth, xi3
     real(c_double) :: w_nl, gamma_nl                      ! wNL, dnuNL
     integer(c_int32_t) :: raman_form = 0         ! FDTD_RAMAN_EXACT (3D module) or _CENTRAL (2D)
     integer(c_int32_t) :: normal_axis = 1        ! y, as the reference's sheet; -1: none
  end type fdtd_graphene_cp_desc

  type, bind(c) :: fdtd_pml_desc                  ! pmly%initialize (3D/BERpmly_mod.f90:485-508)
     integer(c_int32_t) :: mode
     integer(c_int32_t) :: npml(2, 3)             ! (side, axis)
     real(c_double) :: eps_lo, eps_hi, sigma_max, order
  end type fdtd_pml_desc

  type, bind(c) :: fdtd_source_desc               ! 3D/.../program.f90:396-406
     integer(c_int32_t) :: component
     integer(c_int32_t) :: lo(3), hi(3)
     real(c_double) :: amp, t0, st, w0
  end type fdtd_source_desc

  type, bind(c) :: fdtd_monitor_desc              ! 3D/.../program.f90:441-540
     integer(c_int32_t) :: lo(3), hi(3)
     integer(c_int32_t) :: comp_mask
     integer(c_int32_t) :: n_first, n_last, nfreq
     type(c_ptr) :: omega = c_null_ptr            ! real(c_double) (nfreq): arg(m)
     integer(c_int32_t) :: reduce = 0             ! FDTD_MONITOR_CELLS or FDTD_MONITOR_MEAN
  end type fdtd_monitor_desc

  type, bind(c) :: fdtd_probe_desc
     integer(c_int32_t) :: cell(3)
     integer(c_int32_t) :: comp_mask
     integer(c_int32_t) :: n_first, n_last
  end type fdtd_probe_desc

  type, bind(c) :: fdtd_tfsf1d_desc               ! 1D/.../program.f90:217-262
     integer(c_int32_t) :: boundary
     real(c_double) :: eps_lo, eps_hi
  end type fdtd_tfsf1d_desc

  type, bind(c) :: fdtd_tfsf_desc                 ! 3D/.../include/myTFSF_incEzHx_3Dfunc.f90
     integer(c_int32_t) :: lo(3), hi(3)
     real(c_double) :: eps_line
  end type fdtd_tfsf_desc

  type, bind(c) :: fdtd_server_desc
     integer(c_int64_t) :: hbm_budget
     integer(c_int32_t) :: max_active, chunk_steps, pack_cells
  end type fdtd_server_desc

  type, bind(c) :: fdtd_server_status
     integer(c_int32_t) :: queued, active
     integer(c_int64_t) :: finished
     integer(c_int64_t) :: held_bytes, held_bytes_max, budget_bytes
     integer(c_int64_t) :: packed_rings, pack_builds
     real(c_double) :: pack_build_s
  end type fdtd_server_status

  interface
     ! ---- job lifecycle ----
     integer(c_int) function fdtd_create(grid, out) bind(c, name='fdtd_create')
       import :: c_int, c_ptr, fdtd_grid_desc
       type(fdtd_grid_desc), intent(in) :: grid
       type(c_ptr), intent(out) :: out
     end function fdtd_create
     integer(c_int) function fdtd_destroy(job) bind(c, name='fdtd_destroy')
       import :: c_int, c_ptr
       type(c_ptr), value :: job
     end function fdtd_destroy
     integer(c_int) function fdtd_last_error(buf, len) bind(c, name='fdtd_last_error')
       import :: c_int, c_char, c_size_t
       character(kind=c_char), intent(out) :: buf(*)
       integer(c_size_t), value :: len
     end function fdtd_last_error
     integer(c_int) function fdtd_device_count(count) bind(c, name='fdtd_device_count')
       import :: c_int, c_int32_t
       integer(c_int32_t), intent(out) :: count
     end function fdtd_device_count

     ! ---- set-up: materials (initialize_material), PML, TFSF, sources, monitors ----
     integer(c_int) function fdtd_add_dielectric(job, region, eps_r, material_id) bind(c, name='fdtd_add_dielectric')
       import :: c_int, c_ptr, c_double, c_int32_t, fdtd_region
       type(c_ptr), value :: job
       type(fdtd_region), intent(in) :: region
       real(c_double), value :: eps_r
       integer(c_int32_t), intent(out) :: material_id
     end function fdtd_add_dielectric
     integer(c_int) function fdtd_add_gold(job, region, params, material_id) bind(c, name='fdtd_add_gold')
       import :: c_int, c_ptr, c_int32_t, fdtd_region, fdtd_drude2cp
       type(c_ptr), value :: job
       type(fdtd_region), intent(in) :: region
       type(fdtd_drude2cp), intent(in) :: params
       integer(c_int32_t), intent(out) :: material_id
     end function fdtd_add_gold
     integer(c_int) function fdtd_add_graphene(job, region, params, material_id) bind(c, name='fdtd_add_graphene')
       import :: c_int, c_ptr, c_int32_t, fdtd_region, fdtd_graphene_desc
       type(c_ptr), value :: job
       type(fdtd_region), intent(in) :: region
       type(fdtd_graphene_desc), intent(in) :: params
       integer(c_int32_t), intent(out) :: material_id
     end function fdtd_add_graphene
     integer(c_int) function fdtd_add_lorentz(job, region, params, material_id) bind(c, name='fdtd_add_lorentz')
       import :: c_int, c_ptr, c_int32_t, fdtd_region, fdtd_lorentz_desc
       type(c_ptr), value :: job
       type(fdtd_region), intent(in) :: region
       type(fdtd_lorentz_desc), intent(in) :: params
       integer(c_int32_t), intent(out) :: material_id
     end function fdtd_add_lorentz
     integer(c_int) function fdtd_add_conductive(job, region, eps_inf, sigma, material_id) &
          bind(c, name='fdtd_add_conductive')
       import :: c_int, c_ptr, c_double, c_int32_t, fdtd_region
       type(c_ptr), value :: job
       type(fdtd_region), intent(in) :: region
       real(c_double), value :: eps_inf, sigma
       integer(c_int32_t), intent(out) :: material_id
     end function fdtd_add_conductive
     integer(c_int) function fdtd_add_graphene_nk(job, region, params, material_id) bind(c, name='fdtd_add_graphene_nk')
       import :: c_int, c_ptr, c_int32_t, fdtd_region, fdtd_graphene_nk_desc
       type(c_ptr), value :: job
       type(fdtd_region), intent(in) :: region
       type(fdtd_graphene_nk_desc), intent(in) :: params
       integer(c_int32_t), intent(out) :: material_id
     end function fdtd_add_graphene_nk
     integer(c_int) function fdtd_add_graphene_cp(job, region, params, material_id) bind(c, name='fdtd_add_graphene_cp')
       import :: c_int, c_ptr, c_int32_t, fdtd_region, fdtd_graphene_cp_desc
       type(c_ptr), value :: job
       type(fdtd_region), intent(in) :: region
       type(fdtd_graphene_cp_desc), intent(in) :: params
       integer(c_int32_t), intent(out) :: material_id
     end function fdtd_add_graphene_cp
     integer(c_int) function fdtd_add_pml(job, pml) bind(c, name='fdtd_add_pml')
       import :: c_int, c_ptr, fdtd_pml_desc
       type(c_ptr), value :: job
       type(fdtd_pml_desc), intent(in) :: pml
     end function fdtd_add_pml
     integer(c_int) function fdtd_add_tfsf_1d(job, tfsf) bind(c, name='fdtd_add_tfsf_1d')
       import :: c_int, c_ptr, fdtd_tfsf1d_desc
       type(c_ptr), value :: job
       type(fdtd_tfsf1d_desc), intent(in) :: tfsf
     end function fdtd_add_tfsf_1d
     integer(c_int) function fdtd_add_tfsf(job, tfsf) bind(c, name='fdtd_add_tfsf')
       import :: c_int, c_ptr, fdtd_tfsf_desc
       type(c_ptr), value :: job
       type(fdtd_tfsf_desc), intent(in) :: tfsf
     end function fdtd_add_tfsf
     integer(c_int) function fdtd_add_source(job, src, id) bind(c, name='fdtd_add_source')
       import :: c_int, c_ptr, c_int32_t, fdtd_source_desc
       type(c_ptr), value :: job
       type(fdtd_source_desc), intent(in) :: src
       integer(c_int32_t), intent(out) :: id
     end function fdtd_add_source
     integer(c_int) function fdtd_add_monitor(job, mon, id) bind(c, name='fdtd_add_monitor')
       import :: c_int, c_ptr, c_int32_t, fdtd_monitor_desc
       type(c_ptr), value :: job
       type(fdtd_monitor_desc), intent(in) :: mon
       integer(c_int32_t), intent(out) :: id
     end function fdtd_add_monitor
     integer(c_int) function fdtd_add_probe(job, probe, id) bind(c, name='fdtd_add_probe')
       import :: c_int, c_ptr, c_int32_t, fdtd_probe_desc
       type(c_ptr), value :: job
       type(fdtd_probe_desc), intent(in) :: probe
       integer(c_int32_t), intent(out) :: id
     end function fdtd_add_probe
     integer(c_int) function fdtd_commit(job) bind(c, name='fdtd_commit')
       import :: c_int, c_ptr
       type(c_ptr), value :: job
     end function fdtd_commit

     ! ---- the time loop: the whole body, or the reference's procedures one by one ----
     integer(c_int) function fdtd_step(job, n_first, n_steps) bind(c, name='fdtd_step')
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: job
       integer(c_int32_t), value :: n_first, n_steps
     end function fdtd_step
     integer(c_int) function fdtd_update_DE(job, n) bind(c, name='fdtd_update_DE')
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: job
       integer(c_int32_t), value :: n
     end function fdtd_update_DE
     integer(c_int) function fdtd_pml_update_E(job, n) bind(c, name='fdtd_pml_update_E')
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: job
       integer(c_int32_t), value :: n
     end function fdtd_pml_update_E
     integer(c_int) function fdtd_interchange(job, which) bind(c, name='fdtd_interchange')
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: job
       integer(c_int32_t), value :: which
     end function fdtd_interchange
     integer(c_int) function fdtd_update_H(job, n) bind(c, name='fdtd_update_H')
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: job
       integer(c_int32_t), value :: n
     end function fdtd_update_H
     integer(c_int) function fdtd_pml_update_H(job, n) bind(c, name='fdtd_pml_update_H')
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: job
       integer(c_int32_t), value :: n
     end function fdtd_pml_update_H
     integer(c_int) function fdtd_sample(job, n) bind(c, name='fdtd_sample')
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: job
       integer(c_int32_t), value :: n
     end function fdtd_sample

     ! ---- checkpoints and health ----
     integer(c_int) function fdtd_state_bytes(job, bytes) bind(c, name='fdtd_state_bytes')
       import :: c_int, c_ptr, c_int64_t
       type(c_ptr), value :: job
       integer(c_int64_t), intent(out) :: bytes
     end function fdtd_state_bytes
     integer(c_int) function fdtd_save_state(job, buf, bytes) bind(c, name='fdtd_save_state')
       import :: c_int, c_ptr, c_int8_t, c_int64_t
       type(c_ptr), value :: job
       integer(c_int8_t), intent(out) :: buf(*)
       integer(c_int64_t), value :: bytes
     end function fdtd_save_state
     integer(c_int) function fdtd_load_state(job, buf, bytes) bind(c, name='fdtd_load_state')
       import :: c_int, c_ptr, c_int8_t, c_int64_t
       type(c_ptr), value :: job
       integer(c_int8_t), intent(in) :: buf(*)
       integer(c_int64_t), value :: bytes
     end function fdtd_load_state
     integer(c_int) function fdtd_check_finite(job, count) bind(c, name='fdtd_check_finite')
       import :: c_int, c_ptr, c_int64_t
       type(c_ptr), value :: job
       integer(c_int64_t), intent(out) :: count
     end function fdtd_check_finite
     integer(c_int) function fdtd_debug_fail_alloc(after) bind(c, name='fdtd_debug_fail_alloc')
       import :: c_int, c_int32_t
       integer(c_int32_t), value :: after
     end function fdtd_debug_fail_alloc
     integer(c_int) function fdtd_debug_wait_limit(job, rounds) bind(c, name='fdtd_debug_wait_limit')
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: job
       integer(c_int32_t), value :: rounds
     end function fdtd_debug_wait_limit

     ! ---- results ----
     integer(c_int) function fdtd_sync(job) bind(c, name='fdtd_sync')
       import :: c_int, c_ptr
       type(c_ptr), value :: job
     end function fdtd_sync
     integer(c_int) function fdtd_get_field(job, comp, host) bind(c, name='fdtd_get_field')
       import :: c_int, c_ptr, c_int32_t, c_double
       type(c_ptr), value :: job
       integer(c_int32_t), value :: comp
       real(c_double), intent(out) :: host(*)
     end function fdtd_get_field
     integer(c_int) function fdtd_set_field(job, comp, host) bind(c, name='fdtd_set_field')
       import :: c_int, c_ptr, c_int32_t, c_double
       type(c_ptr), value :: job
       integer(c_int32_t), value :: comp
       real(c_double), intent(in) :: host(*)
     end function fdtd_set_field
     integer(c_int) function fdtd_get_monitor(job, id, re, im) bind(c, name='fdtd_get_monitor')
       import :: c_int, c_ptr, c_int32_t, c_double
       type(c_ptr), value :: job
       integer(c_int32_t), value :: id
       real(c_double), intent(out) :: re(*), im(*)
     end function fdtd_get_monitor
     integer(c_int) function fdtd_get_probe(job, id, host, count) bind(c, name='fdtd_get_probe')
       import :: c_int, c_ptr, c_int32_t, c_double
       type(c_ptr), value :: job
       integer(c_int32_t), value :: id
       real(c_double), intent(out) :: host(*)
       integer(c_int32_t), intent(out) :: count
     end function fdtd_get_probe
     integer(c_int) function fdtd_device_bytes(job, bytes) bind(c, name='fdtd_device_bytes')
       import :: c_int, c_ptr, c_int64_t
       type(c_ptr), value :: job
       integer(c_int64_t), intent(out) :: bytes
     end function fdtd_device_bytes
     integer(c_int) function fdtd_estimate_bytes(job, bytes) bind(c, name='fdtd_estimate_bytes')
       import :: c_int, c_ptr, c_int64_t
       type(c_ptr), value :: job
       integer(c_int64_t), intent(out) :: bytes
     end function fdtd_estimate_bytes

     ! ---- measurement ----
     integer(c_int) function fdtd_profile(job, enable) bind(c, name='fdtd_profile')
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: job
       integer(c_int32_t), value :: enable
     end function fdtd_profile
     integer(c_int) function fdtd_kernel_time(job, kind, launches, ms) bind(c, name='fdtd_kernel_time')
       import :: c_int, c_ptr, c_int32_t, c_int64_t, c_double
       type(c_ptr), value :: job
       integer(c_int32_t), value :: kind
       integer(c_int64_t), intent(out) :: launches
       real(c_double), intent(out) :: ms
     end function fdtd_kernel_time
     integer(c_int) function fdtd_set_tile(job, tile) bind(c, name='fdtd_set_tile')
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: job
       integer(c_int32_t), value :: tile
     end function fdtd_set_tile
     integer(c_int) function fdtd_get_tile(job, tile) bind(c, name='fdtd_get_tile')
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: job
       integer(c_int32_t), intent(out) :: tile
     end function fdtd_get_tile
     integer(c_int) function fdtd_kernel_cells(job, kind, cells) bind(c, name='fdtd_kernel_cells')
       import :: c_int, c_ptr, c_int32_t, c_int64_t
       type(c_ptr), value :: job
       integer(c_int32_t), value :: kind
       integer(c_int64_t), intent(out) :: cells
     end function fdtd_kernel_cells
     integer(c_int) function fdtd_launch_count(job, launches) bind(c, name='fdtd_launch_count')
       import :: c_int, c_ptr, c_int64_t
       type(c_ptr), value :: job
       integer(c_int64_t), intent(out) :: launches
     end function fdtd_launch_count
     integer(c_int) function fdtd_set_stream(job, cuda_stream) bind(c, name='fdtd_set_stream')
       import :: c_int, c_ptr
       type(c_ptr), value :: job
       type(c_ptr), value :: cuda_stream
     end function fdtd_set_stream
     integer(c_int) function fdtd_transfer_bytes(job, h2d, d2h) bind(c, name='fdtd_transfer_bytes')
       import :: c_int, c_ptr, c_int64_t
       type(c_ptr), value :: job
       integer(c_int64_t), intent(out) :: h2d, d2h
     end function fdtd_transfer_bytes

     ! ---- serving many jobs ----
     integer(c_int) function fdtd_server_create(desc, server) bind(c, name='fdtd_server_create')
       import :: c_int, c_ptr, fdtd_server_desc
       type(fdtd_server_desc), intent(in) :: desc
       type(c_ptr), intent(out) :: server
     end function fdtd_server_create
     integer(c_int) function fdtd_server_submit(server, job, n_steps, ticket) bind(c, name='fdtd_server_submit')
       import :: c_int, c_ptr, c_int32_t, c_int64_t
       type(c_ptr), value :: server
       type(c_ptr), value :: job
       integer(c_int32_t), value :: n_steps
       integer(c_int64_t), intent(out) :: ticket
     end function fdtd_server_submit
     integer(c_int) function fdtd_server_wait(server, ticket, timeout_ms, state) bind(c, name='fdtd_server_wait')
       import :: c_int, c_ptr, c_int32_t, c_int64_t
       type(c_ptr), value :: server
       integer(c_int64_t), value :: ticket
       integer(c_int32_t), value :: timeout_ms
       integer(c_int32_t), intent(out) :: state
     end function fdtd_server_wait
     integer(c_int) function fdtd_server_job(server, ticket, job) bind(c, name='fdtd_server_job')
       import :: c_int, c_ptr, c_int64_t
       type(c_ptr), value :: server
       integer(c_int64_t), value :: ticket
       type(c_ptr), intent(out) :: job
     end function fdtd_server_job
     integer(c_int) function fdtd_server_times(server, ticket, t_submit, t_admit, t_done) bind(c, name='fdtd_server_times')
       import :: c_int, c_ptr, c_int64_t, c_double
       type(c_ptr), value :: server
       integer(c_int64_t), value :: ticket
       real(c_double), intent(out) :: t_submit, t_admit, t_done
     end function fdtd_server_times
     integer(c_int) function fdtd_server_release(server, ticket) bind(c, name='fdtd_server_release')
       import :: c_int, c_ptr, c_int64_t
       type(c_ptr), value :: server
       integer(c_int64_t), value :: ticket
     end function fdtd_server_release
     integer(c_int) function fdtd_server_stats(server, stats) bind(c, name='fdtd_server_stats')
       import :: c_int, c_ptr, fdtd_server_status
       type(c_ptr), value :: server
       type(fdtd_server_status), intent(out) :: stats
     end function fdtd_server_stats
     integer(c_int) function fdtd_server_destroy(server) bind(c, name='fdtd_server_destroy')
       import :: c_int, c_ptr
       type(c_ptr), value :: server
     end function fdtd_server_destroy

     ! ---- the allocation-free DFT of a caller-owned device field ----
     integer(c_int) function fdtd_dft_sample_noalloc(field, precision, nx, ny, nz, lo, hi, n, n_first, n_last, &
          dt, omega, nfreq, acc_re, acc_im, flush, stream) bind(c, name='fdtd_dft_sample_noalloc')
       import :: c_int, c_ptr, c_int32_t, c_double
       type(c_ptr), value :: field                ! device array
       integer(c_int32_t), value :: precision, nx, ny, nz
       integer(c_int32_t), intent(in) :: lo(3), hi(3)
       integer(c_int32_t), value :: n, n_first, n_last
       real(c_double), value :: dt
       type(c_ptr), value :: omega                ! device array (nfreq)
       integer(c_int32_t), value :: nfreq
       type(c_ptr), value :: acc_re, acc_im       ! device arrays (nfreq * cells)
       integer(c_int32_t), value :: flush
       type(c_ptr), value :: stream
     end function fdtd_dft_sample_noalloc
  end interface
end module fdtd_gpu_mod
