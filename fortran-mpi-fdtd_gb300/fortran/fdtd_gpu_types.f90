! fdtd_gpu_types -- the reference's object names on top of fdtd_gpu_mod: a
! program written against the reference's modules (ConstantDielectric, Gold,
! pmly, and the time loop's updateD / updateH / interchange_E / interchange_H)
! changes its use lines and object types and keeps its calls.
!
! A gpu_domain holds the job (the whole grid on one GPU: the MPI slabs become
! one array).  The engine does every material's D -> E update inside
! fdtd_update_DE, so each material's update_E is a no-op and the order of the
! initialize_material calls takes the place of the order of the update_E
! calls (3D/air-AuAntennasSiO2-Si/program.f90:411-414): a later material wins
! on shared cells.  It builds against the reference's own mydatatypes and
! constants_mod (modules/src/misc).
module fdtd_gpu_types
  use iso_c_binding
  use fdtd_gpu_mod
  use mydatatypes, only: Irange          ! the reference's own range type
  use constants_mod, only: ep0
  implicit none
  private
  public :: gpu_domain, gpu_dielectric, gpu_gold, gpu_pmly

  type :: gpu_domain                     ! the whole grid: one job
     type(c_ptr) :: job = c_null_ptr
     logical :: committed = .false.
  contains
     procedure :: create => domain_create
     procedure :: updateD => domain_updateD          ! updateD + source + every update_E
     procedure :: updateH => domain_updateH
     procedure :: interchange_E => domain_interchange_E
     procedure :: interchange_H => domain_interchange_H
     procedure :: sample => domain_sample            ! the DFT blocks of step n
  end type

  type :: gpu_material                   ! material_mod's extent (M3/material_mod.f90:8)
     integer :: xinit = 0, xend = 0, yinit = 0, yend = 0, zinit = 0, zend = 0
     type(gpu_domain), pointer :: dom => null()
     integer(c_int32_t) :: id = -1
  contains
     procedure :: update_E => material_update_E
  end type
  type, extends(gpu_material) :: gpu_dielectric   ! ConstantDielectric
     real(c_double) :: constant_ep = 1.d0
  contains
     procedure :: initialize_material => dielectric_initialize
  end type
  type, extends(gpu_material) :: gpu_gold         ! Gold, with its defaults (M3/gold_mod.f90:28-34)
     real(c_double) :: epinf = 1.1431d0, dnur = 1.0805d14, wD = 1.3202d16
     real(c_double) :: ap(2) = (/ 0.26698d0, 3.0834d0 /), phip(2) = (/ -1.2371d0, -1.0968d0 /)
     real(c_double) :: omp(2) = (/ 3.8711d15, 4.1684d15 /), rp(2) = (/ 4.4642d14, 2.4555d15 /)
  contains
     procedure :: initialize_material => gold_initialize
  end type
  type :: gpu_pmly                       ! pmly (M3/BERpmly_mod.f90:485-508)
     type(gpu_domain), pointer :: dom => null()
  contains
     procedure :: initialize => pmly_initialize
     procedure :: updateE => pmly_updateE
     procedure :: updateH => pmly_updateH
  end type

contains

  subroutine check(ierr)
     integer(c_int), intent(in) :: ierr
     character(kind=c_char) :: msg(512)
     integer(c_int) :: rc
     if (ierr /= 0) then
        rc = fdtd_last_error(msg, int(size(msg), c_size_t))
        write(*,*) 'fdtd error ', ierr, ': ', msg(1:index(transfer(msg, repeat(' ', 512)), c_null_char) - 1)
        stop 1
     end if
  end subroutine

  subroutine domain_create(this, g)
     class(gpu_domain), intent(inout) :: this
     type(fdtd_grid_desc), intent(in) :: g
     call check(fdtd_create(g, this%job))
  end subroutine

  subroutine commit_once(this)           ! after every material, the PML, sources and monitors
     class(gpu_domain), intent(inout) :: this
     if (.not. this%committed) call check(fdtd_commit(this%job))
     this%committed = .true.
  end subroutine

  subroutine domain_updateD(this, n)
     class(gpu_domain), intent(inout) :: this
     integer, intent(in) :: n
     call commit_once(this)
     call check(fdtd_update_DE(this%job, int(n, c_int32_t)))
  end subroutine
  subroutine domain_updateH(this, n)
     class(gpu_domain), intent(inout) :: this
     integer, intent(in) :: n
     call check(fdtd_update_H(this%job, int(n, c_int32_t)))
  end subroutine
  subroutine domain_interchange_E(this)
     class(gpu_domain), intent(inout) :: this
     call check(fdtd_interchange(this%job, 0_c_int32_t))
  end subroutine
  subroutine domain_interchange_H(this)
     class(gpu_domain), intent(inout) :: this
     call check(fdtd_interchange(this%job, 1_c_int32_t))
  end subroutine
  subroutine domain_sample(this, n)
     class(gpu_domain), intent(inout) :: this
     integer, intent(in) :: n
     call check(fdtd_sample(this%job, int(n, c_int32_t)))
  end subroutine

  subroutine material_update_E(this, Ex_pointer, Ey_pointer, Ez_pointer, Dx_pointer, Dy_pointer, Dz_pointer)
     class(gpu_material) :: this
     real*8, pointer, intent(inout) :: Ex_pointer(:,:,:), Ey_pointer(:,:,:), Ez_pointer(:,:,:)
     real*8, pointer, intent(inout) :: Dx_pointer(:,:,:), Dy_pointer(:,:,:), Dz_pointer(:,:,:)
     ! nothing: domain%updateD ran this material's D -> E update on the device
  end subroutine

  function extent(this) result(r)       ! absolute 1-based ranges -> a 0-based box
     class(gpu_material), intent(in) :: this
     type(fdtd_region) :: r
     r%kind = FDTD_REGION_BOX
     r%lo = (/ this%xinit, this%yinit, this%zinit /) - 1
     r%hi = (/ this%xend, this%yend, this%zend /) - 1
     r%count = 0
  end function

  subroutine dielectric_initialize(this, rangex, rangey, rangez, range_localdim)
     class(gpu_dielectric), intent(inout) :: this
     type(Irange), intent(in) :: rangex, rangey, rangez     ! one domain: the whole grid
     integer, intent(in) :: range_localdim(3)
     call check(fdtd_add_dielectric(this%dom%job, extent(this), this%constant_ep, this%id))
  end subroutine

  subroutine gold_initialize(this, rangex, rangey, rangez, range_localdim)
     class(gpu_gold), intent(inout) :: this
     type(Irange), intent(in) :: rangex, rangey, rangez
     integer, intent(in) :: range_localdim(3)
     type(fdtd_drude2cp) :: p
     p = fdtd_drude2cp(this%epinf, this%wD, this%dnur, this%ap, this%phip, this%omp, this%rp)
     call check(fdtd_add_gold(this%dom%job, extent(this), p, this%id))
  end subroutine

  subroutine pmly_initialize(this, eplow, ephigh, sigmam, npmls, order, dt, ds, coords, ranks, maxs)
     class(gpu_pmly), intent(inout) :: this
     real*8, intent(in) :: eplow, ephigh, sigmam, order, dt, ds
     integer, intent(in) :: npmls(3), coords(3), ranks(3), maxs(3)
     type(fdtd_pml_desc) :: p
     p%mode = FDTD_PML_REFERENCE
     p%npml = reshape((/ npmls(1), npmls(1), npmls(2), npmls(2), npmls(3), npmls(3) /), (/ 2, 3 /))
     p%eps_lo = eplow / ep0
     p%eps_hi = ephigh / ep0
     p%sigma_max = sigmam
     p%order = order
     call check(fdtd_add_pml(this%dom%job, p))
  end subroutine
  subroutine pmly_updateE(this, n)
     class(gpu_pmly), intent(inout) :: this
     integer, intent(in) :: n
     call check(fdtd_pml_update_E(this%dom%job, int(n, c_int32_t)))
  end subroutine
  subroutine pmly_updateH(this, n)
     class(gpu_pmly), intent(inout) :: this
     integer, intent(in) :: n
     call check(fdtd_pml_update_H(this%dom%job, int(n, c_int32_t)))
  end subroutine
end module fdtd_gpu_types
