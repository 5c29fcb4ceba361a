!------------------------------------------------------------------------------
! vpm_gb300.f90 -- Fortran 2003 binding of libvpmg.so (include/vpmg.h).
!
! Drop-in replacement, for a one-block run on one GPU, of the modules that a
! vpm_free host program uses on its hot path:
!   module vpm_vars, vpm_size, openmpth : the scalars and mesh descriptors
!                    of source/vpm.f90:1-39 that hosts read or set (mrem,
!                    interf_iproj, neqpm, Xbound, Dpm, NN, NN_bl, st, et, ...)
!   module vpm_lib : re-exports them (source/vpm.f90:42-44) and holds
!                    subroutine vpm(XP,QP,UP,GP,NVR,neqpm,WhatToDo,RHS_pm,
!                    velx,vely,velz,NTIME,NI,NVRM)      (source/vpm.f90:54-74)
!                    subroutine remesh_particles_3d(iflag)
!                                                      (source/vpm_remesh.f90:5)
!   module pmgrid  : mesh extents and counts that the host reads after
!                    WhatToDo = 0, and velvr[xyz]_pm (source/main_pm.f90:2-45)
!   module projlib : projection_fun (source/pmproject.f90:391-431)
! The host keeps its particle arrays (XPR, QPR from module test_mod,
! source/testmod.f90:2) and pm.inp; the library copies particles to and from
! the GPU inside each call.  Link this file and -lvpmg -lcudart in place of
! vpm.o pmlib.o pmproject.o yaps.o vpm_mpi.o vpm_time.o vpm_gcalc.o
! vpm_remesh.o main_pm.o libpm.o mkl_dfti.o (and without -mkl).
!------------------------------------------------------------------------------
module vpmg_c
  use iso_c_binding
  implicit none

  type, bind(C) :: vpmg_config
     real(c_double)  :: dpm(3)
     integer(c_int)  :: interf_iproj, ibctyp, idvpm
     real(c_double)  :: epsvol
     integer(c_int)  :: ncoarse, nbi, nbj, nbk, nremesh, ncell_rem, iyntree, ilevmax
     integer(c_int)  :: ompthreads, idefine, iynslice, use_box
     real(c_double)  :: box(6)
     integer(c_int)  :: ipmwrite, ipmwstart(10), ipmwsteps(10)
  end type vpmg_config

  type, bind(C) :: vpmg_sizes
     real(c_double)  :: xbound(6), dpm(3)
     integer(c_int)  :: nn(3), nn_bl(6)
     real(c_double)  :: xbound_bl(6)
     integer(c_int)  :: nnbl(3), nnbl_bl(6)
     real(c_double)  :: xbound_coarse(6), dpm_coarse(3)
     integer(c_int)  :: nn_coarse(3), nn_bl_coarse(6)
     integer(c_int)  :: ilevmax
     real(c_double)  :: dvpm
     integer(c_int)  :: defined
  end type vpmg_sizes

  integer(c_int), parameter :: VPMG_F_VEL = 2

  interface
     integer(c_int) function vpmg_read_pm_inp(path, cfg) bind(C, name="vpmg_read_pm_inp")
       import :: c_int, c_char, vpmg_config
       character(kind=c_char), dimension(*), intent(in) :: path
       type(vpmg_config), intent(out) :: cfg
     end function vpmg_read_pm_inp

     integer(c_int) function vpmg_create(cfg, device, h) bind(C, name="vpmg_create")
       import :: c_int, c_ptr, vpmg_config
       type(vpmg_config), intent(in) :: cfg
       integer(c_int), value :: device
       type(c_ptr), intent(out) :: h
     end function vpmg_create

     integer(c_int) function vpmg_vpm(h, xp, qp, up, gp, nvr, neqpm, whattodo, ntime, ni, nvrm) &
          bind(C, name="vpmg_vpm")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: h
       real(c_double), intent(inout) :: xp(*), qp(*), up(*), gp(*)
       integer(c_int), intent(inout) :: nvr
       integer(c_int), value :: neqpm, whattodo, ntime, nvrm
       real(c_double), value :: ni
     end function vpmg_vpm

     integer(c_int) function vpmg_remesh_particles_3d(h, iflag, xp, qp, nvr, capacity) &
          bind(C, name="vpmg_remesh_particles_3d")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: h
       integer(c_int), value :: iflag, capacity
       real(c_double), intent(inout) :: xp(*), qp(*)
       integer(c_int), intent(inout) :: nvr
     end function vpmg_remesh_particles_3d

     integer(c_int) function vpmg_get_sizes(h, s) bind(C, name="vpmg_get_sizes")
       import :: c_int, c_ptr, vpmg_sizes
       type(c_ptr), value :: h
       type(vpmg_sizes), intent(out) :: s
     end function vpmg_get_sizes

     integer(c_int) function vpmg_get_field(h, which, out, capacity, count) bind(C, name="vpmg_get_field")
       import :: c_int, c_ptr, c_double, c_size_t
       type(c_ptr), value :: h
       integer(c_int), value :: which
       real(c_double), intent(out) :: out(*)
       integer(c_size_t), value :: capacity
       integer(c_size_t), intent(out) :: count
     end function vpmg_get_field

     type(c_ptr) function vpmg_last_error(h) bind(C, name="vpmg_last_error")
       import :: c_ptr
       type(c_ptr), value :: h
     end function vpmg_last_error

     integer(c_int) function vpmg_set_output(h, dir, flags) bind(C, name="vpmg_set_output")
       import :: c_int, c_ptr, c_char
       type(c_ptr), value :: h
       character(kind=c_char), dimension(*) :: dir
       integer(c_int), value :: flags
     end function vpmg_set_output

     real(c_double) function vpmg_projection_fun(itype, x) bind(C, name="vpmg_projection_fun")
       import :: c_int, c_double
       integer(c_int), value :: itype
       real(c_double), value :: x
     end function vpmg_projection_fun
  end interface
end module vpmg_c

! The scalars of the reference's vpm_vars (source/vpm.f90:1-12) that host
! programs read or set; the library keeps its own copies in the handle.
module vpm_vars
  double precision :: DT_c, V_ref, NI
  integer          :: interf_iproj, ncell_rem, iynhj
  integer          :: ncoarse, nparcell1d
  integer          :: neqpm, NVR_p, NVR_size, iwrite, NTIME_pm
  integer, save    :: IPMWRITE, mrem, idefine, iynslice
  integer, save    :: IPMWSTART(10), IPMWSTEPS(10)
end module vpm_vars

! The mesh descriptors of vpm_size (source/vpm.f90:14-30), one block,
! filled by vpm(..., WhatToDo = 0, ...); st/et/ct are the hosts' timers.
module vpm_size
  double precision, save :: Xbound(6), Dpm(3), Xbound0(6), Dpm0(3)
  integer, save          :: NN_bl(6), NN(3), NN0_bl(6), NN0(3)
  double precision, save :: Xbound_tmp(6), Xbound_coarse(6), Dpm_coarse(3)
  integer, save          :: NN_tmp(3), NN_bl_tmp(6), NN_coarse(3), NN_bl_coarse(6)
  integer, save          :: NBB, NXbl, NYbl, NZbl, BLOCKS
  double precision       :: starttime, endtime, st, et, ct
  integer, save          :: iynbc, iret, NBI, NBJ, NBK, NVR_out_thres, NREMESH, ntorder, &
                            iyntree, ilevmax, itree, nsize_out(3), ibctyp, NWRITE
end module vpm_size

module openmpth
  integer :: OMPTHREADS
end module openmpth

module pmgrid
  ! the mesh variables of source/main_pm.f90 that host programs read
  double precision, save :: XMIN_pm, XMAX_pm, YMIN_pm, YMAX_pm, ZMIN_pm, ZMAX_pm
  double precision, save :: DXpm, DYpm, DZpm, DVpm
  integer, save          :: NXpm, NYpm, NZpm
  integer, save          :: NXs_bl(10), NYs_bl(10), NXf_bl(10), NYf_bl(10), NZs_bl(10), NZf_bl(10)
  double precision, allocatable, target, save :: velvrx_pm(:,:,:), velvry_pm(:,:,:), velvrz_pm(:,:,:)
end module pmgrid

! projection_fun of source/pmproject.f90:391-431, evaluated by the library.
module projlib
  use vpmg_c, only: vpmg_projection_fun, c_int, c_double
  implicit none
contains
  double precision function projection_fun(itype, x)
    integer, intent(in) :: itype
    double precision, intent(in) :: x
    projection_fun = vpmg_projection_fun(int(itype, c_int), real(x, c_double))
  end function projection_fun
end module projlib

module vpm_lib
  use vpmg_c
  use vpm_vars
  use vpm_size
  use openmpth
  implicit none
  type(c_ptr), save :: vpmg_h = c_null_ptr
  private :: vpmg_h, check, sync_sizes, velocity_to_host

contains

  subroutine check(rc, where)
    integer(c_int), intent(in) :: rc
    character(*), intent(in)   :: where
    character(kind=c_char), pointer :: msg(:)
    integer :: n
    if (rc == 0) return
    write(*,*) 'vpmg error ', rc, ' in ', where
    if (c_associated(vpmg_h)) then
       call c_f_pointer(vpmg_last_error(vpmg_h), msg, [512])
       n = 0
       do while (n < 512)
          if (msg(n + 1) == c_null_char) exit
          n = n + 1
       end do
       write(*,*) msg(1:n)
    end if
    stop
  end subroutine check

  ! pmgrid, vpm_size and vpm_vars after define_sizes (WhatToDo = 0)
  subroutine sync_sizes(cfg)
    use pmgrid
    type(vpmg_config), intent(in) :: cfg
    type(vpmg_sizes) :: s
    call check(vpmg_get_sizes(vpmg_h, s), 'vpmg_get_sizes')
    XMIN_pm = s%xbound(1); YMIN_pm = s%xbound(2); ZMIN_pm = s%xbound(3)
    XMAX_pm = s%xbound(4); YMAX_pm = s%xbound(5); ZMAX_pm = s%xbound(6)
    DXpm = s%dpm(1); DYpm = s%dpm(2); DZpm = s%dpm(3); DVpm = s%dvpm
    NXpm = s%nn(1); NYpm = s%nn(2); NZpm = s%nn(3)
    NXs_bl(1) = s%nn_bl(1); NYs_bl(1) = s%nn_bl(2); NZs_bl(1) = s%nn_bl(3)
    NXf_bl(1) = s%nn_bl(4); NYf_bl(1) = s%nn_bl(5); NZf_bl(1) = s%nn_bl(6)
    Xbound = s%xbound; Dpm = s%dpm; NN = s%nn; NN_bl = s%nn_bl
    Xbound_coarse = s%xbound_coarse; Dpm_coarse = s%dpm_coarse
    NN_coarse = s%nn_coarse; NN_bl_coarse = s%nn_bl_coarse
    ilevmax = s%ilevmax
    interf_iproj = cfg%interf_iproj; ibctyp = cfg%ibctyp; ncoarse = cfg%ncoarse
    NBI = cfg%nbi; NBJ = cfg%nbj; NBK = cfg%nbk; BLOCKS = NBI * NBJ * NBK
    NREMESH = cfg%nremesh; ncell_rem = cfg%ncell_rem; iyntree = cfg%iyntree
    idefine = cfg%idefine; iynslice = cfg%iynslice; OMPTHREADS = cfg%ompthreads
    IPMWRITE = cfg%ipmwrite; IPMWSTART = cfg%ipmwstart; IPMWSTEPS = cfg%ipmwsteps
  end subroutine sync_sizes

  ! velvr[xyz]_pm <- the resident velocity field (x fastest, as pmgrid's arrays)
  subroutine velocity_to_host()
    use pmgrid
    double precision, allocatable :: f(:)
    integer(c_size_t) :: n, cnt
    n = int(NXpm, c_size_t) * int(NYpm, c_size_t) * int(NZpm, c_size_t)
    allocate(f(3 * n))
    call check(vpmg_get_field(vpmg_h, VPMG_F_VEL, f, 3 * n, cnt), 'vpmg_get_field')
    velvrx_pm = reshape(f(1:n), [NXpm, NYpm, NZpm])
    velvry_pm = reshape(f(n + 1:2 * n), [NXpm, NYpm, NZpm])
    velvrz_pm = reshape(f(2 * n + 1:3 * n), [NXpm, NYpm, NZpm])
    deallocate(f)
  end subroutine velocity_to_host

  ! source/vpm.f90:54-74 signature.  WhatToDo 0: sizes (velvr[xyz]_pm
  ! zeroed, velx/y/z pointed at them, vpm.f90:155-166); 1: Poisson solve,
  ! velvr[xyz]_pm = the velocity (vpm.f90:228-262); 2 and 4: UP += the
  ! interpolated velocity, GP = stretching x volume; 5: viscous diffusion
  ! into GP, velvr[xyz]_pm zeroed (vpm.f90:345-360).  After WhatToDo = 2
  ! the reference deallocates velvr[xyz]_pm (vpm.f90:310); here they keep
  ! their last contents.
  subroutine vpm(XP_in, QP_in, UP_in, GP_in, NVR_in, neqpm_in, WhatToDo, RHS_pm_in, velx, vely, velz, &
                 NTIME_in, NI_in, NVRM_in)
    use pmgrid
    double precision, intent(inout), target  :: XP_in(:,:), QP_in(:,:), UP_in(:,:), GP_in(:,:)
    double precision, intent(inout), pointer :: RHS_pm_in(:,:,:,:)
    double precision, intent(inout), pointer :: velx(:,:,:), vely(:,:,:), velz(:,:,:)
    integer, intent(inout) :: NVR_in
    integer, intent(in)    :: neqpm_in, WhatToDo, NVRM_in, NTIME_in
    double precision, intent(in) :: NI_in
    type(vpmg_config), save :: cfg
    integer(c_int) :: nvr
    double precision :: dummy(1)

    nullify(RHS_pm_in)
    if (.not. c_associated(vpmg_h)) then
       call check(vpmg_read_pm_inp('pm.inp'//c_null_char, cfg), 'pm.inp')
       call check(vpmg_create(cfg, -1_c_int, vpmg_h), 'vpmg_create')
       ! the reference's writers after the velocity: solution windows and hist lines
       call check(vpmg_set_output(vpmg_h, '.'//c_null_char, 3_c_int), 'vpmg_set_output')
    end if
    neqpm = neqpm_in; NTIME_pm = NTIME_in; NI = NI_in
    nvr = NVR_in
    if (WhatToDo == 0) then
       call check(vpmg_vpm(vpmg_h, XP_in, QP_in, dummy, dummy, nvr, neqpm_in, 0, NTIME_in, NI_in, NVRM_in), 'vpm(0)')
       call sync_sizes(cfg)
       if (allocated(velvrx_pm)) deallocate(velvrx_pm, velvry_pm, velvrz_pm)
       allocate(velvrx_pm(NXpm, NYpm, NZpm), velvry_pm(NXpm, NYpm, NZpm), velvrz_pm(NXpm, NYpm, NZpm))
       velvrx_pm = 0.d0; velvry_pm = 0.d0; velvrz_pm = 0.d0
       nullify(velx, vely, velz)
       velx => velvrx_pm; vely => velvry_pm; velz => velvrz_pm
    else
       call check(vpmg_vpm(vpmg_h, XP_in, QP_in, UP_in, GP_in, nvr, neqpm_in, WhatToDo, NTIME_in, NI_in, &
                           NVRM_in), 'vpm')
       if ((WhatToDo == 1 .or. WhatToDo == 5) .and. nvr > 0) then
          if (.not. allocated(velvrx_pm)) &
             allocate(velvrx_pm(NXpm, NYpm, NZpm), velvry_pm(NXpm, NYpm, NZpm), velvrz_pm(NXpm, NYpm, NZpm))
          if (WhatToDo == 1) then
             call velocity_to_host()
          else
             velvrx_pm = 0.d0; velvry_pm = 0.d0; velvrz_pm = 0.d0
          end if
          nullify(velx, vely, velz)
          velx => velvrx_pm; vely => velvry_pm; velz => velvrz_pm
       end if
    end if
    NVR_in = nvr
  end subroutine vpm

  ! source/vpm_remesh.f90:5: works on (and reallocates) XPR/QPR of test_mod.
  subroutine remesh_particles_3d(iflag)
    use test_mod
    use pmgrid
    integer, intent(in) :: iflag
    double precision, allocatable :: xb(:,:), qb(:,:)
    integer(c_int) :: nvr, cap
    cap = NXpm * NYpm * NZpm
    allocate(xb(3, cap), qb(4, cap))
    nvr = NVR_ext
    xb(:, 1:nvr) = XPR(:, 1:nvr)
    qb(:, 1:nvr) = QPR(:, 1:nvr)
    call check(vpmg_remesh_particles_3d(vpmg_h, iflag, xb, qb, nvr, cap), 'remesh_particles_3d')
    deallocate(XPR, QPR)
    allocate(XPR(3, nvr), QPR(4, nvr))
    XPR = xb(:, 1:nvr)
    QPR = qb(:, 1:nvr)
    NVR_ext = nvr
    deallocate(xb, qb)
  end subroutine remesh_particles_3d

end module vpm_lib
