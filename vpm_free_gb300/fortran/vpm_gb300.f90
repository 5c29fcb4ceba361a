!------------------------------------------------------------------------------
! vpm_gb300.f90 -- Fortran 2003 binding of libvpmg.so (include/vpmg.h).
!
! Drop-in replacement, for a one-block run on one GPU, of the modules that a
! vpm_free host program uses on its hot path:
!   module vpm_lib : subroutine vpm(XP,QP,UP,GP,NVR,neqpm,WhatToDo,RHS_pm,
!                    velx,vely,velz,NTIME,NI,NVRM)      (source/vpm.f90:54-74)
!                    subroutine remesh_particles_3d(iflag)
!                                                      (source/vpm_remesh.f90:5)
!   module pmgrid  : mesh extents and counts that the host reads after
!                    WhatToDo = 0 (source/main_pm.f90:15-22)
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
  end interface
end module vpmg_c

module pmgrid
  ! the mesh variables of source/main_pm.f90 that host programs read
  double precision, save :: XMIN_pm, XMAX_pm, YMIN_pm, YMAX_pm, ZMIN_pm, ZMAX_pm
  double precision, save :: DXpm, DYpm, DZpm, DVpm
  integer, save          :: NXpm, NYpm, NZpm
  integer, save          :: NXs_bl(10), NYs_bl(10), NXf_bl(10), NYf_bl(10), NZs_bl(10), NZf_bl(10)
  double precision, allocatable, target, save :: velvrx_pm(:,:,:), velvry_pm(:,:,:), velvrz_pm(:,:,:)
end module pmgrid

module vpm_lib
  use vpmg_c
  implicit none
  type(c_ptr), save :: vpmg_h = c_null_ptr
  private :: vpmg_h, check, sync_pmgrid

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

  subroutine sync_pmgrid()
    use pmgrid
    type(vpmg_sizes) :: s
    call check(vpmg_get_sizes(vpmg_h, s), 'vpmg_get_sizes')
    XMIN_pm = s%xbound(1); YMIN_pm = s%xbound(2); ZMIN_pm = s%xbound(3)
    XMAX_pm = s%xbound(4); YMAX_pm = s%xbound(5); ZMAX_pm = s%xbound(6)
    DXpm = s%dpm(1); DYpm = s%dpm(2); DZpm = s%dpm(3); DVpm = s%dvpm
    NXpm = s%nn(1); NYpm = s%nn(2); NZpm = s%nn(3)
    NXs_bl(1) = s%nn_bl(1); NYs_bl(1) = s%nn_bl(2); NZs_bl(1) = s%nn_bl(3)
    NXf_bl(1) = s%nn_bl(4); NYf_bl(1) = s%nn_bl(5); NZf_bl(1) = s%nn_bl(6)
  end subroutine sync_pmgrid

  ! source/vpm.f90:54-74 signature; WhatToDo 0 and 2 on the GPU.
  subroutine vpm(XP_in, QP_in, UP_in, GP_in, NVR_in, neqpm_in, WhatToDo, RHS_pm_in, velx, vely, velz, &
                 NTIME_in, NI_in, NVRM_in)
    use pmgrid
    double precision, intent(inout), target  :: XP_in(:,:), QP_in(:,:), UP_in(:,:), GP_in(:,:)
    double precision, intent(inout), pointer :: RHS_pm_in(:,:,:,:)
    double precision, intent(inout), pointer :: velx(:,:,:), vely(:,:,:), velz(:,:,:)
    integer, intent(inout) :: NVR_in
    integer, intent(in)    :: neqpm_in, WhatToDo, NVRM_in, NTIME_in
    double precision, intent(in) :: NI_in
    type(vpmg_config) :: cfg
    integer(c_int) :: nvr
    double precision :: dummy(1)

    nullify(RHS_pm_in)
    if (.not. c_associated(vpmg_h)) then
       call check(vpmg_read_pm_inp('pm.inp'//c_null_char, cfg), 'pm.inp')
       call check(vpmg_create(cfg, -1_c_int, vpmg_h), 'vpmg_create')
       ! the reference's writers after the velocity: solution windows and hist lines
       call check(vpmg_set_output(vpmg_h, '.'//c_null_char, 3_c_int), 'vpmg_set_output')
    end if
    nvr = NVR_in
    if (WhatToDo == 0) then
       call check(vpmg_vpm(vpmg_h, XP_in, QP_in, dummy, dummy, nvr, neqpm_in, 0, NTIME_in, NI_in, NVRM_in), 'vpm(0)')
       call sync_pmgrid()
       if (allocated(velvrx_pm)) deallocate(velvrx_pm, velvry_pm, velvrz_pm)
       allocate(velvrx_pm(NXpm, NYpm, NZpm), velvry_pm(NXpm, NYpm, NZpm), velvrz_pm(NXpm, NYpm, NZpm))
       velvrx_pm = 0.d0; velvry_pm = 0.d0; velvrz_pm = 0.d0
       nullify(velx, vely, velz)
       velx => velvrx_pm; vely => velvry_pm; velz => velvrz_pm
    else
       call check(vpmg_vpm(vpmg_h, XP_in, QP_in, UP_in, GP_in, nvr, neqpm_in, WhatToDo, NTIME_in, NI_in, &
                           NVRM_in), 'vpm')
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
