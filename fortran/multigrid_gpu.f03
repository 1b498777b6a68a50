!***********************************************************************
! multigrid_gpu.f03 -- drop-in replacement of PLES's fsrc/multigrid.f03.
!
! The module keeps the name, the public variables and the three entry points
! the rest of PLES uses, with the reference's argument lists:
!   * jpos, islor, nlevmultimax, omega  set by read_simulation_setting
!                                        (fsrc/read_simulation_setting.f03:15)
!   * mul_met(nlevel,jxc,jyc,jzc)        fsrc/stratiParticle.f03:768
!   * wall(nlevel,jxc,jyc,jzc,ncolperproc)                      :769
!   * multi(eps,ficycle,nlevel,jxc,jyc,jzc,kparasta,kparaend,myid,nproc,
!           rightpe,leftpe,tagls,taglr,tagrs,tagrr,islor,bodyforce,
!           bodypressure,tipo,deepl,deepr,iterat,freesurface,ti)  :2881-2887
! so that a PLES build compiles this file in place of fsrc/multigrid.f03
! and links libples_mg.so; no call site changes.  The bodies call the C ABI
! of include/ples_mg.h through ples_mg_iface:
!   * mul_met builds the coefficient hierarchy on the GPU from the node
!     coordinates x, y, z of myarrays_metri3 (what mul_met and wall/sett
!     compute on the CPU); wall has nothing left to do;
!   * multi is one ples_mg_solve on the module arrays fi, rhs and cs1..cs6
!     of myarrays_velo3: the reference's absolute max-norm stop
!     max|r| < eps (multigrid.f03:598-631) and its cap ficycle (counted
!     here in outer FP64 iterations of the defect correction, each a few
!     V-cycles); islor selects the smoother (0 the multicolour point SOR
!     with the module's omega, 1 the eta-line smoother); bodyforce = 1
!     takes tipo for the stop test over fluid cells (multigrid.f03:615-631);
!     freesurface = 1 (with islor = 0; the reference's line SOR ignores it,
!     multigrid.f03:2019) puts the surface pressure next_prs (zero at the
!     first time step, iterat = 1) on the top wall (multigrid.f03:1188-1222).
!     nlevel is overwritten with nlevmultimax, as the reference does
!     (multigrid.f03:122).  The potenziale_ibm calls inside the reference's
!     V-cycle (multigrid.f03:235-241, 515-543) change fi, which the cycle
!     then overwrites with pr1 (:586-592), so they leave the result as it
!     is and none is made here; the pressure step calls
!     ples_mg_potenziale_ibm where PLES calls potenziale_ibm after the solve.
! One MPI rank holds the whole domain on one GPU (nproc = 1); the reference
! needs two or more ranks for z-periodic grids only because of its own
! plane exchanges, which the GPU solve does not have.  On an error the
! solve stops the program with the library's message, where the reference
! would have printed its residual and carried on.
!
! Not compiled in this repository's build (no Fortran compiler on the build
! machines); the bind(C) layouts are checked at set-up against the library
! (ples_mg_layout_ok).
!***********************************************************************
module multigrid_module
    use iso_c_binding
    use ples_mg_iface
    implicit none

    integer jpos
    integer islor
    integer nlevmultimax
    real omega

    ! precision of the GPU V-cycles (mixed: FP32 inside FP64 defect correction)
    integer, save :: gpu_precision = PLES_MG_PREC_MIXED
    ! the handle's settings: islor, bodyforce, freesurface
    integer, private, save :: built(3) = -1

contains

    !-------------------------------------------------------------------
    ! (re)build the GPU hierarchy for a smoother, cell types and surface
    subroutine gpu_build(islor_, bodyforce, freesurface, tipo)
        use scala3
        use period
        use myarrays_metri3
        integer, intent(in) :: islor_, bodyforce, freesurface
        integer(c_int), target, intent(in), optional :: tipo(0:, 0:, 0:)
        type(ples_mg_desc) :: d

        if (.not. ples_mg_layout_ok()) error stop 'multigrid_module: ples_mg.h and libples_mg.so differ'
        d = ples_mg_desc(jx=jx, jy=jy, jz=jz, ip=ip, jp=jp, kp=kp, nlevmax=nlevmultimax, omega=0.d0, &
                         precision=gpu_precision, coords_layout=PLES_MG_COORDS_GHOSTED8, &
                         x=c_null_ptr, y=c_null_ptr, z=c_null_ptr, &
                         dt=dt, device=0, nu_pre=0, nu_post=0, nu_coarse=0, inner_cycles=0, &
                         smoother=PLES_MG_SMOOTHER_LINE, coarsening=0, solid=c_null_ptr, tipo=c_null_ptr, &
                         freesurface=0)
        if (islor_ == 0) then
            d%smoother = PLES_MG_SMOOTHER_POINT
            d%omega = real(omega, c_double)
            d%freesurface = freesurface
        end if
        if (bodyforce == 1 .and. present(tipo)) d%tipo = c_loc(tipo(0, 0, 0))
        if (c_associated(mg_handle)) call ples_mg_destroy(mg_handle)
        call create_on(d, x, y, z)
        built = [islor_, bodyforce, d%freesurface]
    end subroutine gpu_build

    ! ples_mg_create with the node arrays of myarrays_metri3 (extent
    ! -8:n1+8, -8:n2+8, -8:... on one rank); the dummies carry TARGET for
    ! c_loc, the library copies the nodes during the call
    subroutine create_on(d, xg, yg, zg)
        type(ples_mg_desc), intent(inout) :: d
        real(c_double), target, intent(in) :: xg(-8:, -8:, -8:), yg(-8:, -8:, -8:), zg(-8:, -8:, -8:)
        integer(c_int) :: stat
        d%x = c_loc(xg(-8, -8, -8))
        d%y = c_loc(yg(-8, -8, -8))
        d%z = c_loc(zg(-8, -8, -8))
        stat = ples_mg_create(d, mg_handle)
        if (stat /= PLES_MG_OK) error stop 'multigrid_module: ples_mg_create failed'
    end subroutine create_on

    ! ples_mg_solve on fi (0:jx+1,0:jy+1,0:jz+1), rhs (1:jx,1:jy,1:jz) and
    ! cs1..cs6; TARGET dummies for c_loc
    subroutine solve_on(fi_, rhs_, c1, c2, c3, c4, c5, c6, eps, ficycle, st, stat)
        real(c_double), target, contiguous, intent(inout) :: fi_(0:, 0:, 0:)
        real(c_double), target, contiguous, intent(in) :: rhs_(:, :, :)
        real(c_double), target, contiguous, intent(in) :: c1(:, :), c2(:, :), c3(:, :), c4(:, :), c5(:, :), c6(:, :)
        real(c_double), intent(in) :: eps
        integer, intent(in) :: ficycle
        type(ples_mg_stats), intent(out) :: st
        integer(c_int), intent(out) :: stat
        type(c_ptr), target :: cs(6)
        cs = [c_loc(c1), c_loc(c2), c_loc(c3), c_loc(c4), c_loc(c5), c_loc(c6)]
        stat = ples_mg_solve(mg_handle, c_loc(fi_), c_loc(rhs_), c_loc(cs), 0.d0, eps, int(ficycle, c_int), st)
    end subroutine solve_on

    ! the surface pressure of level 1: next_prs(1:jx,1:jz), which carries
    ! the halo of its rank, arrives here as an explicit-shape (copied,
    ! contiguous) array
    subroutine surface_on(prs, nx, nz)
        integer, intent(in) :: nx, nz
        real(c_double), target, intent(in) :: prs(nx, nz)
        integer(c_int) :: stat
        stat = ples_mg_set_surface_pressure(mg_handle, c_loc(prs))
        if (stat /= PLES_MG_OK) error stop 'multi: ples_mg_set_surface_pressure failed'
    end subroutine surface_on

    !-------------------------------------------------------------------
    ! set-up of the coarse metric (fsrc/multigrid.f03:2293-3052): the whole
    ! hierarchy is built on the GPU from the node coordinates
    subroutine mul_met(nlevel, jxc, jyc, jzc)
        integer nlevel
        integer jxc(0:4), jyc(0:4), jzc(0:4)
        call gpu_build(islor, 0, 0)
    end subroutine mul_met

    !-------------------------------------------------------------------
    ! set-up of the line-solve coefficients (fsrc/multigrid.f03:3151-3264):
    ! part of the hierarchy mul_met built
    subroutine wall(nlevel, jxc, jyc, jzc, ncolperproc)
        integer nlevel, ncolperproc
        integer jxc(0:4), jyc(0:4), jzc(0:4)
    end subroutine wall

    !-------------------------------------------------------------------
    ! the pressure solve (fsrc/multigrid.f03:42-653)
    subroutine multi(eps, ficycle, nlevel, &
        jxc, jyc, jzc, &
        kparasta, kparaend, myid, nproc, &
        rightpe, leftpe, &
        tagls, taglr, tagrs, tagrr, islor, &
        bodyforce, bodypressure, tipo, deepl, deepr, iterat, &
        freesurface, ti)
        use myarrays_velo3
        use scala3
        integer nlevel, ficycle
        integer jxc(0:4), jyc(0:4), jzc(0:4)
        integer kparasta, kparaend, myid, nproc
        integer rightpe, leftpe, tagls, taglr, tagrs, tagrr
        integer islor, bodyforce, bodypressure
        integer deepl, deepr, iterat, freesurface
        integer, target :: tipo(0:n1+1, 0:n2+1, kparasta-deepl:kparaend+deepr)
        real eps, ti
        integer(c_int), allocatable, target :: tipo_c(:, :, :)
        real(c_double), allocatable :: fi_c(:, :, :)
        type(ples_mg_stats) :: st
        integer(c_int) :: stat
        integer :: fs

        if (nproc /= 1) error stop 'multi: the GPU solve holds the whole domain on one rank (nproc = 1)'
        nlevel = nlevmultimax
        fs = 0
        if (islor == 0) fs = freesurface
        if (any(built /= [islor, bodyforce, fs])) then
            if (bodyforce == 1) then
                allocate(tipo_c(0:jx+1, 0:jy+1, 0:jz+1))
                tipo_c = int(tipo(0:jx+1, 0:jy+1, 0:jz+1), c_int)
                call gpu_build(islor, bodyforce, fs, tipo_c)
                deallocate(tipo_c)
            else
                call gpu_build(islor, bodyforce, fs)
            end if
        end if
        if (fs == 1) then
            if (iterat == 1) then  ! the first time step imposes PrS0 = 0 (multigrid.f03:1196-1205)
                stat = ples_mg_set_surface_pressure(mg_handle, c_null_ptr)
                if (stat /= PLES_MG_OK) error stop 'multi: ples_mg_set_surface_pressure failed'
            else
                call surface_on(next_prs(1:jx, 1:jz), jx, jz)
            end if
        end if
        ! fi (0:n1+1, 0:n2+1, kparasta-deepl:kparaend+deepr) on one rank:
        ! the solver's extent has one ghost plane, so deeper halos go through
        ! a copy (an array section passed to solve_on is copied in and out)
        if (deepl == 1 .and. deepr == 1) then
            call solve_on(fi, rhs, cs1, cs2, cs3, cs4, cs5, cs6, real(eps, c_double), ficycle, st, stat)
        else
            allocate(fi_c(0:jx+1, 0:jy+1, 0:jz+1))
            fi_c = fi(0:jx+1, 0:jy+1, 0:jz+1)
            call solve_on(fi_c, rhs, cs1, cs2, cs3, cs4, cs5, cs6, real(eps, c_double), ficycle, st, stat)
            fi(0:jx+1, 0:jy+1, 0:jz+1) = fi_c
            deallocate(fi_c)
        end if
        if (stat /= PLES_MG_OK .and. stat /= PLES_MG_NOT_CONVERGED) error stop 'multi: ples_mg_solve failed'
        if (myid == 0) write(*, *) 'multi (GPU):', st%outer_iterations, st%max_residual
    end subroutine multi

end module multigrid_module
