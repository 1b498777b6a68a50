!***********************************************************************
! ples_mg_iface -- iso_c_binding interface of the GB300 pressure multigrid
! (include/ples_mg.h) and the two calls that replace PLES's CPU solver:
!
!   ples_mg_setup : after metrica (fsrc/stratiParticle.f03:767), in place of
!                   mul_met / wall (:768-769); builds the coefficient
!                   hierarchy on the GPU from the node coordinates x,y,z
!                   (myarrays_metri3, single-domain extent -8:n1+8, ...).
!   multi_gpu     : drop-in body for multi (fsrc/multigrid.f03:42-653) at
!                   the call site fsrc/stratiParticle.f03:2881-2887: same
!                   eps (absolute max-norm stop) and ficycle meaning; fi
!                   (myarrays_velo3, 0:n1+1,0:n2+1,0:n3+1 on one rank) is
!                   overwritten with the solution including its ghost layer.
!
! Not compiled in this repository's build (no Fortran compiler is assumed);
! a PLES build adds it to its object list and links libples_mg.so.
!***********************************************************************
module ples_mg_iface
    use iso_c_binding
    implicit none

    integer(c_int), parameter :: PLES_MG_ABI_VERSION = 5
    integer(c_int), parameter :: PLES_MG_OK = 0, PLES_MG_NOT_CONVERGED = 1
    integer(c_int), parameter :: PLES_MG_SMOOTHER_LINE = 0, PLES_MG_SMOOTHER_POINT = 3
    integer(c_int), parameter :: PLES_MG_PREC_FP64 = 0, PLES_MG_PREC_MIXED = 1
    integer(c_int), parameter :: PLES_MG_COORDS_NODES = 0, PLES_MG_COORDS_GHOSTED8 = 1

    type, bind(C) :: ples_mg_desc
        integer(c_int) :: jx, jy, jz
        integer(c_int) :: ip, jp, kp
        integer(c_int) :: nlevmax
        real(c_double) :: omega
        integer(c_int) :: precision
        integer(c_int) :: coords_layout
        type(c_ptr)    :: x, y, z
        real(c_double) :: dt
        integer(c_int) :: device
        integer(c_int) :: nu_pre, nu_post
        integer(c_int) :: nu_coarse
        integer(c_int) :: inner_cycles
        integer(c_int) :: smoother
        integer(c_int) :: coarsening
        type(c_ptr)    :: solid
        type(c_ptr)    :: tipo
        integer(c_int) :: freesurface
    end type ples_mg_desc

    type, bind(C) :: ples_mg_stats
        integer(c_int) :: outer_iterations
        integer(c_int) :: vcycles
        real(c_double) :: rel_residual
        real(c_double) :: max_residual
        real(c_double) :: rhs_norm
        real(c_double) :: rhs_mean_removed
        real(c_double) :: seconds
        integer(c_int) :: status
    end type ples_mg_stats

    interface
        integer(c_int) function ples_mg_create(desc, handle) bind(C, name="ples_mg_create")
            import :: ples_mg_desc, c_int, c_ptr
            type(ples_mg_desc), intent(in) :: desc
            type(c_ptr), intent(out) :: handle
        end function ples_mg_create

        integer(c_int) function ples_mg_solve(handle, fi, rhs, cs, rel_tol, abs_tol_max, &
                                              max_cycles, stats) bind(C, name="ples_mg_solve")
            import :: c_int, c_ptr, c_double, ples_mg_stats
            type(c_ptr), value :: handle, fi, rhs, cs
            real(c_double), value :: rel_tol, abs_tol_max
            integer(c_int), value :: max_cycles
            type(ples_mg_stats), intent(out) :: stats
        end function ples_mg_solve

        subroutine ples_mg_destroy(handle) bind(C, name="ples_mg_destroy")
            import :: c_ptr
            type(c_ptr), value :: handle
        end subroutine ples_mg_destroy

        function ples_mg_strerror(code) bind(C, name="ples_mg_strerror")
            import :: c_int, c_ptr
            integer(c_int), value :: code
            type(c_ptr) :: ples_mg_strerror
        end function ples_mg_strerror

        integer(c_int) function ples_mg_step(handle, u, v, w, uc, vc, wc, fi, rel_tol, max_cycles, &
                                             stats) bind(C, name="ples_mg_step")
            import :: c_int, c_ptr, c_double, ples_mg_stats
            type(c_ptr), value :: handle, u, v, w, uc, vc, wc, fi
            real(c_double), value :: rel_tol
            integer(c_int), value :: max_cycles
            type(ples_mg_stats), intent(out) :: stats
        end function ples_mg_step

        integer(c_int) function ples_mg_potenziale_ibm(handle, fi) bind(C, name="ples_mg_potenziale_ibm")
            import :: c_int, c_ptr
            type(c_ptr), value :: handle, fi
        end function ples_mg_potenziale_ibm

        integer(c_int) function ples_mg_set_surface_pressure(handle, next_prs) &
                bind(C, name="ples_mg_set_surface_pressure")
            import :: c_int, c_ptr
            type(c_ptr), value :: handle, next_prs
        end function ples_mg_set_surface_pressure

        integer(c_int) function ples_mg_abi_layout(abi_version, desc_size, stats_size, desc_offsets, &
                                                   stats_offsets) bind(C, name="ples_mg_abi_layout")
            import :: c_int, c_long_long
            integer(c_int), intent(out) :: abi_version
            integer(c_long_long), intent(out) :: desc_size, stats_size
            integer(c_long_long), intent(out) :: desc_offsets(24), stats_offsets(8)
        end function ples_mg_abi_layout

        integer(c_int) function ples_mg_read_grid(path, lengths, dims, x, y, z) bind(C, name="ples_mg_read_grid")
            import :: c_int, c_ptr, c_char, c_double
            character(kind=c_char), dimension(*), intent(in) :: path
            real(c_double), intent(out) :: lengths(3)
            integer(c_int), intent(out) :: dims(3)
            type(c_ptr), value :: x, y, z
        end function ples_mg_read_grid
    end interface

    type(c_ptr), save :: mg_handle = c_null_ptr

contains

    !-------------------------------------------------------------------
    ! .true. when the bind(C) types above have the layout the library was
    ! compiled with (size of each type and the byte offset of every field)
    logical function ples_mg_layout_ok()
        type(ples_mg_desc), target :: d
        type(ples_mg_stats), target :: s
        integer(c_int) :: ver
        integer(c_long_long) :: dsize, ssize, doff(24), soff(8), mine_d(24), mine_s(8), base
        integer :: stat
        stat = ples_mg_abi_layout(ver, dsize, ssize, doff, soff)
        base = transfer(c_loc(d), base)
        mine_d = [transfer(c_loc(d%jx), base), transfer(c_loc(d%jy), base), transfer(c_loc(d%jz), base), &
                  transfer(c_loc(d%ip), base), transfer(c_loc(d%jp), base), transfer(c_loc(d%kp), base), &
                  transfer(c_loc(d%nlevmax), base), transfer(c_loc(d%omega), base), &
                  transfer(c_loc(d%precision), base), transfer(c_loc(d%coords_layout), base), &
                  transfer(c_loc(d%x), base), transfer(c_loc(d%y), base), transfer(c_loc(d%z), base), &
                  transfer(c_loc(d%dt), base), transfer(c_loc(d%device), base), &
                  transfer(c_loc(d%nu_pre), base), transfer(c_loc(d%nu_post), base), &
                  transfer(c_loc(d%nu_coarse), base), transfer(c_loc(d%inner_cycles), base), &
                  transfer(c_loc(d%smoother), base), transfer(c_loc(d%coarsening), base), &
                  transfer(c_loc(d%solid), base), transfer(c_loc(d%tipo), base), &
                  transfer(c_loc(d%freesurface), base)] - base
        base = transfer(c_loc(s), base)
        mine_s = [transfer(c_loc(s%outer_iterations), base), transfer(c_loc(s%vcycles), base), &
                  transfer(c_loc(s%rel_residual), base), transfer(c_loc(s%max_residual), base), &
                  transfer(c_loc(s%rhs_norm), base), transfer(c_loc(s%rhs_mean_removed), base), &
                  transfer(c_loc(s%seconds), base), transfer(c_loc(s%status), base)] - base
        ples_mg_layout_ok = stat == PLES_MG_OK .and. ver == PLES_MG_ABI_VERSION .and. &
                            dsize == c_sizeof(d) .and. ssize == c_sizeof(s) .and. &
                            all(doff == mine_d) .and. all(soff == mine_s)
    end function ples_mg_layout_ok

    !-------------------------------------------------------------------
    ! after metrica: x, y, z are the ghosted node arrays of myarrays_metri3
    ! (one rank holds the whole domain); only planes -8..jz+8 are read.
    subroutine ples_mg_setup(x, y, z, jx, jy, jz, ip, jp, kp, dt, precision)
        real(c_double), target, intent(in) :: x(-8:, -8:, -8:), y(-8:, -8:, -8:), z(-8:, -8:, -8:)
        integer, intent(in) :: jx, jy, jz, ip, jp, kp, precision
        real(c_double), intent(in) :: dt
        type(ples_mg_desc) :: d
        integer(c_int) :: stat

        if (size(x, 1) /= jx + 17 .or. size(x, 2) /= jy + 17) error stop 'ples_mg_setup: x extents'
        d = ples_mg_desc(jx=jx, jy=jy, jz=jz, ip=ip, jp=jp, kp=kp, nlevmax=0, omega=0.d0, &
                         precision=precision, coords_layout=PLES_MG_COORDS_GHOSTED8, &
                         x=c_loc(x(-8, -8, -8)), y=c_loc(y(-8, -8, -8)), z=c_loc(z(-8, -8, -8)), &
                         dt=dt, device=0, nu_pre=0, nu_post=0, nu_coarse=0, inner_cycles=0, &
                         smoother=0, coarsening=0, solid=c_null_ptr, tipo=c_null_ptr, freesurface=0)
        if (c_associated(mg_handle)) call ples_mg_destroy(mg_handle)
        stat = ples_mg_create(d, mg_handle)
        if (stat /= PLES_MG_OK) error stop 'ples_mg_create failed'
    end subroutine ples_mg_setup

    !-------------------------------------------------------------------
    ! replacement of multi: eps and ficycle as in Agenerale.in; returns the
    ! number of cycles in ktime like the reference's loop counter
    subroutine multi_gpu(eps, ficycle, fi, rhs, cs1, cs2, cs3, cs4, cs5, cs6, ktime)
        real(c_double), intent(in) :: eps
        integer, intent(in) :: ficycle
        real(c_double), target, intent(inout) :: fi(0:, 0:, 0:)
        real(c_double), target, intent(in) :: rhs(:, :, :)
        real(c_double), target, intent(in) :: cs1(:, :), cs2(:, :), cs3(:, :), cs4(:, :), cs5(:, :), cs6(:, :)
        integer, intent(out) :: ktime
        type(c_ptr), target :: cs(6)
        type(ples_mg_stats) :: st
        integer(c_int) :: stat

        cs = [c_loc(cs1), c_loc(cs2), c_loc(cs3), c_loc(cs4), c_loc(cs5), c_loc(cs6)]
        stat = ples_mg_solve(mg_handle, c_loc(fi), c_loc(rhs), c_loc(cs), 0.d0, eps, &
                             int(ficycle, c_int), st)
        if (stat /= PLES_MG_OK .and. stat /= PLES_MG_NOT_CONVERGED) error stop 'ples_mg_solve failed'
        ktime = st%outer_iterations
    end subroutine multi_gpu

    !-------------------------------------------------------------------
    ! the whole pressure step of a time step (contra, diver, multi, gradie,
    ! vel_up; fsrc/stratiParticle.f03:2845-2937) on the GPU: u, v, w are the
    ! intermediate Cartesian velocities (0:n1+1,0:n2+1,0:n3+1), uc, vc, wc the
    ! previous contravariant ones (iniz.f03:103-105 extents on one rank); all
    ! are updated in place, fi takes the pressure; stop at ||r||/||b|| <= rel_tol
    subroutine pressure_step_gpu(u, v, w, uc, vc, wc, fi, rel_tol, ficycle, ktime)
        real(c_double), target, intent(inout) :: u(0:, 0:, 0:), v(0:, 0:, 0:), w(0:, 0:, 0:)
        real(c_double), target, intent(inout) :: uc(0:, :, :), vc(:, 0:, :), wc(:, :, 0:)
        real(c_double), target, intent(inout) :: fi(0:, 0:, 0:)
        real(c_double), intent(in) :: rel_tol
        integer, intent(in) :: ficycle
        integer, intent(out) :: ktime
        type(ples_mg_stats) :: st
        integer(c_int) :: stat

        stat = ples_mg_step(mg_handle, c_loc(u), c_loc(v), c_loc(w), c_loc(uc), c_loc(vc), c_loc(wc), &
                            c_loc(fi), rel_tol, int(ficycle, c_int), st)
        if (stat /= PLES_MG_OK .and. stat /= PLES_MG_NOT_CONVERGED) error stop 'ples_mg_step failed'
        ktime = st%outer_iterations
    end subroutine pressure_step_gpu

end module ples_mg_iface
