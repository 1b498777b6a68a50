/*
 * ples_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU FP64 restatement of the PLES pressure-Poisson multigrid (the Fortran
 * module `multigrid_module` in fsrc/multigrid.f03 and its helpers).  It is the
 * checker for the CUDA library in ples_gb300/ and the timed CPU baseline; the
 * product never links, loads or calls it.
 *
 * Parity status: the reference ships no tests, golden vectors or a buildable
 * CPU path here (Fortran + MPI, no compiler in this image), so this oracle is
 * pinned by known-answer checks built on the reference's own sample deck
 * (uniform 32^3 grid: exact metric values, spectral exact solution of the
 * discrete problem) rather than by reference outputs.
 *
 * Arrays cross this interface as column-major (Fortran order) FP64 buffers
 * with the reference's lower bounds; the extents are given per function.
 */
#ifndef PLES_ORACLE_H
#define PLES_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_problem orc_problem;

/* Build the grid, ghost nodes (cellep.f03), level sizes (indy.f03),
 * fine metric (metrica.f03), coarse metric (multigrid.f03 mul_met),
 * masks and tridiagonal coefficients (sett.f03) for `nproc` emulated
 * k-slab ranks.
 *   xn,yn,zn : node coordinates (0:jx,0:jy,0:jz), column-major.
 *   ip,jp,kp : 0 periodic, 1 wall (reference convention, Aboundary.in)
 *   nlevmax  : nlevmultimax (<=4); the level count is min(indy, nlevmax).
 * Returns NULL on a bad argument (message in orc_last_error()). */
orc_problem *orc_create(int jx, int jy, int jz, int ip, int jp, int kp,
                        int nlevmax, int nproc, double omega, int islor,
                        double dt, const double *xn, const double *yn,
                        const double *zn);
void orc_destroy(orc_problem *p);
const char *orc_last_error(void);

/* multi's freesurface argument (multigrid.f03:48): 1 puts the free-surface
 * relation of mul_boun_sndrcv (multigrid.f03:1188-1222) on the top ghost row
 * of the point SOR's ghost fill (the line SOR keeps the wall relation, as the
 * reference's sets freesurface = 0, multigrid.f03:2019) and of
 * orc_ghost_fill.  next_prs (1:jx,1:jz): the surface pressure PrS0 of level
 * 1 (myarrays_velo3 next_prs, set by contourp.f03:160), or NULL for the
 * first time step, where the reference uses PrS0 = 0. */
int orc_set_free_surface(orc_problem *p, int freesurface, const double *next_prs);

int orc_nlevel(const orc_problem *p);
/* jxc(n), jyc(n), jzc(n) for n=1..nlevel */
void orc_level_dims(const orc_problem *p, int n, int *nx, int *ny, int *nz);

/* Copy one metric array of level n into out.
 * which: 0..8 = g11,g12,g13,g21,g22,g23,g31,g32,g33; 9 = giac (level 1).
 * Extents: g1* (0:nx,1:ny,1:nz), g2* (1:nx,0:ny,1:nz), g3* (1:nx,1:ny,0:nz),
 * giac (1:nx,1:ny,1:nz). */
int orc_get_metric(const orc_problem *p, int n, int which, double *out);
/* Node coordinates with ghosts (-8:jx+8,-8:jy+8,-8:jz+8); c=0,1,2 -> x,y,z */
int orc_get_coords(const orc_problem *p, int c, double *out);

/* Single-level operators on one domain (nproc ignored, one rank).
 * pr  : (0:nx+1,0:ny+1,0:nz+1), rh/out : (1:nx,1:ny,1:nz)
 * cs  : cs1..cs6 of the fine level, cs1/2 (1:jy,1:jz), cs3/4 (1:jx,1:jz),
 *       cs5/6 (1:jx,1:jy); NULL means zero. */
int orc_resid(orc_problem *p, int n, const double *pr, const double *rh,
              double *out);
int orc_ghost_fill(orc_problem *p, int n, double *pr,
                   const double *const cs[6]);
int orc_restrict(orc_problem *p, int n, const double *rh, double *out);
int orc_prolong(orc_problem *p, int n, double *prf, const double *prc);

/* The V-cycle driver `multi` (multigrid.f03:42-653) over nproc ranks.
 *   fi  : (0:jx+1,0:jy+1,0:jz+1) in/out, initial guess and solution.
 *   rhs : (1:jx,1:jy,1:jz).
 *   Stop when ktime >= ficycle, or (stop_mode 0) max|r| < eps as the
 *   reference does, or (stop_mode 1) ||r||_2/||rhs||_2 <= eps.
 * Outputs: cycles run, final max|r| and ||r||_2/||rhs||_2.
 * Returns 0, or -1 on a bad argument. */
int orc_multi(orc_problem *p, double *fi, const double *rhs,
              const double *const cs[6], double eps, int ficycle,
              int stop_mode, int *cycles, double *resmax,
              double *relres);

/* FP64 residual of the fine-level system after solving the fine wall-ghost
 * relations to a fixed point (used by tests to measure the true residual):
 * ghost passes until the ghost update is below tol or maxpass passes. */
int orc_true_residual(orc_problem *p, double *fi, const double *rhs,
                      const double *const cs[6], double *out, int maxpass);

#ifdef __cplusplus
}
#endif
#endif
