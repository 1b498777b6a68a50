/*
 * ples_mg.h -- C ABI of the GB300 pressure-Poisson multigrid.
 *
 * Drop-in for the pressure solve of PLES: the Fortran subroutine `multi`
 * (fsrc/multigrid.f03:42-48, called at fsrc/stratiParticle.f03:2881-2887)
 * and its set-up chain metrica -> mul_met -> wall (fsrc/stratiParticle.f03:
 * 767-769).  Arrays cross the boundary as plain pointers to caller-owned,
 * column-major FP64 buffers with the reference's lower bounds; no C++ or
 * CUDA types appear in the signatures, so the functions bind directly from
 * Fortran through iso_c_binding.
 *
 * Threading: one handle per host thread.  Every entry point returns a status
 * code (PLES_MG_OK == 0); the handle also keeps the last error message.
 */
#ifndef PLES_MG_H
#define PLES_MG_H

#ifdef __cplusplus
extern "C" {
#endif

#define PLES_MG_ABI_VERSION 5

/* status codes */
enum {
    PLES_MG_OK = 0,
    PLES_MG_NOT_CONVERGED = 1, /* max_cycles reached above tolerance        */
    PLES_MG_BAD_ARG = 2,       /* invalid descriptor, size or pointer       */
    PLES_MG_OOM = 3,           /* device allocation or HBM budget exceeded  */
    PLES_MG_DEVICE_TIMEOUT = 4,/* a bounded device wait gave up             */
    PLES_MG_CUDA_ERROR = 5,    /* CUDA runtime error                        */
    PLES_MG_DIVERGED = 6,      /* NaN/Inf or residual growth                */
    PLES_MG_NO_DEVICE = 7      /* no usable CUDA device                     */
};

/* inner-solve precision */
enum {
    PLES_MG_PREC_FP64 = 0,  /* plain: every kernel in FP64                          */
    PLES_MG_PREC_MIXED = 1, /* FP32 V-cycle inside an FP64 defect-correction loop   */
    PLES_MG_PREC_OUTER = 2  /* ples_mg_apply_residual only: the solver's own outer
                               residual of level 1 (double-float products on a
                               mixed handle, FP64 on an FP64 one)               */
};

/* layout of the node coordinates in the descriptor */
enum {
    PLES_MG_COORDS_NODES = 0,    /* x,y,z(0:jx, 0:jy, 0:jz)                         */
    PLES_MG_COORDS_GHOSTED8 = 1  /* x,y,z(-8:jx+8, -8:jy+8, -8:jz+8), the single-   */
                                 /* domain extent of myarrays_metri3 (iniz_metrica) */
};

/* ghost-layer fill rules, fsrc/multigrid.f03:1013-1936 */
typedef struct {
    int jx, jy, jz;        /* fine cells (scala3 jx, jy, jz)                        */
    int ip, jp, kp;        /* 0 periodic, 1 wall (module period, Aboundary.in:6-8);
                              jp must be 1 (multigrid.f03:1744-1746)                */
    int nlevmax;           /* maximum multigrid levels; 0 = automatic: coarsen until a level has
                              at most 3072 unknowns (wall rows included), solved by a dense inverse */
    double omega;          /* relaxation factor of the smoother (0 = default: 1.4 for
                              smoothers 0 and 2, 0.8 for 1, 1.0 for 3)          */
    int precision;         /* PLES_MG_PREC_*                                        */
    int coords_layout;     /* PLES_MG_COORDS_*                                      */
    const double *x, *y, *z; /* host node coordinates, column-major                 */
    double dt;             /* time step dividing the cs1..cs6 wall fluxes           */
    int device;            /* CUDA device ordinal                                   */
    int nu_pre, nu_post;   /* smoothing sweeps per level before / after the coarse
                              correction (0 = default: 1 / 2 for smoothers 0 and 2
                              with an even inner_cycles, else 2 / 2); the sweeps of
                              one outer iteration, (nu_pre + nu_post) x
                              inner_cycles, must be even.  When omega, nu_pre,
                              nu_post and inner_cycles are all 0 for smoother 0
                              or 2, creation solves a pseudo-random right-hand
                              side for two outer iterations and, if that does
                              not converge, takes 2 / 2 sweeps, 5 V-cycles and
                              omega 1.3 instead (stable where 1 / 2 and 1.4 are
                              not, about 6% slower on the benchmark grid)      */
    int nu_coarse;         /* sweeps on the coarsest level (0 = default)            */
    int inner_cycles;      /* V-cycles per outer FP64 iteration (0 = default: 6 for
                              smoothers 0 and 2, else 5)                        */
    int smoother;          /* 0 = zebra eta-line SOR (Gauss-Seidel in x and z as the
                              reference's line SOR, islor = 1); 1 = eta-line Jacobi;
                              2 = zebra with its rows staged by TMA (FP32);
                              3 = multicolour point SOR, the reference's
                              default islor = 0 (solut_sndrcv_sor,
                              multigrid.f03:656-1010; omega default 1.0;
                              periodic directions need even cell counts on
                              every smoothed level) */
    int coarsening;        /* 0 = full, the reference's hierarchy (mul_met);
                              1 = semi-coarsening where x/z spacings differ     */
    const unsigned char *solid; /* immersed-boundary mask (1:jx,1:jy,1:jz), 1 =
                              solid cell, or NULL.  No counterpart in the
                              reference's multigrid: solid cells are removed
                              from the system (Neumann at their faces); the
                              solution is 0 there and rhs, compatibility and
                              mean refer to the fluid cells. */
    const int *tipo;       /* PLES's immersed-boundary cell types (0:jx+1,0:jy+1,
                              0:jz+1) (0 solid, 1 IB, >= 2 fluid), or NULL.  As
                              in multi with bodyforce = 1 (multigrid.f03:615-
                              631), the max-norm stop test (eps / max_residual)
                              then runs over the fluid cells only; the operator
                              is unchanged.  Also the input of
                              ples_mg_potenziale_ibm. */
    int freesurface;       /* multi's freesurface argument (multigrid.f03:48): 1 =
                              the top wall row takes the free-surface relation
                              of mul_boun_sndrcv (multigrid.f03:1188-1222) with
                              the surface pressure of
                              ples_mg_set_surface_pressure; the pressure level
                              is then fixed (no compatibility shift, no mean
                              removal).  Needs smoother 3: the reference's line
                              SOR keeps the wall relation (multigrid.f03:2019).
                              Not for batches. */
} ples_mg_desc;

typedef struct {
    int outer_iterations;   /* FP64 residual evaluations after the first           */
    int vcycles;            /* inner V-cycles run                                   */
    double rel_residual;    /* ||r||_2 / ||b||_2 of the returned solution           */
    double max_residual;    /* max |r| of the returned solution                     */
    double rhs_norm;        /* ||b||_2 after the compatibility projection          */
    double rhs_mean_removed;/* mean subtracted from b (compatibility)               */
    double seconds;         /* wall time of the call                                */
    int status;
} ples_mg_stats;

typedef struct ples_mg_handle ples_mg_handle;

/* Layout of the two structures above as this library was compiled: its
 * PLES_MG_ABI_VERSION, sizeof(ples_mg_desc), sizeof(ples_mg_stats) and the
 * byte offset of every field in declaration order (desc_offsets holds
 * PLES_MG_DESC_FIELDS values, stats_offsets PLES_MG_STATS_FIELDS; any
 * pointer may be NULL).  A binding compiled against its own copy of this
 * header (C, Fortran bind(C) types, a ctypes mirror) compares them with
 * its own to detect a stale copy.  No counterpart in the reference, whose
 * multi exchanges module variables, not structures. */
#define PLES_MG_DESC_FIELDS 24
#define PLES_MG_STATS_FIELDS 8
int ples_mg_abi_layout(int *abi_version, long long *desc_size, long long *stats_size,
                       long long *desc_offsets, long long *stats_offsets);

/* Build the coefficient hierarchy on the device and keep it resident.
 * Replaces metrica (fsrc/metrica.f03:2-501), cellep (fsrc/cellep.f03),
 * indy (fsrc/indy.f03), mul_met (fsrc/multigrid.f03:2293-3052) and
 * wall/sett (fsrc/multigrid.f03:3151-3264, fsrc/sett.f03). */
int ples_mg_create(const ples_mg_desc *desc, ples_mg_handle **out);

/* Replaces multi (fsrc/multigrid.f03:42-653).
 *   fi  : in/out (0:jx+1, 0:jy+1, 0:jz+1); initial guess, returned solution
 *         with its ghost layer filled (periodic copies and wall relations).
 *   rhs : (1:jx, 1:jy, 1:jz) (fsrc/diver.f03); made compatible by removing
 *         its mean net of the wall fluxes.
 *   cs  : cs1..cs6 wall fluxes (myarrays_velo3): cs1,cs2 (1:jy,1:jz),
 *         cs3,cs4 (1:jx,1:jz), cs5,cs6 (1:jx,1:jy); NULL = all zero.
 *   Stops when ||r||_2/||b||_2 <= rel_tol (if rel_tol > 0) or
 *   max|r| < abs_tol_max (if abs_tol_max > 0, the reference's eps test,
 *   multigrid.f03:598-631), or after max_cycles outer iterations
 *   (the reference's ficycle).  The solution is returned with zero mean. */
int ples_mg_solve(ples_mg_handle *h, double *fi, const double *rhs,
                  const double *const cs[6], double rel_tol,
                  double abs_tol_max, int max_cycles, ples_mg_stats *stats);

/* Same, on device-resident buffers with the same extents (column-major,
 * FP64): no host copies.  stream is a cudaStream_t or NULL. */
int ples_mg_solve_device(ples_mg_handle *h, double *d_fi, const double *d_rhs,
                         const double *const d_cs[6], double rel_tol,
                         double abs_tol_max, int max_cycles, void *stream,
                         ples_mg_stats *stats);

void ples_mg_destroy(ples_mg_handle *h);
const char *ples_mg_strerror(int code);
const char *ples_mg_last_error(const ples_mg_handle *h);

/* ---- per-level operators (the hot-path routines one by one) --------- */
int ples_mg_levels(const ples_mg_handle *h, int *nlevel);
int ples_mg_level_dims(const ples_mg_handle *h, int level, int *nx, int *ny,
                       int *nz);
/* FP64 face metric of a level as built on the device, reference extents:
 * which 0..8 = g11..g33 (before any scaling): g1* (0:nx,1:ny,1:nz),
 * g2* (1:nx,0:ny,1:nz), g3* (1:nx,1:ny,0:nz).  Replaces the arrays of
 * metrica (level 1) and mul_met (levels >= 2). */
int ples_mg_get_metric(ples_mg_handle *h, int level, int which, double *out);
/* rh1 = L_n(pr) - rh on the device (resid_sndrcv.f03:2-156);
 * pr (0:nx+1,0:ny+1,0:nz+1), rh/out (1:nx,1:ny,1:nz).  precision selects
 * the FP64 or the FP32 kernel, or (level 1) PLES_MG_PREC_OUTER the kernel
 * the solve's stop test and defect correction use. */
int ples_mg_apply_residual(ples_mg_handle *h, int level, const double *pr,
                           const double *rh, double *out, int precision);
/* Ghost layer of pr at level `level` driven to the fixed point of the
 * reference's fill (mul_boun_sndrcv, multigrid.f03:1013-1936): `passes`
 * Jacobi passes; cs (level 1 only) as in ples_mg_solve. */
int ples_mg_apply_ghost_fill(ples_mg_handle *h, int level, double *pr,
                             const double *const cs[6], int passes);
/* out = restriction of rh (restrict_sndrcv.f03:2-56), level -> level+1 */
int ples_mg_apply_restrict(ples_mg_handle *h, int level, const double *rh,
                           double *out);
/* prf += prolongation of prc (prolong.f03:2-261), level+1 -> level */
int ples_mg_apply_prolong(ples_mg_handle *h, int level, double *prf,
                          const double *prc);

/* ---- instrumentation (the reference's only instrument is the wall-clock
 * mlt timer around multi, fsrc/stratiParticle.f03:2874,2921-2927) ------- */
/* kernels launched on the device by this handle so far, and its resident
 * device bytes */
int ples_mg_counters(ples_mg_handle *h, long long *launches, long long *device_bytes);
/* Polls a bounded device wait makes before it gives up (the mbarrier waits
 * of the TMA-staged smoother, smoother 2, the only waits on the device; they
 * also give up after 2 s): polls < 0 restores the default (2^26).  A wait
 * that gives up makes the solve return PLES_MG_DEVICE_TIMEOUT, after its CTA
 * has waited (with the default limits) for its copies still in flight; the
 * handle stays usable.  For tests of that path: 0 makes every wait give up
 * at once.  No counterpart in the reference. */
int ples_mg_set_wait_limit(ples_mg_handle *h, long long polls);

/* time one kernel kind at one level with CUDA events on the solve stream:
 * kind 0 eta-line smoother, 1 residual+restriction, 2 prolongation,
 * 3 FP64 outer residual; kind -1 switches timing off.  Resets the totals. */
int ples_mg_kernel_timing(ples_mg_handle *h, int kind, int level);
int ples_mg_kernel_time(ples_mg_handle *h, double *total_ms, long long *launches);

/* ---- the projection step around the solve -------------------------------
 * One call for the pressure-correction step of a PLES time step
 * (fsrc/stratiParticle.f03:2845-2937, potenziale = 0, no free surface):
 * diver (rhs = div(uc,vc,wc)/dt, fsrc/diver.f03:25-27), multi (the solve,
 * warm-started from fi), gradie (fsrc/gradie.f03:30-116) and vel_up
 * (fsrc/vel_up.f03:40-52, 188-285): uc -= dt cgra1 on i = 0..jx, vc -= dt
 * cgra2 on j = 1..jy-1 (the wall faces keep their flux), wc -= dt cgra3 on
 * k = 0..jz, and u,v,w += -dt/2 J^-1 grad(fi) at the cells with their
 * periodic images.  Host arrays: uc (0:jx,1:jy,1:jz), vc (1:jx,0:jy,1:jz),
 * wc (1:jx,1:jy,0:jz), u,v,w and fi (0:jx+1,0:jy+1,0:jz+1); u,v,w may all
 * be NULL (contravariant part only).  dt is the descriptor's.  The face
 * normals and the cell Jacobian are built on the device at the first call
 * with u,v,w (nine face arrays and one cell array, FP64). */
int ples_mg_project(ples_mg_handle *h, double *uc, double *vc, double *wc, double *u,
                    double *v, double *w, double *fi, double rel_tol, int max_cycles,
                    ples_mg_stats *stats);

/* The whole pressure step: contra (fsrc/contra.f03:31-219, jp = 1,
 * potenziale = 0; with x / z walls their faces also take the wall velocity
 * and give cs1/cs2, cs5/cs6, as on several ranks) and then the projection
 * above (wall faces keep their flux).  On entry u,v,w are
 * the intermediate Cartesian velocities with their ghost cells (the wall
 * velocity in j = 0 and jy+1, periodic images in x and z) and uc,vc,wc the
 * previous contravariant ones, of which only the wall faces vc(:,0,:),
 * vc(:,jy,:) are read: the faces get the face-normal projection of the
 * average of their two cells, the wall faces that of the wall velocity,
 * and cs3/cs4 = new minus old wall flux drive the solve's wall condition.
 * On return all six hold the projected velocities and fi the pressure.
 * Replaces contra + diver + multi + gradie + vel_up
 * (fsrc/stratiParticle.f03:2845-2937). */
int ples_mg_step(ples_mg_handle *h, double *u, double *v, double *w, double *uc, double *vc,
                 double *wc, double *fi, double rel_tol, int max_cycles, ples_mg_stats *stats);

/* potenziale_ibm (fsrc/potenziale_ibm.f03:37-88): every solid cell (tipo 0)
 * of fi takes the mean of its face neighbours that are IB cells (tipo 1), in
 * the order i+1, i-1, j+1, j-1, k+1, k-1, and keeps its value if it has
 * none.  fi (0:jx+1,0:jy+1,0:jz+1) host, in/out; ghost cells are read, not
 * written.  Needs the descriptor's tipo (BAD_ARG without). */
int ples_mg_potenziale_ibm(ples_mg_handle *h, double *fi);

/* ---- grid file ------------------------------------------------------------
 * Reads PLES's grid file gri3dp_in.dat as fsrc/stratiParticle.f03:364-412
 * does (list-directed: the lengths alx aly alz, the cell counts jx jy jz,
 * then one record per coordinate, x y z of every node, i fastest).  With
 * x, y, z all NULL only lengths (may be NULL) and dims are filled; then call
 * again with three caller arrays of (jx+1)(jy+1)(jz+1) doubles, which take
 * the node coordinates in the (0:jx,0:jy,0:jz) layout of ples_mg_desc.
 * Needs no device.  BAD_ARG for a missing or malformed file. */
int ples_mg_read_grid(const char *path, double lengths[3], int dims[3], double *x, double *y,
                      double *z);

/* ---- autotuner ----------------------------------------------------------
 * No counterpart in the reference (its kss, nlevel and omega are fixed
 * inputs).  Times candidate settings on this handle's grid and keeps the
 * fastest: the form of the eta-line smoother per level (128, 256 or 512
 * threads on 32-line tiles, or 1024 for 512 threads on 64-line tiles, by
 * kernel time) and then the sweeps per level before and after the coarse
 * correction (1..3 each, seven pairs), the V-cycles per outer iteration (2
 * to 8) and, for the zebra smoothers, omega (the handle's, 1.3, 1.4), by
 * the time of a whole solve to ||r||/||b|| <= 1e-10 from zero.  rhs (host, (1:jx,1:jy,
 * 1:jz)) or NULL for a pseudo-random compatible one.  Batches created
 * afterwards use the tuned settings of their members. */
typedef struct {
    int nu;               /* sweeps per level before the coarse correction (nu_pre) */
    int inner_cycles;     /* V-cycles per FP64 outer iteration */
    int line_threads[12]; /* smoother form per level, as ples_mg_set_line_threads (0 past the last level) */
    double solve_ms;      /* one solve with the chosen setting */
    int candidates;       /* settings timed */
    int nu_post;          /* sweeps per level after the coarse correction */
    double omega;         /* relaxation factor */
} ples_mg_tuning;
int ples_mg_autotune(ples_mg_handle *h, const double *rhs, ples_mg_tuning *out);
/* Set the form of the eta-line smoother at one level (1-based), as the
 * autotuner does: 128, 256 or 512 threads per CTA on 32-line tiles, 1024
 * for the 64-line-tile form (512 threads; mixed precision, zebra smoother,
 * x and z periodic, nx of the level even, nz >= 2), 2048 for the same tiles
 * with rows built two lines per thread (256 threads), or 4096 for the
 * 64-line tiles with both k parities of a sweep in one launch (an even-k
 * tile starts once the odd planes either side of it are stored; its wait is
 * bounded by ples_mg_set_wait_limit, and one that runs out ends the solve
 * with PLES_MG_DEVICE_TIMEOUT).  No counterpart in the
 * reference (its sweeps are scalar loops, multigrid.f03:1939-2290).  BAD_ARG
 * for another value, a form that does not apply at that level or whose
 * shared memory does not fit. */
int ples_mg_set_line_threads(ples_mg_handle *h, int level, int threads);
/* The surface pressure PrS0 of a free-surface handle: next_prs (1:jx,1:jz)
 * (myarrays_velo3, set by fsrc/contourp.f03:160), host, used by the
 * following solves on level 1 (multigrid.f03:1207-1213); NULL = zero, as the
 * reference's first time step (iterat = 1).  BAD_ARG without
 * desc.freesurface. */
int ples_mg_set_surface_pressure(ples_mg_handle *h, const double *next_prs);
/* The form of the eta-line smoother at one level (1-based) as
 * ples_mg_set_line_threads takes it: the default or the autotuner's
 * choice.  No counterpart in the reference. */
int ples_mg_get_line_threads(const ples_mg_handle *h, int level, int *threads);

/* ---- many grids at once ------------------------------------------------
 * No counterpart in the reference, which solves one grid per run.  A batch
 * groups existing handles on one device; each keeps its resident hierarchy.
 * Members with mixed precision, the zebra smoother, full coarsening,
 * periodic x and z and a dense coarsest level (immersed-boundary masks and
 * cell types allowed) share the batched step list; any other member (x or
 * z walls, FP64, another smoother, semi-coarsening) is solved by the
 * single-grid solver within the same call, after the batched members, and
 * the server solves such a member's requests when it admits them.  One
 * outer iteration of the batched members is a captured
 * CUDA graph of persistent step kernels that walk (member, level, tile)
 * queues; convergence is decided per member on the device, so members of
 * different sizes finish independently.  The stop rule is the relative one
 * of ples_mg_solve (rel_tol), with max_cycles outer iterations. */
typedef struct ples_mg_batch ples_mg_batch;
int ples_mg_batch_create(ples_mg_handle *const *members, int n, ples_mg_batch **out);
/* fi[i] (host, (0:jx+1,0:jy+1,0:jz+1)) in/out, or fi == NULL / fi[i] ==
 * NULL to start from the member's resident solution and keep the result
 * on the device; rhs[i] (host, (1:jx,1:jy,1:jz)); stats[n] or NULL.
 * Returns OK, NOT_CONVERGED or DIVERGED (the worst member) or an error. */
int ples_mg_batch_solve(ples_mg_batch *b, double *const *fi, const double *const *rhs,
                        double rel_tol, int max_cycles, ples_mg_stats *stats);
/* the same with device buffers in the same layouts */
int ples_mg_batch_solve_device(ples_mg_batch *b, double *const *d_fi, const double *const *d_rhs,
                               double rel_tol, int max_cycles, ples_mg_stats *stats);
/* steps (launches) per outer iteration and graph replays so far */
int ples_mg_batch_info(const ples_mg_batch *b, int *steps, long long *replays);
const char *ples_mg_batch_last_error(const ples_mg_batch *b);
void ples_mg_batch_destroy(ples_mg_batch *b);

/* ---- request server with continuous batching ---------------------------
 * No counterpart in the reference.  A server owns a batch over the member
 * handles (their resident hierarchies must fit hbm_budget_bytes, else
 * PLES_MG_OOM; 0 = no budget) and a worker thread.  Requests arrive from
 * any host thread; a request is admitted as soon as its member has no
 * request in flight and joins the next outer iteration of the members
 * already running, so the work of all admitted requests overlaps on the
 * device.  Each solve starts from its member's previous solution (warm
 * start; zero for the first).  A member's requests are served in the order
 * they were submitted; while one solves, the next one's right-hand side is
 * staged, and it is admitted as soon as the first finishes.  Thread-safe. */
typedef struct ples_srv ples_srv;
int ples_srv_create(ples_mg_handle *const *members, int n, double hbm_budget_bytes, ples_srv **out);
/* rhs (host, (1:jx,1:jy,1:jz)) is copied before the call returns; fi_out
 * (host, (0:jx+1,0:jy+1,0:jz+1)) receives the solution and must stay valid
 * until ples_srv_wait returns for the ticket. */
int ples_srv_submit(ples_srv *s, int member, const double *rhs, double *fi_out, double rel_tol,
                    int max_cycles, long long *ticket);
/* blocks until the request completes; returns its status, stats->seconds =
 * latency from submission to completion */
int ples_srv_wait(ples_srv *s, long long ticket, ples_mg_stats *stats);
/* latency percentiles (ms) and throughput of the completed requests */
int ples_srv_report(ples_srv *s, double *p50_ms, double *p99_ms, double *p999_ms,
                    long long *completed, double *solves_per_s);
void ples_srv_destroy(ples_srv *s);

/* ---- fine-level residual norms without device allocation -------------
 * No counterpart in the reference: it has no device and no allocator to
 * avoid.  For callers that must not allocate device memory during the call
 * (a time-step loop whose fields fill the card, an allocator-free section):
 * it calls no cudaMalloc/cudaFree and no allocating library routine, and
 * works in a fixed scratch array inside the library (1 MiB + 16 B per
 * device).  Grids needing more than 65536 blocks of 32 x 8 x 8 cells (about
 * 512^3 cells) are rejected with PLES_MG_BAD_ARG.
 *
 * On the fine level: r = L(fi) - rhs as in ples_mg_apply_residual with
 * level 1 and FP64 (resid_sndrcv.f03:2-156), and norms[0] = sum of r^2,
 * norms[1] = max |r| (the stop test of multi, multigrid.f03:595-631).  With
 * the descriptor's tipo, norms[1] runs over the fluid cells (tipo >= 2), as
 * that stop test with bodyforce = 1 (multigrid.f03:615-631) and the solve's
 * max_residual; with the descriptor's solid mask, solid cells are rows
 * removed from the system: r = 0 there.
 * d_fi (0:jx+1,0:jy+1,0:jz+1) and d_rhs (1:jx,1:jy,1:jz) are device
 * buffers; the ghost layer of d_fi is used as given.  d_r (1:jx,1:jy,1:jz,
 * device) receives r, or is NULL.  norms is host memory; the call returns
 * after the result reached it.  stream NULL = the handle's stream.
 * The scratch's device address is looked up (cudaGetSymbolAddress) when
 * the handle is created, on the handle's device.  All calls on one device
 * share the scratch: calls that overlap in time on that device race;
 * serialise them. */
int ples_mg_residual_norms_device(ples_mg_handle *h, const double *d_fi,
                                  const double *d_rhs, double *d_r, void *stream,
                                  double norms[2]);

#ifdef __cplusplus
}
#endif
#endif /* PLES_MG_H */
