/*
 * ples_oracle.c -- TEST INFRASTRUCTURE ONLY (see ples_oracle.h).
 *
 * FP64 CPU restatement of the PLES pressure-Poisson multigrid.  Each
 * function names the reference routine and lines it follows (paths are
 * relative to the PLES source tree).  The MPI k-slab decomposition is
 * emulated with one pthread per rank; every MPI send/receive pair becomes a
 * barrier-protected copy between the ranks' arrays, so the iterates of an
 * nproc-rank run are reproduced.  With nproc == 1 the reference deadlocks on
 * its self-sends for z-periodic grids (multigrid.f03:784-812, 1335-1340);
 * here the intended single-domain semantics (periodic copies) are used.
 *
 * Parity unpinned by reference outputs (no Fortran compiler or MPI in this
 * image, no golden data in the reference); pinned by known-answer tests on
 * the reference's sample deck instead.
 */
#include "ples_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define MAXLEV 4
#define NGH 8 /* ghost node layers, iniz_metrica.f03:52 */

static __thread char g_err[256];
const char *orc_last_error(void) { return g_err; }
static void set_err(const char *m) { snprintf(g_err, sizeof g_err, "%s", m); }

/* ------------------------------------------------------------------ */
/* Fortran-style arrays with arbitrary lower bounds, column-major.      */
typedef struct {
    double *d;
    int i0, i1, j0, j1, k0, k1;
    long sj, sk;
} arr3;

static arr3 a3(int i0, int i1, int j0, int j1, int k0, int k1) {
    arr3 a;
    a.i0 = i0; a.i1 = i1; a.j0 = j0; a.j1 = j1; a.k0 = k0; a.k1 = k1;
    a.sj = (long)(i1 - i0 + 1);
    a.sk = a.sj * (long)(j1 - j0 + 1);
    a.d = (double *)calloc((size_t)(a.sk * (long)(k1 - k0 + 1)), sizeof(double));
    return a;
}
static void a3_free(arr3 *a) { free(a->d); a->d = NULL; }
static long a3_size(const arr3 *a) { return a->sk * (long)(a->k1 - a->k0 + 1); }

#define AT(a, i, j, k) \
    ((a).d[((long)(k) - (a).k0) * (a).sk + ((long)(j) - (a).j0) * (a).sj + ((long)(i) - (a).i0)])

/* ------------------------------------------------------------------ */
typedef struct {
    int nx, ny, nz;
    arr3 g[9]; /* g11 g12 g13 g21 g22 g23 g31 g32 g33 (r11..r33 in the solver) */
    arr3 i_dx, i_sn, i_sp, i_st, i_av, i_in; /* sett.f03 masks (as reals) */
    arr3 aa, bb, cc;                          /* sett.f03:114-143 */
} orc_level;

struct orc_problem {
    int jx, jy, jz, ip, jp, kp, nproc, nlevel, islor;
    int jxc[MAXLEV + 1], jyc[MAXLEV + 1], jzc[MAXLEV + 1];
    double omega, dt;
    int freesurface;  /* multi's freesurface argument (multigrid.f03:48) */
    double *next_prs; /* surface pressure next_prs(1:jx,1:jz) of myarrays_velo3, or NULL */
    arr3 x, y, z;
    arr3 giac;
    orc_level lev[MAXLEV + 1];
};

#define G11(L) (L)->g[0]
#define G12(L) (L)->g[1]
#define G13(L) (L)->g[2]
#define G21(L) (L)->g[3]
#define G22(L) (L)->g[4]
#define G23(L) (L)->g[5]
#define G31(L) (L)->g[6]
#define G32(L) (L)->g[7]
#define G33(L) (L)->g[8]

/* ------------------------------------------------------------------ */
/* indy.f03:2-100 -- level count and per-level cell counts.             */
static int indy_levels(int n, int cap) {
    int mez1 = n, mez3 = mez1, mez2 = mez1, k = 0;
    while (mez3 == mez1 && k < cap) {
        mez1 = mez2;
        k = k + 1;
        mez2 = mez1 / 2;
        mez3 = 2 * mez2;
    }
    if (mez1 == 1) k = k - 1;
    return k;
}

static void indy(orc_problem *p) {
    int kx = indy_levels(p->jx, 20);
    int ky = indy_levels(p->jy, 4);
    int kz = indy_levels(p->jz / p->nproc, 4);
    int nl = kx < ky ? kx : ky;
    if (kz < nl) nl = kz;
    p->nlevel = nl;
    p->jxc[0] = p->jyc[0] = p->jzc[0] = 0;
    p->jxc[1] = p->jx; p->jyc[1] = p->jy; p->jzc[1] = p->jz;
    for (int n = 2; n <= MAXLEV; n++) {
        p->jxc[n] = p->jxc[n - 1] / 2;
        p->jyc[n] = p->jyc[n - 1] / 2;
        p->jzc[n] = p->jzc[n - 1] / 2;
    }
}

/* ------------------------------------------------------------------ */
/* cellep.f03:2-129 -- ghost node coordinates, one domain (all ranks'    */
/* slabs together).  x-direction first, then z (which copies the        */
/* x-ghosted end blocks xx1/xx2), then y.                                */
static void cellep(orc_problem *p) {
    int jx = p->jx, jy = p->jy, jz = p->jz;
    arr3 *x = &p->x, *y = &p->y, *z = &p->z;
    for (int i = 1; i <= NGH; i++)
        for (int j = 0; j <= jy; j++)
            for (int k = 0; k <= jz; k++) {
                AT(*x, -i, j, k) = AT(*x, 0, j, k) - (AT(*x, jx, j, k) - AT(*x, jx - i, j, k));
                AT(*y, -i, j, k) = AT(*y, jx - i, j, k);
                AT(*z, -i, j, k) = AT(*z, jx - i, j, k);
                AT(*x, jx + i, j, k) = AT(*x, jx, j, k) - (AT(*x, 0, j, k) - AT(*x, i, j, k));
                AT(*y, jx + i, j, k) = AT(*y, i, j, k);
                AT(*z, jx + i, j, k) = AT(*z, i, j, k);
            }
    /* xx1 = planes jz-8..jz, xx2 = planes 0..8 (both x-ghosted above) */
    for (int k = 1; k <= NGH; k++)
        for (int i = -NGH; i <= jx + NGH; i++)
            for (int j = 0; j <= jy; j++) {
                AT(*x, i, j, -k) = AT(*x, i, j, jz - k);
                AT(*y, i, j, -k) = AT(*y, i, j, jz - k);
                AT(*z, i, j, -k) = AT(*z, i, j, 0) - (AT(*z, i, j, jz) - AT(*z, i, j, jz - k));
                AT(*x, i, j, jz + k) = AT(*x, i, j, k);
                AT(*y, i, j, jz + k) = AT(*y, i, j, k);
                AT(*z, i, j, jz + k) = AT(*z, i, j, jz) - (AT(*z, i, j, 0) - AT(*z, i, j, k));
            }
    for (int j = 1; j <= NGH; j++)
        for (int i = -NGH; i <= jx + NGH; i++)
            for (int k = -NGH; k <= jz + NGH; k++) {
                AT(*x, i, -j, k) = AT(*x, i, jy - j, k);
                AT(*y, i, -j, k) = AT(*y, i, 0, k) - (AT(*y, i, jy, k) - AT(*y, i, jy - j, k));
                AT(*z, i, -j, k) = AT(*z, i, jy - j, k);
                AT(*x, i, jy + j, k) = AT(*x, i, j, k);
                AT(*y, i, jy + j, k) = AT(*y, i, jy, k) - (AT(*y, i, 0, k) - AT(*y, i, j, k));
                AT(*z, i, jy + j, k) = AT(*z, i, j, k);
            }
}

/* ------------------------------------------------------------------ */
/* Contravariant metric rows from the nine covariant derivatives:       */
/* gprima.f03, gseconda.f03, gterza.f03 (and the inline copies in       */
/* metrica.f03:170-180, 271-292, 396-410).                              */
static double jac(double xcsi, double ycsi, double zcsi, double xeta, double yeta,
                  double zeta, double xzet, double yzet, double zzet) {
    return xcsi * (yeta * zzet - yzet * zeta) - xeta * (ycsi * zzet - yzet * zcsi) +
           xzet * (ycsi * zeta - yeta * zcsi);
}

/* row 1: t11 = |grad csi|^2/J, t22 = grad csi . grad eta / J, ... */
static void gprima(double xcsi, double ycsi, double zcsi, double xeta, double yeta,
                   double zeta, double xzet, double yzet, double zzet, double *t11,
                   double *t22, double *t33) {
    double giac = jac(xcsi, ycsi, zcsi, xeta, yeta, zeta, xzet, yzet, zzet);
    double csx = yeta * zzet - yzet * zeta;
    double csy = xzet * zeta - xeta * zzet;
    double csz = xeta * yzet - xzet * yeta;
    double etx = yzet * zcsi - ycsi * zzet;
    double ety = xcsi * zzet - xzet * zcsi;
    double etz = xzet * ycsi - xcsi * yzet;
    double ztx = ycsi * zeta - yeta * zcsi;
    double zty = xeta * zcsi - xcsi * zeta;
    double ztz = xcsi * yeta - xeta * ycsi;
    *t11 = (csx * csx + csy * csy + csz * csz) / giac;
    *t22 = (csx * etx + csy * ety + csz * etz) / giac;
    *t33 = (csx * ztx + csy * zty + csz * ztz) / giac;
}
static void gseconda(double xcsi, double ycsi, double zcsi, double xeta, double yeta,
                     double zeta, double xzet, double yzet, double zzet, double *t11,
                     double *t22, double *t33) {
    double etx = yzet * zcsi - ycsi * zzet;
    double ety = xcsi * zzet - xzet * zcsi;
    double etz = xzet * ycsi - xcsi * yzet;
    double csx = yeta * zzet - yzet * zeta;
    double csy = xzet * zeta - xeta * zzet;
    double csz = xeta * yzet - xzet * yeta;
    double ztx = ycsi * zeta - yeta * zcsi;
    double zty = xeta * zcsi - xcsi * zeta;
    double ztz = xcsi * yeta - xeta * ycsi;
    double giac = jac(xcsi, ycsi, zcsi, xeta, yeta, zeta, xzet, yzet, zzet);
    *t11 = (etx * csx + ety * csy + etz * csz) / giac;
    *t22 = (etx * etx + ety * ety + etz * etz) / giac;
    *t33 = (etx * ztx + ety * zty + etz * ztz) / giac;
}
static void gterza(double xcsi, double ycsi, double zcsi, double xeta, double yeta,
                   double zeta, double xzet, double yzet, double zzet, double *t11,
                   double *t22, double *t33) {
    double csx = yeta * zzet - yzet * zeta;
    double csy = xzet * zeta - xeta * zzet;
    double csz = xeta * yzet - xzet * yeta;
    double etx = yzet * zcsi - ycsi * zzet;
    double ety = xcsi * zzet - xzet * zcsi;
    double etz = xzet * ycsi - xcsi * yzet;
    double ztx = ycsi * zeta - yeta * zcsi;
    double zty = xeta * zcsi - xcsi * zeta;
    double ztz = xcsi * yeta - xeta * ycsi;
    double giac = jac(xcsi, ycsi, zcsi, xeta, yeta, zeta, xzet, yzet, zzet);
    *t11 = (ztx * csx + zty * csy + ztz * csz) / giac;
    *t22 = (ztx * etx + zty * ety + ztz * etz) / giac;
    *t33 = (ztx * ztx + zty * zty + ztz * ztz) / giac;
}

/* ------------------------------------------------------------------ */
/* Face metric of level n from fine nodes sub-sampled with stride s =    */
/* 2^(n-1).  For s == 1 these are exactly the expressions of            */
/* metrica.f03:85-419 (node indices i+1 <-> i2 etc.); for s > 1 they are */
/* mul_met, multigrid.f03:2520-2988, with the result divided by pot = s. */
/* Node (a,b,c) below means fine node (a,b,c) of the ghosted arrays.     */
#define QX(a, b, c) AT(p->x, a, b, c)
#define QY(a, b, c) AT(p->y, a, b, c)
#define QZ(a, b, c) AT(p->z, a, b, c)

/* csi-faces: face i of level n, cells j,k (multigrid.f03:2520-2666) */
static void face_csi(const orc_problem *p, int s, int nxl, int i, int j, int k,
                     double t[3]) {
    int jx = p->jx;
    int j2 = j * s, j1 = (j - 1) * s, k2 = k * s, k1 = (k - 1) * s, ic = i * s;
    double xcsi, ycsi, zcsi;
    if (i == 0 && p->ip == 1) {
        int i1 = (i + 1) * s, i2 = (i + 2) * s;
        double x2 = .25 * (QX(i2, j2, k2) + QX(i2, j2, k1) + QX(i2, j1, k2) + QX(i2, j1, k1));
        double x1 = .25 * (QX(i1, j2, k2) + QX(i1, j2, k1) + QX(i1, j1, k2) + QX(i1, j1, k1));
        double x0 = .25 * (QX(0, j2, k2) + QX(0, j2, k1) + QX(0, j1, k2) + QX(0, j1, k1));
        double y2 = .25 * (QY(i2, j2, k2) + QY(i2, j2, k1) + QY(i2, j1, k2) + QY(i2, j1, k1));
        double y1 = .25 * (QY(i1, j2, k2) + QY(i1, j2, k1) + QY(i1, j1, k2) + QY(i1, j1, k1));
        double y0 = .25 * (QY(0, j2, k2) + QY(0, j2, k1) + QY(0, j1, k2) + QY(0, j1, k1));
        double z2 = .25 * (QZ(i2, j2, k2) + QZ(i2, j2, k1) + QZ(i2, j1, k2) + QZ(i2, j1, k1));
        double z1 = .25 * (QZ(i1, j2, k2) + QZ(i1, j2, k1) + QZ(i1, j1, k2) + QZ(i1, j1, k1));
        double z0 = .25 * (QZ(0, j2, k2) + QZ(0, j2, k1) + QZ(0, j1, k2) + QZ(0, j1, k1));
        xcsi = .5 * (-3. * x0 + 4. * x1 - x2);
        ycsi = .5 * (-3. * y0 + 4. * y1 - y2);
        zcsi = .5 * (-3. * z0 + 4. * z1 - z2);
    } else if (i == nxl && p->ip == 1) {
        int i1 = (i - 1) * s, i2 = (i - 2) * s;
        double x2 = .25 * (QX(i2, j2, k2) + QX(i2, j2, k1) + QX(i2, j1, k2) + QX(i2, j1, k1));
        double x1 = .25 * (QX(i1, j2, k2) + QX(i1, j2, k1) + QX(i1, j1, k2) + QX(i1, j1, k1));
        double x0 = .25 * (QX(jx, j2, k2) + QX(jx, j2, k1) + QX(jx, j1, k2) + QX(jx, j1, k1));
        double y2 = .25 * (QY(i2, j2, k2) + QY(i2, j2, k1) + QY(i2, j1, k2) + QY(i2, j1, k1));
        double y1 = .25 * (QY(i1, j2, k2) + QY(i1, j2, k1) + QY(i1, j1, k2) + QY(i1, j1, k1));
        double y0 = .25 * (QY(jx, j2, k2) + QY(jx, j2, k1) + QY(jx, j1, k2) + QY(jx, j1, k1));
        double z2 = .25 * (QZ(i2, j2, k2) + QZ(i2, j2, k1) + QZ(i2, j1, k2) + QZ(i2, j1, k1));
        double z1 = .25 * (QZ(i1, j2, k2) + QZ(i1, j2, k1) + QZ(i1, j1, k2) + QZ(i1, j1, k1));
        double z0 = .25 * (QZ(jx, j2, k2) + QZ(jx, j2, k1) + QZ(jx, j1, k2) + QZ(jx, j1, k1));
        xcsi = .5 * (3. * x0 - 4. * x1 + x2);
        ycsi = .5 * (3. * y0 - 4. * y1 + y2);
        zcsi = .5 * (3. * z0 - 4. * z1 + z2);
    } else {
        int i2 = (i + 1) * s, i1 = (i - 1) * s;
        double xdx = .25 * (QX(i2, j2, k2) + QX(i2, j2, k1) + QX(i2, j1, k2) + QX(i2, j1, k1));
        double xsn = .25 * (QX(i1, j2, k2) + QX(i1, j2, k1) + QX(i1, j1, k2) + QX(i1, j1, k1));
        double ydx = .25 * (QY(i2, j2, k2) + QY(i2, j2, k1) + QY(i2, j1, k2) + QY(i2, j1, k1));
        double ysn = .25 * (QY(i1, j2, k2) + QY(i1, j2, k1) + QY(i1, j1, k2) + QY(i1, j1, k1));
        double zdx = .25 * (QZ(i2, j2, k2) + QZ(i2, j2, k1) + QZ(i2, j1, k2) + QZ(i2, j1, k1));
        double zsn = .25 * (QZ(i1, j2, k2) + QZ(i1, j2, k1) + QZ(i1, j1, k2) + QZ(i1, j1, k1));
        xcsi = .5 * (xdx - xsn);
        ycsi = .5 * (ydx - ysn);
        zcsi = .5 * (zdx - zsn);
    }
    double xeta = .5 * (QX(ic, j2, k2) + QX(ic, j2, k1)) - .5 * (QX(ic, j1, k2) + QX(ic, j1, k1));
    double yeta = .5 * (QY(ic, j2, k2) + QY(ic, j2, k1)) - .5 * (QY(ic, j1, k2) + QY(ic, j1, k1));
    double zeta = .5 * (QZ(ic, j2, k2) + QZ(ic, j2, k1)) - .5 * (QZ(ic, j1, k2) + QZ(ic, j1, k1));
    double xzet = .5 * (QX(ic, j2, k2) + QX(ic, j1, k2)) - .5 * (QX(ic, j2, k1) + QX(ic, j1, k1));
    double yzet = .5 * (QY(ic, j2, k2) + QY(ic, j1, k2)) - .5 * (QY(ic, j2, k1) + QY(ic, j1, k1));
    double zzet = .5 * (QZ(ic, j2, k2) + QZ(ic, j1, k2)) - .5 * (QZ(ic, j2, k1) + QZ(ic, j1, k1));
    gprima(xcsi, ycsi, zcsi, xeta, yeta, zeta, xzet, yzet, zzet, &t[0], &t[1], &t[2]);
}

/* eta-faces: face j of level n, cells i,k (multigrid.f03:2675-2827) */
static void face_eta(const orc_problem *p, int s, int nyl, int i, int j, int k,
                     double t[3]) {
    int jy = p->jy;
    int i2 = i * s, i1 = (i - 1) * s, k2 = k * s, k1 = (k - 1) * s, jc = j * s;
    double xeta, yeta, zeta;
    if (j == 0 && p->jp == 1) {
        int j1 = (j + 1) * s, j2 = (j + 2) * s;
        int j0 = j; /* node index 0 */
        double x2 = .25 * (QX(i2, j2, k2) + QX(i2, j2, k1) + QX(i1, j2, k1) + QX(i1, j2, k2));
        double x1 = .25 * (QX(i2, j1, k2) + QX(i2, j1, k1) + QX(i1, j1, k1) + QX(i1, j1, k2));
        double x0 = .25 * (QX(i2, j0, k2) + QX(i2, j0, k1) + QX(i1, j0, k1) + QX(i1, j0, k2));
        double y2 = .25 * (QY(i2, j2, k2) + QY(i2, j2, k1) + QY(i1, j2, k1) + QY(i1, j2, k2));
        double y1 = .25 * (QY(i2, j1, k2) + QY(i2, j1, k1) + QY(i1, j1, k1) + QY(i1, j1, k2));
        double y0 = .25 * (QY(i2, j0, k2) + QY(i2, j0, k1) + QY(i1, j0, k1) + QY(i1, j0, k2));
        double z2 = .25 * (QZ(i2, j2, k2) + QZ(i2, j2, k1) + QZ(i1, j2, k1) + QZ(i1, j2, k2));
        double z1 = .25 * (QZ(i2, j1, k2) + QZ(i2, j1, k1) + QZ(i1, j1, k1) + QZ(i1, j1, k2));
        double z0 = .25 * (QZ(i2, j0, k2) + QZ(i2, j0, k1) + QZ(i1, j0, k1) + QZ(i1, j0, k2));
        xeta = .5 * (-3. * x0 + 4. * x1 - x2);
        yeta = .5 * (-3. * y0 + 4. * y1 - y2);
        zeta = .5 * (-3. * z0 + 4. * z1 - z2);
    } else if (j == nyl && p->jp == 1) {
        int j1 = (j - 1) * s, j2 = (j - 2) * s;
        double x2 = .25 * (QX(i2, j2, k2) + QX(i2, j2, k1) + QX(i1, j2, k1) + QX(i1, j2, k2));
        double x1 = .25 * (QX(i2, j1, k2) + QX(i2, j1, k1) + QX(i1, j1, k1) + QX(i1, j1, k2));
        double x0 = .25 * (QX(i2, jy, k2) + QX(i2, jy, k1) + QX(i1, jy, k1) + QX(i1, jy, k2));
        double y2 = .25 * (QY(i2, j2, k2) + QY(i2, j2, k1) + QY(i1, j2, k1) + QY(i1, j2, k2));
        double y1 = .25 * (QY(i2, j1, k2) + QY(i2, j1, k1) + QY(i1, j1, k1) + QY(i1, j1, k2));
        double y0 = .25 * (QY(i2, jy, k2) + QY(i2, jy, k1) + QY(i1, jy, k1) + QY(i1, jy, k2));
        double z2 = .25 * (QZ(i2, j2, k2) + QZ(i2, j2, k1) + QZ(i1, j2, k1) + QZ(i1, j2, k2));
        double z1 = .25 * (QZ(i2, j1, k2) + QZ(i2, j1, k1) + QZ(i1, j1, k1) + QZ(i1, j1, k2));
        double z0 = .25 * (QZ(i2, jy, k2) + QZ(i2, jy, k1) + QZ(i1, jy, k1) + QZ(i1, jy, k2));
        xeta = .5 * (3. * x0 - 4. * x1 + x2);
        yeta = .5 * (3. * y0 - 4. * y1 + y2);
        zeta = .5 * (3. * z0 - 4. * z1 + z2);
    } else {
        int j2 = (j + 1) * s, j1 = (j - 1) * s;
        double xsop = .25 * (QX(i2, j2, k2) + QX(i2, j2, k1) + QX(i1, j2, k1) + QX(i1, j2, k2));
        double xsot = .25 * (QX(i2, j1, k2) + QX(i2, j1, k1) + QX(i1, j1, k1) + QX(i1, j1, k2));
        double ysop = .25 * (QY(i2, j2, k2) + QY(i2, j2, k1) + QY(i1, j2, k1) + QY(i1, j2, k2));
        double ysot = .25 * (QY(i2, j1, k2) + QY(i2, j1, k1) + QY(i1, j1, k1) + QY(i1, j1, k2));
        double zsop = .25 * (QZ(i2, j2, k2) + QZ(i2, j2, k1) + QZ(i1, j2, k1) + QZ(i1, j2, k2));
        double zsot = .25 * (QZ(i2, j1, k2) + QZ(i2, j1, k1) + QZ(i1, j1, k1) + QZ(i1, j1, k2));
        xeta = .5 * (xsop - xsot);
        yeta = .5 * (ysop - ysot);
        zeta = .5 * (zsop - zsot);
    }
    double yzet = .5 * (QY(i2, jc, k2) + QY(i1, jc, k2)) - .5 * (QY(i2, jc, k1) + QY(i1, jc, k1));
    double zcsi = .5 * (QZ(i2, jc, k2) + QZ(i2, jc, k1)) - .5 * (QZ(i1, jc, k2) + QZ(i1, jc, k1));
    double ycsi = .5 * (QY(i2, jc, k2) + QY(i2, jc, k1)) - .5 * (QY(i1, jc, k2) + QY(i1, jc, k1));
    double zzet = .5 * (QZ(i2, jc, k2) + QZ(i1, jc, k2)) - .5 * (QZ(i2, jc, k1) + QZ(i1, jc, k1));
    double xcsi = .5 * (QX(i2, jc, k2) + QX(i2, jc, k1)) - .5 * (QX(i1, jc, k2) + QX(i1, jc, k1));
    double xzet = .5 * (QX(i2, jc, k2) + QX(i1, jc, k2)) - .5 * (QX(i2, jc, k1) + QX(i1, jc, k1));
    gseconda(xcsi, ycsi, zcsi, xeta, yeta, zeta, xzet, yzet, zzet, &t[0], &t[1], &t[2]);
}

/* zeta-faces: face k of level n, cells i,j (multigrid.f03:2836-2988) */
static void face_zet(const orc_problem *p, int s, int nzl, int i, int j, int k,
                     double t[3]) {
    int jz = p->jz;
    int i2 = i * s, i1 = (i - 1) * s, j2 = j * s, j1 = (j - 1) * s, kc = k * s;
    double xzet, yzet, zzet;
    if (k == 0 && p->kp == 1) {
        int k1 = (k + 1) * s, k2 = (k + 2) * s, k0 = k;
        double x2 = .25 * (QX(i2, j2, k2) + QX(i2, j1, k2) + QX(i1, j1, k2) + QX(i1, j2, k2));
        double x1 = .25 * (QX(i2, j2, k1) + QX(i2, j1, k1) + QX(i1, j1, k1) + QX(i1, j2, k1));
        double x0 = .25 * (QX(i2, j2, k0) + QX(i2, j1, k0) + QX(i1, j1, k0) + QX(i1, j2, k0));
        double y2 = .25 * (QY(i2, j2, k2) + QY(i2, j1, k2) + QY(i1, j1, k2) + QY(i1, j2, k2));
        double y1 = .25 * (QY(i2, j2, k1) + QY(i2, j1, k1) + QY(i1, j1, k1) + QY(i1, j2, k1));
        double y0 = .25 * (QY(i2, j2, k0) + QY(i2, j1, k0) + QY(i1, j1, k0) + QY(i1, j2, k0));
        double z2 = .25 * (QZ(i2, j2, k2) + QZ(i2, j1, k2) + QZ(i1, j1, k2) + QZ(i1, j2, k2));
        double z1 = .25 * (QZ(i2, j2, k1) + QZ(i2, j1, k1) + QZ(i1, j1, k1) + QZ(i1, j2, k1));
        double z0 = .25 * (QZ(i2, j2, k0) + QZ(i2, j1, k0) + QZ(i1, j1, k0) + QZ(i1, j2, k0));
        xzet = .5 * (-3. * x0 + 4. * x1 - x2);
        yzet = .5 * (-3. * y0 + 4. * y1 - y2);
        zzet = .5 * (-3. * z0 + 4. * z1 - z2);
    } else if (k == nzl && p->kp == 1) {
        int k1 = (k - 1) * s, k2 = (k - 2) * s;
        double x2 = .25 * (QX(i2, j2, k2) + QX(i2, j1, k2) + QX(i1, j1, k2) + QX(i1, j2, k2));
        double x1 = .25 * (QX(i2, j2, k1) + QX(i2, j1, k1) + QX(i1, j1, k1) + QX(i1, j2, k1));
        double x0 = .25 * (QX(i2, j2, jz) + QX(i2, j1, jz) + QX(i1, j1, jz) + QX(i1, j2, jz));
        double y2 = .25 * (QY(i2, j2, k2) + QY(i2, j1, k2) + QY(i1, j1, k2) + QY(i1, j2, k2));
        double y1 = .25 * (QY(i2, j2, k1) + QY(i2, j1, k1) + QY(i1, j1, k1) + QY(i1, j2, k1));
        double y0 = .25 * (QY(i2, j2, jz) + QY(i2, j1, jz) + QY(i1, j1, jz) + QY(i1, j2, jz));
        double z2 = .25 * (QZ(i2, j2, k2) + QZ(i2, j1, k2) + QZ(i1, j1, k2) + QZ(i1, j2, k2));
        double z1 = .25 * (QZ(i2, j2, k1) + QZ(i2, j1, k1) + QZ(i1, j1, k1) + QZ(i1, j2, k1));
        double z0 = .25 * (QZ(i2, j2, jz) + QZ(i2, j1, jz) + QZ(i1, j1, jz) + QZ(i1, j2, jz));
        xzet = .5 * (3. * x0 - 4. * x1 + x2);
        yzet = .5 * (3. * y0 - 4. * y1 + y2);
        zzet = .5 * (3. * z0 - 4. * z1 + z2);
    } else {
        int k2 = (k + 1) * s, k1 = (k - 1) * s;
        double xav = .25 * (QX(i2, j2, k2) + QX(i2, j1, k2) + QX(i1, j1, k2) + QX(i1, j2, k2));
        double xdt = .25 * (QX(i2, j2, k1) + QX(i2, j1, k1) + QX(i1, j1, k1) + QX(i1, j2, k1));
        double yav = .25 * (QY(i2, j2, k2) + QY(i2, j1, k2) + QY(i1, j1, k2) + QY(i1, j2, k2));
        double ydt = .25 * (QY(i2, j2, k1) + QY(i2, j1, k1) + QY(i1, j1, k1) + QY(i1, j2, k1));
        double zav = .25 * (QZ(i2, j2, k2) + QZ(i2, j1, k2) + QZ(i1, j1, k2) + QZ(i1, j2, k2));
        double zdt = .25 * (QZ(i2, j2, k1) + QZ(i2, j1, k1) + QZ(i1, j1, k1) + QZ(i1, j2, k1));
        xzet = .5 * (xav - xdt);
        yzet = .5 * (yav - ydt);
        zzet = .5 * (zav - zdt);
    }
    double ycsi = .5 * (QY(i2, j2, kc) + QY(i2, j1, kc)) - .5 * (QY(i1, j2, kc) + QY(i1, j1, kc));
    double zeta = .5 * (QZ(i2, j2, kc) + QZ(i1, j2, kc)) - .5 * (QZ(i2, j1, kc) + QZ(i1, j1, kc));
    double yeta = .5 * (QY(i2, j2, kc) + QY(i1, j2, kc)) - .5 * (QY(i2, j1, kc) + QY(i1, j1, kc));
    double zcsi = .5 * (QZ(i2, j2, kc) + QZ(i2, j1, kc)) - .5 * (QZ(i1, j2, kc) + QZ(i1, j1, kc));
    double xcsi = .5 * (QX(i2, j2, kc) + QX(i2, j1, kc)) - .5 * (QX(i1, j2, kc) + QX(i1, j1, kc));
    double xeta = .5 * (QX(i2, j2, kc) + QX(i1, j2, kc)) - .5 * (QX(i2, j1, kc) + QX(i1, j1, kc));
    gterza(xcsi, ycsi, zcsi, xeta, yeta, zeta, xzet, yzet, zzet, &t[0], &t[1], &t[2]);
}

/* metrica.f03:85-419 (s = 1) and mul_met multigrid.f03:2520-2988 (s > 1) */
static void build_metric(orc_problem *p, int n) {
    orc_level *L = &p->lev[n];
    int nx = L->nx, ny = L->ny, nz = L->nz;
    int s = 1 << (n - 1);
    double pot = (double)s;
    double t[3];
    G11(L) = a3(0, nx, 1, ny, 1, nz); G12(L) = a3(0, nx, 1, ny, 1, nz); G13(L) = a3(0, nx, 1, ny, 1, nz);
    G21(L) = a3(1, nx, 0, ny, 1, nz); G22(L) = a3(1, nx, 0, ny, 1, nz); G23(L) = a3(1, nx, 0, ny, 1, nz);
    G31(L) = a3(1, nx, 1, ny, 0, nz); G32(L) = a3(1, nx, 1, ny, 0, nz); G33(L) = a3(1, nx, 1, ny, 0, nz);
    for (int i = 0; i <= nx; i++)
        for (int j = 1; j <= ny; j++)
            for (int k = 1; k <= nz; k++) {
                face_csi(p, s, nx, i, j, k, t);
                if (n == 1) {
                    AT(G11(L), i, j, k) = t[0]; AT(G12(L), i, j, k) = t[1]; AT(G13(L), i, j, k) = t[2];
                } else {
                    AT(G11(L), i, j, k) = t[0] / pot; AT(G12(L), i, j, k) = t[1] / pot;
                    AT(G13(L), i, j, k) = t[2] / pot;
                }
            }
    for (int i = 1; i <= nx; i++)
        for (int j = 0; j <= ny; j++)
            for (int k = 1; k <= nz; k++) {
                face_eta(p, s, ny, i, j, k, t);
                if (n == 1) {
                    AT(G21(L), i, j, k) = t[0]; AT(G22(L), i, j, k) = t[1]; AT(G23(L), i, j, k) = t[2];
                } else {
                    AT(G21(L), i, j, k) = t[0] / pot; AT(G22(L), i, j, k) = t[1] / pot;
                    AT(G23(L), i, j, k) = t[2] / pot;
                }
            }
    for (int i = 1; i <= nx; i++)
        for (int j = 1; j <= ny; j++)
            for (int k = 0; k <= nz; k++) {
                face_zet(p, s, nz, i, j, k, t);
                if (n == 1) {
                    AT(G31(L), i, j, k) = t[0]; AT(G32(L), i, j, k) = t[1]; AT(G33(L), i, j, k) = t[2];
                } else {
                    AT(G31(L), i, j, k) = t[0] / pot; AT(G32(L), i, j, k) = t[1] / pot;
                    AT(G33(L), i, j, k) = t[2] / pot;
                }
            }
}

/* metrica.f03:426-494 -- J^-1 at cell centroids (diagnostic only) */
static void build_giac(orc_problem *p) {
    int jx = p->jx, jy = p->jy, jz = p->jz;
    p->giac = a3(1, jx, 1, jy, 1, jz);
    for (int i = 1; i <= jx; i++)
        for (int j = 1; j <= jy; j++)
            for (int k = 1; k <= jz; k++) {
                double xcsi = .25 * (QX(i, j, k) + QX(i, j, k - 1) + QX(i, j - 1, k - 1) + QX(i, j - 1, k)) -
                              .25 * (QX(i - 1, j, k) + QX(i - 1, j, k - 1) + QX(i - 1, j - 1, k - 1) + QX(i - 1, j - 1, k));
                double ycsi = .25 * (QY(i, j, k) + QY(i, j, k - 1) + QY(i, j - 1, k - 1) + QY(i, j - 1, k)) -
                              .25 * (QY(i - 1, j, k) + QY(i - 1, j, k - 1) + QY(i - 1, j - 1, k - 1) + QY(i - 1, j - 1, k));
                double zcsi = .25 * (QZ(i, j, k) + QZ(i, j, k - 1) + QZ(i, j - 1, k - 1) + QZ(i, j - 1, k)) -
                              .25 * (QZ(i - 1, j, k) + QZ(i - 1, j, k - 1) + QZ(i - 1, j - 1, k - 1) + QZ(i - 1, j - 1, k));
                double xeta = .25 * (QX(i, j, k) + QX(i, j, k - 1) + QX(i - 1, j, k - 1) + QX(i - 1, j, k)) -
                              .25 * (QX(i, j - 1, k) + QX(i, j - 1, k - 1) + QX(i - 1, j - 1, k - 1) + QX(i - 1, j - 1, k));
                double yeta = .25 * (QY(i, j, k) + QY(i, j, k - 1) + QY(i - 1, j, k - 1) + QY(i - 1, j, k)) -
                              .25 * (QY(i, j - 1, k) + QY(i, j - 1, k - 1) + QY(i - 1, j - 1, k - 1) + QY(i - 1, j - 1, k));
                double zeta = .25 * (QZ(i, j, k) + QZ(i, j, k - 1) + QZ(i - 1, j, k - 1) + QZ(i - 1, j, k)) -
                              .25 * (QZ(i, j - 1, k) + QZ(i, j - 1, k - 1) + QZ(i - 1, j - 1, k - 1) + QZ(i - 1, j - 1, k));
                double xzet = .25 * (QX(i, j, k) + QX(i, j - 1, k) + QX(i - 1, j - 1, k) + QX(i - 1, j, k)) -
                              .25 * (QX(i, j, k - 1) + QX(i, j - 1, k - 1) + QX(i - 1, j - 1, k - 1) + QX(i - 1, j, k - 1));
                double yzet = .25 * (QY(i, j, k) + QY(i, j - 1, k) + QY(i - 1, j - 1, k) + QY(i - 1, j, k)) -
                              .25 * (QY(i, j, k - 1) + QY(i, j - 1, k - 1) + QY(i - 1, j - 1, k - 1) + QY(i - 1, j, k - 1));
                double zzet = .25 * (QZ(i, j, k) + QZ(i, j - 1, k) + QZ(i - 1, j - 1, k) + QZ(i - 1, j, k)) -
                              .25 * (QZ(i, j, k - 1) + QZ(i, j - 1, k - 1) + QZ(i - 1, j - 1, k - 1) + QZ(i - 1, j, k - 1));
                AT(p->giac, i, j, k) = jac(xcsi, ycsi, zcsi, xeta, yeta, zeta, xzet, yzet, zzet);
            }
}

/* sett.f03:2-146 -- masks and fixed tridiagonal coefficients per level.  */
/* As in the reference, i_in is set on rank 0's first plane and i_av on   */
/* the last rank's last plane only when that rank is not also rank 0.     */
static void sett(orc_problem *p, int n) {
    orc_level *L = &p->lev[n];
    int nx = L->nx, ny = L->ny, nz = L->nz;
    int ip = p->ip, jp = p->jp, kp = p->kp;
    L->i_dx = a3(1, nx, 1, ny, 1, nz); L->i_sn = a3(1, nx, 1, ny, 1, nz);
    L->i_sp = a3(1, nx, 1, ny, 1, nz); L->i_st = a3(1, nx, 1, ny, 1, nz);
    L->i_av = a3(1, nx, 1, ny, 1, nz); L->i_in = a3(1, nx, 1, ny, 1, nz);
    L->aa = a3(1, nx, 0, ny + 1, 1, nz); L->bb = a3(1, nx, 0, ny + 1, 1, nz);
    L->cc = a3(1, nx, 0, ny + 1, 1, nz);
    for (long q = 0; q < a3_size(&L->i_dx); q++) {
        L->i_dx.d[q] = L->i_sn.d[q] = L->i_sp.d[q] = 1.0;
        L->i_st.d[q] = L->i_av.d[q] = L->i_in.d[q] = 1.0;
    }
    for (int j = 1; j <= ny; j++)
        for (int k = 1; k <= nz; k++) {
            AT(L->i_sn, 1, j, k) = 1 - ip;
            AT(L->i_dx, nx, j, k) = 1 - ip;
        }
    for (int i = 1; i <= nx; i++)
        for (int k = 1; k <= nz; k++) {
            AT(L->i_st, i, 1, k) = 1 - jp;
            AT(L->i_sp, i, ny, k) = 1 - jp;
        }
    for (int j = 1; j <= ny; j++)
        for (int i = 1; i <= nx; i++) AT(L->i_in, i, j, 1) = 1 - kp;
    if (p->nproc > 1)
        for (int j = 1; j <= ny; j++)
            for (int i = 1; i <= nx; i++) AT(L->i_av, i, j, nz) = 1 - kp;
    double pot = (double)(1 << (n - 1));
    double ppot2 = 1 / pot / pot;
    for (int k = 1; k <= nz; k++)
        for (int i = 1; i <= nx; i++) {
            for (int j = 1; j <= ny; j++) {
                AT(L->aa, i, j, k) = ppot2 * AT(G22(L), i, j - 1, k);
                AT(L->bb, i, j, k) =
                    -ppot2 * (AT(G22(L), i, j, k) + AT(G22(L), i, j - 1, k) +
                              AT(G11(L), i, j, k) * AT(L->i_dx, i, j, k) +
                              AT(G11(L), i - 1, j, k) * AT(L->i_sn, i, j, k) +
                              AT(G33(L), i, j, k) * AT(L->i_av, i, j, k) +
                              AT(G33(L), i, j, k - 1) * AT(L->i_in, i, j, k));
                AT(L->cc, i, j, k) = ppot2 * AT(G22(L), i, j, k);
            }
            AT(L->aa, i, 0, k) = 0.;
            AT(L->bb, i, 0, k) = AT(G22(L), i, 0, k) * ppot2;
            AT(L->cc, i, 0, k) = -AT(G22(L), i, 0, k) * ppot2;
            AT(L->aa, i, ny + 1, k) = -AT(G22(L), i, ny, k) * ppot2;
            AT(L->bb, i, ny + 1, k) = AT(G22(L), i, ny, k) * ppot2;
            AT(L->cc, i, ny + 1, k) = 0.;
        }
}

/* ------------------------------------------------------------------ */
orc_problem *orc_create(int jx, int jy, int jz, int ip, int jp, int kp, int nlevmax,
                        int nproc, double omega, int islor, double dt, const double *xn,
                        const double *yn, const double *zn) {
    if (jx < NGH || jz < NGH || jy < 4) { set_err("grid too small (jx,jz >= 8, jy >= 4)"); return NULL; }
    if (jp != 1) { set_err("y-periodic grids are not supported (multigrid.f03:1744-1746)"); return NULL; }
    if ((ip != 0 && ip != 1) || (kp != 0 && kp != 1)) { set_err("ip/kp must be 0 or 1"); return NULL; }
    if (nproc < 1 || jz % nproc) { set_err("nproc must divide jz"); return NULL; }
    if (nlevmax < 1 || nlevmax > MAXLEV) { set_err("nlevmax must be 1..4"); return NULL; }
    if (islor != 0 && islor != 1) { set_err("islor must be 0 or 1"); return NULL; }
    orc_problem *p = (orc_problem *)calloc(1, sizeof *p);
    p->jx = jx; p->jy = jy; p->jz = jz; p->ip = ip; p->jp = jp; p->kp = kp;
    p->nproc = nproc; p->omega = omega; p->islor = islor; p->dt = dt;
    indy(p);
    if (p->nlevel > nlevmax) p->nlevel = nlevmax;
    /* stratiParticle.f03:3843-3848 and multigrid.f03:138-142: every level's
     * jzc must split evenly over the ranks */
    for (int n = 1; n <= p->nlevel; n++)
        if (p->jzc[n] % nproc || p->jzc[n] / nproc < 1) {
            set_err("each level's jzc must be divisible by nproc");
            free(p);
            return NULL;
        }
    p->x = a3(-NGH, jx + NGH, -NGH, jy + NGH, -NGH, jz + NGH);
    p->y = a3(-NGH, jx + NGH, -NGH, jy + NGH, -NGH, jz + NGH);
    p->z = a3(-NGH, jx + NGH, -NGH, jy + NGH, -NGH, jz + NGH);
    long q = 0;
    for (int k = 0; k <= jz; k++)
        for (int j = 0; j <= jy; j++)
            for (int i = 0; i <= jx; i++, q++) {
                AT(p->x, i, j, k) = xn[q];
                AT(p->y, i, j, k) = yn[q];
                AT(p->z, i, j, k) = zn[q];
            }
    cellep(p);
    for (int n = 1; n <= p->nlevel; n++) {
        p->lev[n].nx = p->jxc[n];
        p->lev[n].ny = p->jyc[n];
        p->lev[n].nz = p->jzc[n];
        build_metric(p, n);
        sett(p, n);
    }
    build_giac(p);
    return p;
}

void orc_destroy(orc_problem *p) {
    if (!p) return;
    for (int n = 1; n <= p->nlevel; n++) {
        orc_level *L = &p->lev[n];
        for (int c = 0; c < 9; c++) a3_free(&L->g[c]);
        a3_free(&L->i_dx); a3_free(&L->i_sn); a3_free(&L->i_sp);
        a3_free(&L->i_st); a3_free(&L->i_av); a3_free(&L->i_in);
        a3_free(&L->aa); a3_free(&L->bb); a3_free(&L->cc);
    }
    a3_free(&p->x); a3_free(&p->y); a3_free(&p->z); a3_free(&p->giac);
    free(p->next_prs);
    free(p);
}

int orc_set_free_surface(orc_problem *p, int freesurface, const double *next_prs) {
    if (!p || (freesurface != 0 && freesurface != 1)) return -1;
    p->freesurface = freesurface;
    free(p->next_prs);
    p->next_prs = NULL;
    if (next_prs) {
        p->next_prs = (double *)malloc(sizeof(double) * (size_t)p->jx * p->jz);
        memcpy(p->next_prs, next_prs, sizeof(double) * (size_t)p->jx * p->jz);
    }
    return 0;
}

int orc_nlevel(const orc_problem *p) { return p->nlevel; }
void orc_level_dims(const orc_problem *p, int n, int *nx, int *ny, int *nz) {
    *nx = p->jxc[n]; *ny = p->jyc[n]; *nz = p->jzc[n];
}

int orc_get_metric(const orc_problem *p, int n, int which, double *out) {
    if (n < 1 || n > p->nlevel || which < 0 || which > 9) return -1;
    const arr3 *a = which == 9 ? &p->giac : &p->lev[n].g[which];
    if (which == 9 && n != 1) return -1;
    memcpy(out, a->d, sizeof(double) * (size_t)a3_size(a));
    return 0;
}
int orc_get_coords(const orc_problem *p, int c, double *out) {
    const arr3 *a = c == 0 ? &p->x : c == 1 ? &p->y : &p->z;
    memcpy(out, a->d, sizeof(double) * (size_t)a3_size(a));
    return 0;
}

/* ------------------------------------------------------------------ */
/* Rank emulation.                                                      */
typedef struct orc_world orc_world;
typedef struct {
    orc_world *W;
    int r;
    int ks[MAXLEV + 1], ke[MAXLEV + 1];
    arr3 pr[MAXLEV + 1]; /* pr1..pr4 (0:nx+1,0:ny+1,ks-1:ke+1) */
} orc_rank;

struct orc_world {
    orc_problem *P;
    int nproc;
    orc_rank *ranks;
    pthread_barrier_t bar;
    /* fine-level shared inputs and work arrays (global k; ranks write their
     * own planes only) */
    const double *cs[6];
    arr3 cs1, cs2, cs3, cs4, cs5, cs6;
    arr3 rhs;             /* caller rhs (1:jx,1:jy,1:jz) */
    arr3 rhsv[MAXLEV + 1]; /* restricted right-hand sides, levels 2.. */
    arr3 rhsn[MAXLEV + 1]; /* residuals, levels 1..nlevel-1 */
    arr3 fi;              /* caller fi (0:jx+1,0:jy+1,0:jz+1) */
    double eps;
    int ficycle, stop_mode;
    double *loc_max, *loc_sq; /* per-rank stop-test partials */
    double rhs_norm;
    int cycles;
    double resmax, relres;
};

static void sync_all(orc_world *W) {
    if (W->nproc > 1) pthread_barrier_wait(&W->bar);
}

/* copy (ia:ib, ja:jb) of src plane ksrc into dst plane kdst */
static void copy_plane(arr3 *dst, int kdst, const arr3 *src, int ksrc, int ia, int ib,
                       int ja, int jb) {
    for (int j = ja; j <= jb; j++)
        for (int i = ia; i <= ib; i++) AT(*dst, i, j, kdst) = AT(*src, i, j, ksrc);
}

static double cs_at(const arr3 *a, int u, int v) {
    return a->d ? AT(*a, u, v, 0) : 0.0;
}

/* mul_boun_sndrcv, multigrid.f03:1013-1936.  fs: its freesurface argument
 * (the point SOR passes multi's, the line SOR always 0, multigrid.f03:2019) */
static void mul_boun(orc_rank *R, int n, int fs) {
    orc_world *W = R->W;
    orc_problem *P = W->P;
    orc_level *L = &P->lev[n];
    arr3 *pr = &R->pr[n];
    int nx = L->nx, ny = L->ny, nz = L->nz, ks = R->ks[n], ke = R->ke[n];
    int myid = R->r, nproc = W->nproc;
    int ip = P->ip, jp = P->jp, kp = P->kp;
    double inv_dt = 1. / P->dt, coef = 0.25;
    double an = (n == 1) ? 1. : 0.;
    orc_rank *R0 = &W->ranks[0], *RL = &W->ranks[nproc - 1];
    orc_rank *left = myid > 0 ? &W->ranks[myid - 1] : NULL;
    orc_rank *right = myid < nproc - 1 ? &W->ranks[myid + 1] : NULL;
    arr3 *r11 = &G11(L), *r12 = &G12(L), *r13 = &G13(L);
    arr3 *r21 = &G21(L), *r22 = &G22(L), *r23 = &G23(L);
    arr3 *r31 = &G31(L), *r32 = &G32(L), *r33 = &G33(L);

    for (int kkk = 1; kkk <= 5; kkk++) {
        /* left and right (:1111-1158) */
        if (ip == 1) {
            for (int k = ks; k <= ke; k++)
                for (int j = 1; j <= ny; j++) {
                    double inv_r11 = 1. / AT(*r11, 0, j, k);
                    AT(*pr, 0, j, k) =
                        AT(*pr, 1, j, k) - an * cs_at(&W->cs1, j, k) * inv_dt * inv_r11 +
                        coef * inv_r11 *
                            (AT(*r12, 0, j, k) * (AT(*pr, 1, j + 1, k) + AT(*pr, 0, j + 1, k) -
                                                  AT(*pr, 1, j - 1, k) - AT(*pr, 0, j - 1, k)) +
                             AT(*r13, 0, j, k) * (AT(*pr, 1, j, k + 1) + AT(*pr, 0, j, k + 1) -
                                                  AT(*pr, 1, j, k - 1) - AT(*pr, 0, j, k - 1)));
                    inv_r11 = 1. / AT(*r11, nx, j, k);
                    AT(*pr, nx + 1, j, k) =
                        AT(*pr, nx, j, k) + an * cs_at(&W->cs2, j, k) * inv_dt * inv_r11 -
                        coef * inv_r11 *
                            (AT(*r12, nx, j, k) * (AT(*pr, nx + 1, j + 1, k) + AT(*pr, nx, j + 1, k) -
                                                   AT(*pr, nx + 1, j - 1, k) - AT(*pr, nx, j - 1, k)) +
                             AT(*r13, nx, j, k) * (AT(*pr, nx + 1, j, k + 1) + AT(*pr, nx, j, k + 1) -
                                                   AT(*pr, nx + 1, j, k - 1) - AT(*pr, nx, j, k - 1)));
                }
        } else {
            for (int k = ks; k <= ke; k++)
                for (int j = 1; j <= ny; j++) {
                    AT(*pr, 0, j, k) = AT(*pr, nx, j, k);
                    AT(*pr, nx + 1, j, k) = AT(*pr, 1, j, k);
                }
        }
        /* bottom and upper (:1160-1262) */
        for (int k = ks; k <= ke; k++)
            for (int i = 1; i <= nx; i++) {
                if (fs) {
                    /* free surface at the top (:1188-1222): PrS0 = 0 at the
                     * first time step (next_prs not given) and on coarse
                     * levels, next_prs(i,k) on level 1 otherwise; the
                     * bottom keeps its wall relation */
                    double inv_r22 = 1. / AT(*r22, i, 0, k);
                    AT(*pr, i, 0, k) =
                        AT(*pr, i, 1, k) - an * cs_at(&W->cs3, i, k) * inv_dt * inv_r22 +
                        coef * inv_r22 *
                            (AT(*r21, i, 0, k) * (AT(*pr, i + 1, 1, k) + AT(*pr, i + 1, 0, k) -
                                                  AT(*pr, i - 1, 1, k) - AT(*pr, i - 1, 0, k)) +
                             AT(*r23, i, 0, k) * (AT(*pr, i, 1, k + 1) + AT(*pr, i, 0, k + 1) -
                                                  AT(*pr, i, 1, k - 1) - AT(*pr, i, 0, k - 1)));
                    double prs0 = 0.;
                    if (n == 1 && P->next_prs) prs0 = P->next_prs[(size_t)(k - 1) * P->jx + (i - 1)];
                    inv_r22 = 1. / AT(*r22, i, ny, k);
                    AT(*pr, i, ny + 1, k) =
                        (prs0 * 2) -
                        (AT(*pr, i, ny, k) -
                         coef * inv_r22 *
                             (AT(*r21, i, ny, k) * (AT(*pr, i + 1, ny + 1, k) + AT(*pr, i + 1, ny, k) -
                                                    AT(*pr, i - 1, ny + 1, k) - AT(*pr, i - 1, ny, k)) +
                              AT(*r23, i, ny, k) * (AT(*pr, i, ny + 1, k + 1) + AT(*pr, i, ny, k + 1) -
                                                    AT(*pr, i, ny + 1, k - 1) - AT(*pr, i, ny, k - 1))));
                    continue;
                }
                double inv_r22 = 1. / AT(*r22, i, 0, k);
                AT(*pr, i, 0, k) =
                    AT(*pr, i, 1, k) - an * cs_at(&W->cs3, i, k) * inv_dt * inv_r22 +
                    coef * inv_r22 *
                        (AT(*r21, i, 0, k) * (AT(*pr, i + 1, 1, k) + AT(*pr, i + 1, 0, k) -
                                              AT(*pr, i - 1, 1, k) - AT(*pr, i - 1, 0, k)) +
                         AT(*r23, i, 0, k) * (AT(*pr, i, 1, k + 1) + AT(*pr, i, 0, k + 1) -
                                              AT(*pr, i, 1, k - 1) - AT(*pr, i, 0, k - 1)));
                inv_r22 = 1. / AT(*r22, i, ny, k);
                AT(*pr, i, ny + 1, k) =
                    AT(*pr, i, ny, k) + an * cs_at(&W->cs4, i, k) * inv_dt * inv_r22 -
                    coef * inv_r22 *
                        (AT(*r21, i, ny, k) * (AT(*pr, i + 1, ny + 1, k) + AT(*pr, i + 1, ny, k) -
                                               AT(*pr, i - 1, ny + 1, k) - AT(*pr, i - 1, ny, k)) +
                         AT(*r23, i, ny, k) * (AT(*pr, i, ny + 1, k + 1) + AT(*pr, i, ny, k + 1) -
                                               AT(*pr, i, ny + 1, k - 1) - AT(*pr, i, ny, k - 1)));
            }
        (void)jp;
        /* back and front (:1280-1316) */
        if (kp == 1) {
            if (myid == 0)
                for (int i = 1; i <= nx; i++)
                    for (int j = 1; j <= ny; j++) {
                        double inv_r33 = 1. / AT(*r33, i, j, 0);
                        AT(*pr, i, j, 0) =
                            AT(*pr, i, j, 1) - an * cs_at(&W->cs5, i, j) * inv_dt * inv_r33 +
                            coef * inv_r33 *
                                (AT(*r31, i, j, 0) * (AT(*pr, i + 1, j, 1) + AT(*pr, i + 1, j, 0) -
                                                      AT(*pr, i - 1, j, 1) - AT(*pr, i - 1, j, 0)) +
                                 AT(*r32, i, j, 0) * (AT(*pr, i, j + 1, 1) + AT(*pr, i, j + 1, 0) -
                                                      AT(*pr, i, j - 1, 1) - AT(*pr, i, j - 1, 0)));
                    }
            if (myid == nproc - 1)
                for (int i = 1; i <= nx; i++)
                    for (int j = 1; j <= ny; j++) {
                        double inv_r33 = 1. / AT(*r33, i, j, nz);
                        AT(*pr, i, j, nz + 1) =
                            AT(*pr, i, j, nz) + an * cs_at(&W->cs6, i, j) * inv_dt * inv_r33 -
                            coef * inv_r33 *
                                (AT(*r31, i, j, nz) * (AT(*pr, i + 1, j, nz + 1) + AT(*pr, i + 1, j, nz) -
                                                       AT(*pr, i - 1, j, nz + 1) - AT(*pr, i - 1, j, nz)) +
                                 AT(*r32, i, j, nz) * (AT(*pr, i, j + 1, nz + 1) + AT(*pr, i, j + 1, nz) -
                                                       AT(*pr, i, j - 1, nz + 1) - AT(*pr, i, j - 1, nz)));
                    }
        } else {
            /* periodicity (:1325-1354): interior plane exchange 0 <-> nproc-1 */
            sync_all(W);
            if (myid == 0) copy_plane(pr, 0, &RL->pr[n], nz, 1, nx, 1, ny);
            if (myid == nproc - 1) copy_plane(pr, nz + 1, &R0->pr[n], 1, 1, nx, 1, ny);
            sync_all(W);
        }
        /* edges and corners (:1360-1742), jp = 1 */
        if (kp == 0) {
            /* 1) corner lines streamwise */
            sync_all(W);
            if (myid == 0)
                for (int i = 1; i <= nx; i++) {
                    AT(*pr, i, ny + 1, 0) = AT(RL->pr[n], i, ny + 1, nz);
                    AT(*pr, i, 0, 0) = AT(RL->pr[n], i, 0, nz);
                }
            if (myid == nproc - 1)
                for (int i = 1; i <= nx; i++) {
                    AT(*pr, i, ny + 1, nz + 1) = AT(R0->pr[n], i, ny + 1, 1);
                    AT(*pr, i, 0, nz + 1) = AT(R0->pr[n], i, 0, 1);
                }
            sync_all(W);
            /* 2) vertical frame (planes k = 0, nz+1) */
            sync_all(W);
            if (ip == 0) {
                if (myid == 0)
                    for (int j = 0; j <= ny + 1; j++) {
                        AT(*pr, 0, j, 0) = AT(RL->pr[n], nx, j, nz);
                        AT(*pr, nx + 1, j, 0) = AT(RL->pr[n], 1, j, nz);
                    }
                if (myid == nproc - 1)
                    for (int j = 0; j <= ny + 1; j++) {
                        AT(*pr, 0, j, nz + 1) = AT(R0->pr[n], nx, j, 1);
                        AT(*pr, nx + 1, j, nz + 1) = AT(R0->pr[n], 1, j, 1);
                    }
            } else {
                if (myid == 0)
                    for (int j = 0; j <= ny + 1; j++) {
                        AT(*pr, nx + 1, j, 0) = AT(RL->pr[n], nx + 1, j, nz);
                        AT(*pr, 0, j, 0) = AT(RL->pr[n], 0, j, nz);
                    }
                if (myid == nproc - 1)
                    for (int j = 0; j <= ny + 1; j++) {
                        AT(*pr, nx + 1, j, nz + 1) = AT(R0->pr[n], nx + 1, j, 1);
                        AT(*pr, 0, j, nz + 1) = AT(R0->pr[n], 0, j, 1);
                    }
            }
            sync_all(W);
            /* 3) horizontal square */
            if (ip == 0)
                for (int k = ks; k <= ke; k++) {
                    AT(*pr, 0, ny + 1, k) = AT(*pr, nx, ny + 1, k);
                    AT(*pr, 0, 0, k) = AT(*pr, nx, 0, k);
                    AT(*pr, nx + 1, ny + 1, k) = AT(*pr, 1, ny + 1, k);
                    AT(*pr, nx + 1, 0, k) = AT(*pr, 1, 0, k);
                }
            else
                for (int k = ks; k <= ke; k++) {
                    AT(*pr, 0, ny + 1, k) = AT(*pr, 0, ny, k);
                    AT(*pr, 0, 0, k) = AT(*pr, 0, 1, k);
                    AT(*pr, nx + 1, ny + 1, k) = AT(*pr, nx + 1, ny, k);
                    AT(*pr, nx + 1, 0, k) = AT(*pr, nx + 1, 1, k);
                }
        } else {
            /* kp = 1 (:1628-1742) */
            if (myid == 0)
                for (int i = 1; i <= nx; i++) {
                    AT(*pr, i, 0, 0) = AT(*pr, i, 1, 0);
                    AT(*pr, i, ny + 1, 0) = AT(*pr, i, ny, 0);
                }
            else if (myid == nproc - 1)
                for (int i = 1; i <= nx; i++) {
                    AT(*pr, i, 0, nz + 1) = AT(*pr, i, 1, nz + 1);
                    AT(*pr, i, ny + 1, nz + 1) = AT(*pr, i, ny, nz + 1);
                }
            if (ip == 0) {
                if (myid == 0)
                    for (int j = 0; j <= ny + 1; j++) {
                        AT(*pr, 0, j, 0) = AT(*pr, nx, j, 0);
                        AT(*pr, nx + 1, j, 0) = AT(*pr, 1, j, 0);
                    }
                else if (myid == nproc - 1)
                    for (int j = 0; j <= ny + 1; j++) {
                        AT(*pr, 0, j, nz + 1) = AT(*pr, nx, j, nz + 1);
                        AT(*pr, nx + 1, j, nz + 1) = AT(*pr, 1, j, nz + 1);
                    }
            } else {
                if (myid == 0)
                    for (int j = 0; j <= ny + 1; j++) {
                        AT(*pr, 0, j, 0) = AT(*pr, 1, j, 0);
                        AT(*pr, nx + 1, j, 0) = AT(*pr, nx, j, 0);
                    }
                else if (myid == nproc - 1)
                    for (int j = 0; j <= ny + 1; j++) {
                        AT(*pr, 0, j, nz + 1) = AT(*pr, 1, j, nz + 1);
                        AT(*pr, nx + 1, j, nz + 1) = AT(*pr, nx, j, nz + 1);
                    }
            }
            if (ip == 0)
                for (int k = ks; k <= ke; k++) {
                    AT(*pr, 0, ny + 1, k) = AT(*pr, nx, ny + 1, k);
                    AT(*pr, 0, 0, k) = AT(*pr, nx, 0, k);
                    AT(*pr, nx + 1, ny + 1, k) = AT(*pr, 1, ny + 1, k);
                    AT(*pr, nx + 1, 0, k) = AT(*pr, 1, 0, k);
                }
            else
                for (int k = ks; k <= ke; k++) {
                    AT(*pr, 0, ny + 1, k) = AT(*pr, 1, ny + 1, k);
                    AT(*pr, 0, 0, k) = AT(*pr, 1, 0, k);
                    AT(*pr, nx + 1, ny + 1, k) = AT(*pr, nx, ny + 1, k);
                    AT(*pr, nx + 1, 0, k) = AT(*pr, nx, 0, k);
                }
        }
        /* boundary columns across slab boundaries (:1750-1840, ip = 1) */
        if (ip == 1) {
            sync_all(W);
            if (right)
                for (int j = 1; j <= ny; j++) {
                    AT(*pr, 0, j, ke + 1) = AT(right->pr[n], 0, j, right->ks[n]);
                    AT(*pr, 1, j, ke + 1) = AT(right->pr[n], 1, j, right->ks[n]);
                    AT(*pr, nx, j, ke + 1) = AT(right->pr[n], nx, j, right->ks[n]);
                    AT(*pr, nx + 1, j, ke + 1) = AT(right->pr[n], nx + 1, j, right->ks[n]);
                }
            if (left)
                for (int j = 1; j <= ny; j++) {
                    AT(*pr, 0, j, ks - 1) = AT(left->pr[n], 0, j, left->ke[n]);
                    AT(*pr, 1, j, ks - 1) = AT(left->pr[n], 1, j, left->ke[n]);
                    AT(*pr, nx, j, ks - 1) = AT(left->pr[n], nx, j, left->ke[n]);
                    AT(*pr, nx + 1, j, ks - 1) = AT(left->pr[n], nx + 1, j, left->ke[n]);
                }
            sync_all(W);
        }
        /* boundary rows across slab boundaries (:1842-1931, jp = 1) */
        sync_all(W);
        if (right)
            for (int i = 1; i <= nx; i++) {
                AT(*pr, i, 0, ke + 1) = AT(right->pr[n], i, 0, right->ks[n]);
                AT(*pr, i, 1, ke + 1) = AT(right->pr[n], i, 1, right->ks[n]);
                AT(*pr, i, ny, ke + 1) = AT(right->pr[n], i, ny, right->ks[n]);
                AT(*pr, i, ny + 1, ke + 1) = AT(right->pr[n], i, ny + 1, right->ks[n]);
            }
        if (left)
            for (int i = 1; i <= nx; i++) {
                AT(*pr, i, 0, ks - 1) = AT(left->pr[n], i, 0, left->ke[n]);
                AT(*pr, i, 1, ks - 1) = AT(left->pr[n], i, 1, left->ke[n]);
                AT(*pr, i, ny, ks - 1) = AT(left->pr[n], i, ny, left->ke[n]);
                AT(*pr, i, ny + 1, ks - 1) = AT(left->pr[n], i, ny + 1, left->ke[n]);
            }
        sync_all(W);
    }
}

/* z-periodic interior planes before a sweep (multigrid.f03:784-812) */
static void zperiodic_planes(orc_rank *R, int n) {
    orc_world *W = R->W;
    orc_level *L = &W->P->lev[n];
    int nx = L->nx, ny = L->ny, nz = L->nz, nproc = W->nproc, myid = R->r;
    sync_all(W);
    if (myid == 0) copy_plane(&R->pr[n], 0, &W->ranks[nproc - 1].pr[n], nz, 1, nx, 1, ny);
    if (myid == nproc - 1) copy_plane(&R->pr[n], nz + 1, &W->ranks[0].pr[n], 1, 1, nx, 1, ny);
    sync_all(W);
}

/* slab halo after a sweep (multigrid.f03:929-966): interior plane only */
static void slab_halo(orc_rank *R, int n, int full) {
    orc_world *W = R->W;
    orc_level *L = &W->P->lev[n];
    int nx = L->nx, ny = L->ny, myid = R->r, nproc = W->nproc;
    int a0 = full ? 0 : 1, ax = full ? nx + 1 : nx, b0 = full ? 0 : 1, by = full ? ny + 1 : ny;
    sync_all(W);
    if (myid < nproc - 1) {
        orc_rank *rt = &W->ranks[myid + 1];
        copy_plane(&R->pr[n], R->ke[n] + 1, &rt->pr[n], rt->ks[n], a0, ax, b0, by);
    }
    if (myid > 0) {
        orc_rank *lf = &W->ranks[myid - 1];
        copy_plane(&R->pr[n], R->ks[n] - 1, &lf->pr[n], lf->ke[n], a0, ax, b0, by);
    }
    sync_all(W);
}

/* solut_sndrcv_sor, multigrid.f03:656-1010 */
static void smooth_sor(orc_rank *R, int n, int kss, const arr3 *rh) {
    orc_problem *P = R->W->P;
    orc_level *L = &P->lev[n];
    arr3 *pr = &R->pr[n];
    int nx = L->nx, ny = L->ny, ks = R->ks[n], ke = R->ke[n];
    double pot = (double)(1 << (n - 1));
    double ppot1 = 1 / pot, ppot2 = 1 / pot / pot, omega = P->omega;
    arr3 *r11 = &G11(L), *r12 = &G12(L), *r13 = &G13(L);
    arr3 *r21 = &G21(L), *r22 = &G22(L), *r23 = &G23(L);
    arr3 *r31 = &G31(L), *r32 = &G32(L), *r33 = &G33(L);
    for (int kk = 1; kk <= kss; kk++) {
        mul_boun(R, n, P->freesurface);
        if (P->kp == 0) zperiodic_planes(R, n);
        for (int k = ks; k <= ke; k++)
            for (int j = 1; j <= ny; j++) {
                if (P->ip == 0) {
                    AT(*pr, 0, j, k) = AT(*pr, nx, j, k);
                    AT(*pr, nx + 1, j, k) = AT(*pr, 1, j, k);
                }
                for (int i = 1; i <= nx; i++) {
                    double res_dx = (AT(*r11, i, j, k) * (AT(*pr, i + 1, j, k) - AT(*pr, i, j, k)) +
                                     .25 * (AT(*r12, i, j, k) * (AT(*pr, i + 1, j + 1, k) + AT(*pr, i, j + 1, k) -
                                                                 AT(*pr, i + 1, j - 1, k) - AT(*pr, i, j - 1, k)) +
                                            AT(*r13, i, j, k) * (AT(*pr, i + 1, j, k + 1) + AT(*pr, i, j, k + 1) -
                                                                 AT(*pr, i + 1, j, k - 1) - AT(*pr, i, j, k - 1)))) *
                                    ppot1;
                    double den_dx = AT(*r11, i, j, k) * ppot2;
                    double res_sn = (AT(*r11, i - 1, j, k) * (AT(*pr, i, j, k) - AT(*pr, i - 1, j, k)) +
                                     .25 * (AT(*r12, i - 1, j, k) * (AT(*pr, i, j + 1, k) + AT(*pr, i - 1, j + 1, k) -
                                                                     AT(*pr, i, j - 1, k) - AT(*pr, i - 1, j - 1, k)) +
                                            AT(*r13, i - 1, j, k) * (AT(*pr, i, j, k + 1) + AT(*pr, i - 1, j, k + 1) -
                                                                     AT(*pr, i, j, k - 1) - AT(*pr, i - 1, j, k - 1)))) *
                                    ppot1;
                    double den_sn = AT(*r11, i - 1, j, k) * ppot2;
                    double res_sop = (AT(*r22, i, j, k) * (AT(*pr, i, j + 1, k) - AT(*pr, i, j, k)) +
                                      .25 * (AT(*r21, i, j, k) * (AT(*pr, i + 1, j + 1, k) + AT(*pr, i + 1, j, k) -
                                                                  AT(*pr, i - 1, j + 1, k) - AT(*pr, i - 1, j, k)) +
                                             AT(*r23, i, j, k) * (AT(*pr, i, j + 1, k + 1) + AT(*pr, i, j, k + 1) -
                                                                  AT(*pr, i, j + 1, k - 1) - AT(*pr, i, j, k - 1)))) *
                                     ppot1;
                    double den_sop = AT(*r22, i, j, k) * ppot2;
                    double res_sot = (AT(*r22, i, j - 1, k) * (AT(*pr, i, j, k) - AT(*pr, i, j - 1, k)) +
                                      .25 * (AT(*r21, i, j - 1, k) * (AT(*pr, i + 1, j, k) + AT(*pr, i + 1, j - 1, k) -
                                                                      AT(*pr, i - 1, j, k) - AT(*pr, i - 1, j - 1, k)) +
                                             AT(*r23, i, j - 1, k) * (AT(*pr, i, j, k + 1) + AT(*pr, i, j - 1, k + 1) -
                                                                      AT(*pr, i, j, k - 1) - AT(*pr, i, j - 1, k - 1)))) *
                                     ppot1;
                    double den_sot = AT(*r22, i, j - 1, k) * ppot2;
                    double res_av = (AT(*r33, i, j, k) * (AT(*pr, i, j, k + 1) - AT(*pr, i, j, k)) +
                                     .25 * (AT(*r31, i, j, k) * (AT(*pr, i + 1, j, k + 1) + AT(*pr, i + 1, j, k) -
                                                                 AT(*pr, i - 1, j, k + 1) - AT(*pr, i - 1, j, k)) +
                                            AT(*r32, i, j, k) * (AT(*pr, i, j + 1, k + 1) + AT(*pr, i, j + 1, k) -
                                                                 AT(*pr, i, j - 1, k + 1) - AT(*pr, i, j - 1, k)))) *
                                    ppot1;
                    double den_av = AT(*r33, i, j, k) * ppot2;
                    double res_ind = (AT(*r33, i, j, k - 1) * (AT(*pr, i, j, k) - AT(*pr, i, j, k - 1)) +
                                      .25 * (AT(*r31, i, j, k - 1) * (AT(*pr, i + 1, j, k) + AT(*pr, i + 1, j, k - 1) -
                                                                      AT(*pr, i - 1, j, k) - AT(*pr, i - 1, j, k - 1)) +
                                             AT(*r32, i, j, k - 1) * (AT(*pr, i, j + 1, k) + AT(*pr, i, j + 1, k - 1) -
                                                                      AT(*pr, i, j - 1, k) - AT(*pr, i, j - 1, k - 1)))) *
                                     ppot1;
                    double den_ind = AT(*r33, i, j, k - 1) * ppot2;
                    double resi = (res_dx - res_sn + res_sop - res_sot + res_av - res_ind) * ppot1 -
                                  AT(*rh, i, j, k);
                    double den = den_dx + den_sn + den_sop + den_sot + den_av + den_ind;
                    AT(*pr, i, j, k) = AT(*pr, i, j, k) + omega * resi / den;
                }
            }
        slab_halo(R, n, 0);
    }
    slab_halo(R, n, 1);
}

/* tridag.f03:2-32 on 0-based arrays of length m (Fortran a(1..m)) */
static void tridag(double *aa, double *bb, double *cc, double *ff, int m) {
    bb[0] = 1. / bb[0];
    aa[0] = ff[0] * bb[0];
    for (int k = 1; k < m; k++) {
        int k1 = k - 1;
        cc[k1] = cc[k1] * bb[k1];
        bb[k] = bb[k] - aa[k] * cc[k1];
        bb[k] = 1. / bb[k];
        aa[k] = (ff[k] - aa[k] * aa[k1]) * bb[k];
    }
    ff[m - 1] = aa[m - 1];
    for (int k = m - 2; k >= 0; k--) ff[k] = aa[k] - cc[k] * ff[k + 1];
}

/* solut_sndrcv_slor, multigrid.f03:1939-2290 */
static void smooth_slor(orc_rank *R, int n, int kss, const arr3 *rh) {
    orc_world *W = R->W;
    orc_problem *P = W->P;
    orc_level *L = &P->lev[n];
    arr3 *pr = &R->pr[n];
    int nx = L->nx, ny = L->ny, ks = R->ks[n], ke = R->ke[n];
    double an = (n == 1) ? 1. : 0.;
    double pot = (double)(1 << (n - 1));
    double ppot2 = 1 / pot / pot, omega = P->omega, dt = P->dt;
    arr3 *r11 = &G11(L), *r12 = &G12(L), *r13 = &G13(L);
    arr3 *r21 = &G21(L), *r23 = &G23(L);
    arr3 *r31 = &G31(L), *r32 = &G32(L), *r33 = &G33(L);
    double *aa0 = malloc(sizeof(double) * (ny + 2)), *bb0 = malloc(sizeof(double) * (ny + 2));
    double *cc0 = malloc(sizeof(double) * (ny + 2)), *ff0 = malloc(sizeof(double) * (ny + 2));
    for (int kk = 1; kk <= kss; kk++) {
        mul_boun(R, n, 0); /* the line SOR sets freesurface = 0 (multigrid.f03:2019) */
        if (P->kp == 0) zperiodic_planes(R, n);
        for (int k = ks; k <= ke; k++) {
            if (P->ip == 0)
                for (int j = 1; j <= ny; j++) {
                    AT(*pr, 0, j, k) = AT(*pr, nx, j, k);
                    AT(*pr, nx + 1, j, k) = AT(*pr, 1, j, k);
                }
            for (int i = 1; i <= nx; i++) {
                for (int j = 1; j <= ny; j++) {
                    double idx = AT(L->i_dx, i, j, k), isn = AT(L->i_sn, i, j, k);
                    double iav = AT(L->i_av, i, j, k), iin = AT(L->i_in, i, j, k);
                    double f =
                        -AT(*r11, i, j, k) * AT(*pr, i + 1, j, k) * idx -
                        (1. - idx) * an * cs_at(&W->cs2, j, k) / dt -
                        AT(*r11, i - 1, j, k) * AT(*pr, i - 1, j, k) * isn +
                        (1. - isn) * an * cs_at(&W->cs1, j, k) / dt -
                        .25 * AT(*r12, i, j, k) * idx *
                            (AT(*pr, i + 1, j + 1, k) + AT(*pr, i, j + 1, k) - AT(*pr, i + 1, j - 1, k) - AT(*pr, i, j - 1, k)) -
                        .25 * AT(*r13, i, j, k) * idx *
                            (AT(*pr, i + 1, j, k + 1) + AT(*pr, i, j, k + 1) - AT(*pr, i + 1, j, k - 1) - AT(*pr, i, j, k - 1)) +
                        .25 * AT(*r12, i - 1, j, k) * isn *
                            (AT(*pr, i, j + 1, k) + AT(*pr, i - 1, j + 1, k) - AT(*pr, i, j - 1, k) - AT(*pr, i - 1, j - 1, k)) +
                        .25 * AT(*r13, i - 1, j, k) * isn *
                            (AT(*pr, i, j, k + 1) + AT(*pr, i - 1, j, k + 1) - AT(*pr, i, j, k - 1) - AT(*pr, i - 1, j, k - 1))
                        /**/
                        - AT(*r33, i, j, k) * AT(*pr, i, j, k + 1) * iav -
                        (1. - iav) * an * cs_at(&W->cs6, i, j) / dt -
                        AT(*r33, i, j, k - 1) * AT(*pr, i, j, k - 1) * iin +
                        (1. - iin) * an * cs_at(&W->cs5, i, j) / dt -
                        .25 * AT(*r31, i, j, k) * iav *
                            (AT(*pr, i + 1, j, k + 1) + AT(*pr, i + 1, j, k) - AT(*pr, i - 1, j, k + 1) - AT(*pr, i - 1, j, k)) -
                        .25 * AT(*r32, i, j, k) * iav *
                            (AT(*pr, i, j + 1, k + 1) + AT(*pr, i, j + 1, k) - AT(*pr, i, j - 1, k + 1) - AT(*pr, i, j - 1, k)) +
                        .25 * AT(*r31, i, j, k - 1) * iin *
                            (AT(*pr, i + 1, j, k) + AT(*pr, i + 1, j, k - 1) - AT(*pr, i - 1, j, k) - AT(*pr, i - 1, j, k - 1)) +
                        .25 * AT(*r32, i, j, k - 1) * iin *
                            (AT(*pr, i, j + 1, k) + AT(*pr, i, j + 1, k - 1) - AT(*pr, i, j - 1, k) - AT(*pr, i, j - 1, k - 1))
                        /**/
                        - .25 * AT(*r21, i, j, k) *
                              (AT(*pr, i + 1, j + 1, k) + AT(*pr, i + 1, j, k) - AT(*pr, i - 1, j + 1, k) - AT(*pr, i - 1, j, k)) -
                        .25 * AT(*r23, i, j, k) *
                            (AT(*pr, i, j + 1, k + 1) + AT(*pr, i, j, k + 1) - AT(*pr, i, j + 1, k - 1) - AT(*pr, i, j, k - 1)) +
                        .25 * AT(*r21, i, j - 1, k) *
                            (AT(*pr, i + 1, j, k) + AT(*pr, i + 1, j - 1, k) - AT(*pr, i - 1, j, k) - AT(*pr, i - 1, j - 1, k)) +
                        .25 * AT(*r23, i, j - 1, k) *
                            (AT(*pr, i, j, k + 1) + AT(*pr, i, j - 1, k + 1) - AT(*pr, i, j, k - 1) - AT(*pr, i, j - 1, k - 1));
                    ff0[j] = f * ppot2 + AT(*rh, i, j, k);
                }
                ff0[0] = (-an * cs_at(&W->cs3, i, k) / dt +
                          .25 * AT(*r21, i, 0, k) *
                              (AT(*pr, i + 1, 1, k) + AT(*pr, i + 1, 0, k) - AT(*pr, i - 1, 1, k) - AT(*pr, i - 1, 0, k)) +
                          .25 * AT(*r23, i, 0, k) *
                              (AT(*pr, i, 1, k + 1) + AT(*pr, i, 0, k + 1) - AT(*pr, i, 1, k - 1) - AT(*pr, i, 0, k - 1))) *
                         ppot2;
                ff0[ny + 1] =
                    (an * cs_at(&W->cs4, i, k) / dt -
                     .25 * AT(*r21, i, ny, k) *
                         (AT(*pr, i + 1, ny + 1, k) + AT(*pr, i + 1, ny, k) - AT(*pr, i - 1, ny + 1, k) - AT(*pr, i - 1, ny, k)) -
                     .25 * AT(*r23, i, ny, k) *
                         (AT(*pr, i, ny + 1, k + 1) + AT(*pr, i, ny, k + 1) - AT(*pr, i, ny + 1, k - 1) - AT(*pr, i, ny, k - 1))) *
                    ppot2;
                for (int j = 0; j <= ny + 1; j++) {
                    aa0[j] = AT(L->aa, i, j, k);
                    bb0[j] = AT(L->bb, i, j, k);
                    cc0[j] = AT(L->cc, i, j, k);
                }
                tridag(aa0, bb0, cc0, ff0, ny + 2);
                for (int j = 0; j <= ny + 1; j++)
                    AT(*pr, i, j, k) = AT(*pr, i, j, k) + omega * (ff0[j] - AT(*pr, i, j, k));
            }
        }
        slab_halo(R, n, 0);
    }
    slab_halo(R, n, 1);
    free(aa0); free(bb0); free(cc0); free(ff0);
}

/* resid_sndrcv.f03:2-156 on one rank's planes */
static void resid_planes(orc_problem *P, int n, const arr3 *pr, const arr3 *rh, arr3 *rh1,
                         int ks, int ke) {
    orc_level *L = &P->lev[n];
    int nx = L->nx, ny = L->ny;
    double pot = (double)(1 << (n - 1));
    double inv_pot = 1. / pot, coef = 0.25;
    arr3 *r11 = &G11(L), *r12 = &G12(L), *r13 = &G13(L);
    arr3 *r21 = &G21(L), *r22 = &G22(L), *r23 = &G23(L);
    arr3 *r31 = &G31(L), *r32 = &G32(L), *r33 = &G33(L);
    for (int k = ks; k <= ke; k++)
        for (int j = 1; j <= ny; j++)
            for (int i = 1; i <= nx; i++) {
                double res_dx = (AT(*r11, i, j, k) * (AT(*pr, i + 1, j, k) - AT(*pr, i, j, k)) +
                                 coef * (AT(*r12, i, j, k) * (AT(*pr, i + 1, j + 1, k) + AT(*pr, i, j + 1, k) -
                                                              AT(*pr, i + 1, j - 1, k) - AT(*pr, i, j - 1, k)) +
                                         AT(*r13, i, j, k) * (AT(*pr, i + 1, j, k + 1) + AT(*pr, i, j, k + 1) -
                                                              AT(*pr, i + 1, j, k - 1) - AT(*pr, i, j, k - 1)))) *
                                inv_pot;
                double res_sn = (AT(*r11, i - 1, j, k) * (AT(*pr, i, j, k) - AT(*pr, i - 1, j, k)) +
                                 coef * (AT(*r12, i - 1, j, k) * (AT(*pr, i, j + 1, k) + AT(*pr, i - 1, j + 1, k) -
                                                                  AT(*pr, i, j - 1, k) - AT(*pr, i - 1, j - 1, k)) +
                                         AT(*r13, i - 1, j, k) * (AT(*pr, i, j, k + 1) + AT(*pr, i - 1, j, k + 1) -
                                                                  AT(*pr, i, j, k - 1) - AT(*pr, i - 1, j, k - 1)))) *
                                inv_pot;
                double res_sop = (AT(*r22, i, j, k) * (AT(*pr, i, j + 1, k) - AT(*pr, i, j, k)) +
                                  coef * (AT(*r21, i, j, k) * (AT(*pr, i + 1, j + 1, k) + AT(*pr, i + 1, j, k) -
                                                               AT(*pr, i - 1, j + 1, k) - AT(*pr, i - 1, j, k)) +
                                          AT(*r23, i, j, k) * (AT(*pr, i, j + 1, k + 1) + AT(*pr, i, j, k + 1) -
                                                               AT(*pr, i, j + 1, k - 1) - AT(*pr, i, j, k - 1)))) *
                                 inv_pot;
                double res_sot = (AT(*r22, i, j - 1, k) * (AT(*pr, i, j, k) - AT(*pr, i, j - 1, k)) +
                                  coef * (AT(*r21, i, j - 1, k) * (AT(*pr, i + 1, j, k) + AT(*pr, i + 1, j - 1, k) -
                                                                   AT(*pr, i - 1, j, k) - AT(*pr, i - 1, j - 1, k)) +
                                          AT(*r23, i, j - 1, k) * (AT(*pr, i, j, k + 1) + AT(*pr, i, j - 1, k + 1) -
                                                                   AT(*pr, i, j, k - 1) - AT(*pr, i, j - 1, k - 1)))) *
                                 inv_pot;
                double res_av = (AT(*r33, i, j, k) * (AT(*pr, i, j, k + 1) - AT(*pr, i, j, k)) +
                                 coef * (AT(*r31, i, j, k) * (AT(*pr, i + 1, j, k + 1) + AT(*pr, i + 1, j, k) -
                                                              AT(*pr, i - 1, j, k + 1) - AT(*pr, i - 1, j, k)) +
                                         AT(*r32, i, j, k) * (AT(*pr, i, j + 1, k + 1) + AT(*pr, i, j + 1, k) -
                                                              AT(*pr, i, j - 1, k + 1) - AT(*pr, i, j - 1, k)))) *
                                inv_pot;
                double res_ind = (AT(*r33, i, j, k - 1) * (AT(*pr, i, j, k) - AT(*pr, i, j, k - 1)) +
                                  coef * (AT(*r31, i, j, k - 1) * (AT(*pr, i + 1, j, k) + AT(*pr, i + 1, j, k - 1) -
                                                                   AT(*pr, i - 1, j, k) - AT(*pr, i - 1, j, k - 1)) +
                                          AT(*r32, i, j, k - 1) * (AT(*pr, i, j + 1, k) + AT(*pr, i, j + 1, k - 1) -
                                                                   AT(*pr, i, j - 1, k) - AT(*pr, i, j - 1, k - 1)))) *
                                 inv_pot;
                AT(*rh1, i, j, k) = (res_dx - res_sn + res_sop - res_sot + res_av - res_ind) * inv_pot -
                                    AT(*rh, i, j, k);
            }
}

/* restrict_sndrcv.f03:2-56: coarse planes ks2..ke2 of level n+1 */
static void restrict_planes(orc_problem *P, int n, const arr3 *rh, arr3 *rh1, int ks2,
                            int ke2) {
    int nx2 = P->jxc[n + 1], ny2 = P->jyc[n + 1];
    double inv_8 = 1. / 8.;
    for (int k = ks2; k <= ke2; k++)
        for (int j = 1; j <= ny2; j++)
            for (int i = 1; i <= nx2; i++) {
                int id = 2 * i, jd = 2 * j, kd = 2 * k;
                double v = AT(*rh, id, jd, kd) + AT(*rh, id - 1, jd, kd) + AT(*rh, id, jd - 1, kd) +
                           AT(*rh, id - 1, jd - 1, kd) + AT(*rh, id, jd, kd - 1) +
                           AT(*rh, id - 1, jd, kd - 1) + AT(*rh, id, jd - 1, kd - 1) +
                           AT(*rh, id - 1, jd - 1, kd - 1);
                AT(*rh1, i, j, k) = -v * inv_8;
            }
}

/* prolong.f03:2-261: coarse cells k = k0..ke2 into the fine array */
static void prolong_planes(orc_problem *P, int n, arr3 *prf, const arr3 *pr, int k0,
                           int ke2) {
    int nx2 = P->jxc[n + 1], ny2 = P->jyc[n + 1];
    static const double w[8][8] = {
        /* (di,dj,dk) child offsets: 000,100,010,001,110,101,011,111 -- weights of
         * pr(i,j,k), pr(i+1,j,k), pr(i,j+1,k), pr(i,j,k+1), pr(i+1,j+1,k),
         * pr(i+1,j,k+1), pr(i,j+1,k+1), pr(i+1,j+1,k+1) (prolong.f03:64-261) */
        {27., 9., 9., 9., 3., 3., 3., 1.}, {9., 27., 3., 3., 9., 9., 1., 3.},
        {9., 3., 27., 3., 9., 1., 9., 3.}, {9., 3., 3., 27., 1., 9., 9., 3.},
        {3., 9., 9., 1., 27., 3., 3., 9.}, {3., 9., 1., 9., 3., 27., 3., 9.},
        {1., 3., 3., 3., 9., 9., 9., 27.}, {3., 1., 9., 9., 3., 3., 27., 9.}};
    static const int off[8][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1},
                                  {1, 1, 0}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
    double inv_64 = 1. / 64.;
    for (int k = k0; k <= ke2; k++)
        for (int j = 0; j <= ny2; j++)
            for (int i = 0; i <= nx2; i++) {
                double c[8] = {AT(*pr, i, j, k),         AT(*pr, i + 1, j, k),
                               AT(*pr, i, j + 1, k),     AT(*pr, i, j, k + 1),
                               AT(*pr, i + 1, j + 1, k), AT(*pr, i + 1, j, k + 1),
                               AT(*pr, i, j + 1, k + 1), AT(*pr, i + 1, j + 1, k + 1)};
                for (int q = 0; q < 8; q++) {
                    int fi = 2 * i + off[q][0], fj = 2 * j + off[q][1], fk = 2 * k + off[q][2];
                    AT(*prf, fi, fj, fk) =
                        AT(*prf, fi, fj, fk) +
                        (w[q][0] * c[0] + w[q][1] * c[1] + w[q][2] * c[2] + w[q][3] * c[3] +
                         w[q][4] * c[4] + w[q][5] * c[5] + w[q][6] * c[6] + w[q][7] * c[7]) *
                            inv_64;
                }
            }
    (void)nx2;
}

/* prolong + slab plane hand-over (prolong.f03:266-302) */
static void prolong_rank(orc_rank *R, int n) {
    orc_world *W = R->W;
    orc_problem *P = W->P;
    int myid = R->r;
    int k0 = (myid == 0) ? 0 : R->ks[n + 1];
    prolong_planes(P, n, &R->pr[n], &R->pr[n + 1], k0, R->ke[n + 1]);
    int nx = P->jxc[n], ny = P->jyc[n];
    sync_all(W);
    if (myid > 0) {
        orc_rank *lf = &W->ranks[myid - 1];
        copy_plane(&R->pr[n], R->ks[n], &lf->pr[n], lf->ke[n] + 1, 0, nx, 0, ny);
    }
    sync_all(W);
    sync_all(W);
    if (myid > 0) {
        orc_rank *lf = &W->ranks[myid - 1];
        copy_plane(&R->pr[n], R->ks[n] - 1, &lf->pr[n], lf->ke[n], 0, nx, 0, ny);
    }
    sync_all(W);
}

static void smooth(orc_rank *R, int n, int kss, const arr3 *rh) {
    if (R->W->P->islor) smooth_slor(R, n, kss, rh);
    else smooth_sor(R, n, kss, rh);
}

/* multi, multigrid.f03:42-653, executed by each rank */
static void *multi_rank(void *arg) {
    orc_rank *R = (orc_rank *)arg;
    orc_world *W = R->W;
    orc_problem *P = W->P;
    int nlevel = P->nlevel, myid = R->r, nproc = W->nproc;
    int kss[MAXLEV + 1];
    for (int n = 1; n <= nlevel; n++) kss[n] = n > 1 ? 10 : 5;
    int ktime = 0;
    double resmax = 1., relres = 1.;
    for (;;) {
        int go = ktime < W->ficycle &&
                 (W->stop_mode == 0 ? resmax >= W->eps : relres > W->eps);
        if (!go) break;
        ktime++;
        /* pr1 = fi including ghosts; coarse levels = 0 (:177-212) */
        for (int k = R->ks[1] - 1; k <= R->ke[1] + 1; k++)
            for (int j = 0; j <= P->jy + 1; j++)
                for (int i = 0; i <= P->jx + 1; i++) AT(R->pr[1], i, j, k) = AT(W->fi, i, j, k);
        for (int n = 2; n <= nlevel; n++) memset(R->pr[n].d, 0, sizeof(double) * a3_size(&R->pr[n]));
        /* down-leg (:216-420) */
        for (int n = 1; n <= nlevel; n++) {
            const arr3 *rhn = n == 1 ? &W->rhs : &W->rhsv[n];
            smooth(R, n, kss[n], rhn);
            if (n < nlevel) {
                resid_planes(P, n, &R->pr[n], rhn, &W->rhsn[n], R->ks[n], R->ke[n]);
                restrict_planes(P, n, &W->rhsn[n], &W->rhsv[n + 1], R->ks[n + 1], R->ke[n + 1]);
            } else if (n == 1) {
                resid_planes(P, 1, &R->pr[1], &W->rhs, &W->rhsn[1], R->ks[1], R->ke[1]);
            }
        }
        /* up-leg (:426-563) */
        for (int n = nlevel - 1; n >= 1; n--) {
            prolong_rank(R, n);
            smooth(R, n, kss[n], n == 1 ? &W->rhs : &W->rhsv[n]);
        }
        if (nlevel > 1) resid_planes(P, 1, &R->pr[1], &W->rhs, &W->rhsn[1], R->ks[1], R->ke[1]);
        /* fi = pr1 on this rank's planes (and the global ghost planes) */
        sync_all(W);
        for (int k = R->ks[1]; k <= R->ke[1]; k++)
            for (int j = 0; j <= P->jy + 1; j++)
                for (int i = 0; i <= P->jx + 1; i++) AT(W->fi, i, j, k) = AT(R->pr[1], i, j, k);
        if (myid == 0)
            for (int j = 0; j <= P->jy + 1; j++)
                for (int i = 0; i <= P->jx + 1; i++) AT(W->fi, i, j, 0) = AT(R->pr[1], i, j, 0);
        if (myid == nproc - 1)
            for (int j = 0; j <= P->jy + 1; j++)
                for (int i = 0; i <= P->jx + 1; i++)
                    AT(W->fi, i, j, P->jz + 1) = AT(R->pr[1], i, j, P->jz + 1);
        /* stop test (:595-631) */
        double mx = 0., sq = 0.;
        for (int k = R->ks[1]; k <= R->ke[1]; k++)
            for (int j = 1; j <= P->jy; j++)
                for (int i = 1; i <= P->jx; i++) {
                    double a = fabs(AT(W->rhsn[1], i, j, k));
                    mx = a > mx ? a : mx;
                    sq += a * a;
                }
        W->loc_max[myid] = mx;
        W->loc_sq[myid] = sq;
        sync_all(W);
        resmax = 0.;
        double tot = 0.;
        for (int r = 0; r < nproc; r++) {
            resmax = W->loc_max[r] > resmax ? W->loc_max[r] : resmax;
            tot += W->loc_sq[r];
        }
        relres = sqrt(tot) / W->rhs_norm;
        sync_all(W);
    }
    if (myid == 0) {
        W->cycles = ktime;
        W->resmax = resmax;
        W->relres = relres;
    }
    return NULL;
}

static arr3 wrap2(const double *src, int u0, int u1, int v0, int v1) {
    arr3 a;
    memset(&a, 0, sizeof a);
    if (!src) return a;
    a = a3(u0, u1, v0, v1, 0, 0);
    memcpy(a.d, src, sizeof(double) * (size_t)a3_size(&a));
    return a;
}

static void world_init(orc_world *W, orc_problem *P, int nproc, const double *const cs[6]) {
    memset(W, 0, sizeof *W);
    W->P = P;
    W->nproc = nproc;
    const double *c0[6] = {0, 0, 0, 0, 0, 0};
    if (!cs) cs = c0;
    W->cs1 = wrap2(cs[0], 1, P->jy, 1, P->jz);
    W->cs2 = wrap2(cs[1], 1, P->jy, 1, P->jz);
    W->cs3 = wrap2(cs[2], 1, P->jx, 1, P->jz);
    W->cs4 = wrap2(cs[3], 1, P->jx, 1, P->jz);
    W->cs5 = wrap2(cs[4], 1, P->jx, 1, P->jy);
    W->cs6 = wrap2(cs[5], 1, P->jx, 1, P->jy);
    W->ranks = (orc_rank *)calloc((size_t)nproc, sizeof(orc_rank));
    for (int r = 0; r < nproc; r++) {
        orc_rank *R = &W->ranks[r];
        R->W = W;
        R->r = r;
        for (int n = 1; n <= P->nlevel; n++) {
            int nc = P->jzc[n] / nproc;
            R->ks[n] = r * nc + 1;
            R->ke[n] = (r + 1) * nc;
            R->pr[n] = a3(0, P->jxc[n] + 1, 0, P->jyc[n] + 1, R->ks[n] - 1, R->ke[n] + 1);
        }
    }
    for (int n = 1; n <= P->nlevel; n++) {
        W->rhsv[n] = a3(1, P->jxc[n], 1, P->jyc[n], 1, P->jzc[n]);
        W->rhsn[n] = a3(1, P->jxc[n], 1, P->jyc[n], 1, P->jzc[n]);
    }
    W->loc_max = (double *)calloc((size_t)nproc, sizeof(double));
    W->loc_sq = (double *)calloc((size_t)nproc, sizeof(double));
    if (nproc > 1) pthread_barrier_init(&W->bar, NULL, (unsigned)nproc);
}

static void world_free(orc_world *W) {
    for (int r = 0; r < W->nproc; r++)
        for (int n = 1; n <= W->P->nlevel; n++) a3_free(&W->ranks[r].pr[n]);
    for (int n = 1; n <= W->P->nlevel; n++) {
        a3_free(&W->rhsv[n]);
        a3_free(&W->rhsn[n]);
    }
    a3_free(&W->cs1); a3_free(&W->cs2); a3_free(&W->cs3);
    a3_free(&W->cs4); a3_free(&W->cs5); a3_free(&W->cs6);
    free(W->ranks); free(W->loc_max); free(W->loc_sq);
    if (W->nproc > 1) pthread_barrier_destroy(&W->bar);
}

int orc_multi(orc_problem *p, double *fi, const double *rhs, const double *const cs[6],
              double eps, int ficycle, int stop_mode, int *cycles, double *resmax,
              double *relres) {
    if (!p || !fi || !rhs || ficycle < 0 || (stop_mode != 0 && stop_mode != 1)) {
        set_err("bad argument to orc_multi");
        return -1;
    }
    orc_world W;
    world_init(&W, p, p->nproc, cs);
    W.eps = eps;
    W.ficycle = ficycle;
    W.stop_mode = stop_mode;
    W.fi = a3(0, p->jx + 1, 0, p->jy + 1, 0, p->jz + 1);
    memcpy(W.fi.d, fi, sizeof(double) * (size_t)a3_size(&W.fi));
    W.rhs = a3(1, p->jx, 1, p->jy, 1, p->jz);
    memcpy(W.rhs.d, rhs, sizeof(double) * (size_t)a3_size(&W.rhs));
    double nb = 0.;
    for (long q = 0; q < a3_size(&W.rhs); q++) nb += W.rhs.d[q] * W.rhs.d[q];
    W.rhs_norm = nb > 0. ? sqrt(nb) : 1.;
    if (p->nproc == 1) {
        multi_rank(&W.ranks[0]);
    } else {
        pthread_t *th = (pthread_t *)calloc((size_t)p->nproc, sizeof(pthread_t));
        for (int r = 0; r < p->nproc; r++) pthread_create(&th[r], NULL, multi_rank, &W.ranks[r]);
        for (int r = 0; r < p->nproc; r++) pthread_join(th[r], NULL);
        free(th);
    }
    memcpy(fi, W.fi.d, sizeof(double) * (size_t)a3_size(&W.fi));
    if (cycles) *cycles = W.cycles;
    if (resmax) *resmax = W.resmax;
    if (relres) *relres = W.relres;
    a3_free(&W.fi);
    a3_free(&W.rhs);
    world_free(&W);
    return 0;
}

/* ------------------------------------------------------------------ */
/* Single-level entry points for tests (one domain).                    */
static int level_ok(const orc_problem *p, int n) { return p && n >= 1 && n <= p->nlevel; }

int orc_resid(orc_problem *p, int n, const double *pr, const double *rh, double *out) {
    if (!level_ok(p, n)) return -1;
    int nx = p->jxc[n], ny = p->jyc[n], nz = p->jzc[n];
    arr3 P = a3(0, nx + 1, 0, ny + 1, 0, nz + 1), RH = a3(1, nx, 1, ny, 1, nz), O = a3(1, nx, 1, ny, 1, nz);
    memcpy(P.d, pr, sizeof(double) * a3_size(&P));
    memcpy(RH.d, rh, sizeof(double) * a3_size(&RH));
    resid_planes(p, n, &P, &RH, &O, 1, nz);
    memcpy(out, O.d, sizeof(double) * a3_size(&O));
    a3_free(&P); a3_free(&RH); a3_free(&O);
    return 0;
}

int orc_ghost_fill(orc_problem *p, int n, double *pr, const double *const cs[6]) {
    if (!level_ok(p, n)) return -1;
    orc_world W;
    int saved = p->nproc;
    p->nproc = 1; /* single domain */
    world_init(&W, p, 1, cs);
    arr3 *a = &W.ranks[0].pr[n];
    memcpy(a->d, pr, sizeof(double) * a3_size(a));
    mul_boun(&W.ranks[0], n, p->freesurface);
    memcpy(pr, a->d, sizeof(double) * a3_size(a));
    world_free(&W);
    p->nproc = saved;
    return 0;
}

int orc_restrict(orc_problem *p, int n, const double *rh, double *out) {
    if (!level_ok(p, n) || n + 1 > p->nlevel) return -1;
    arr3 A = a3(1, p->jxc[n], 1, p->jyc[n], 1, p->jzc[n]);
    arr3 B = a3(1, p->jxc[n + 1], 1, p->jyc[n + 1], 1, p->jzc[n + 1]);
    memcpy(A.d, rh, sizeof(double) * a3_size(&A));
    restrict_planes(p, n, &A, &B, 1, p->jzc[n + 1]);
    memcpy(out, B.d, sizeof(double) * a3_size(&B));
    a3_free(&A); a3_free(&B);
    return 0;
}

int orc_prolong(orc_problem *p, int n, double *prf, const double *prc) {
    if (!level_ok(p, n) || n + 1 > p->nlevel) return -1;
    arr3 F = a3(0, p->jxc[n] + 1, 0, p->jyc[n] + 1, 0, p->jzc[n] + 1);
    arr3 C = a3(0, p->jxc[n + 1] + 1, 0, p->jyc[n + 1] + 1, 0, p->jzc[n + 1] + 1);
    memcpy(F.d, prf, sizeof(double) * a3_size(&F));
    memcpy(C.d, prc, sizeof(double) * a3_size(&C));
    prolong_planes(p, n, &F, &C, 0, p->jzc[n + 1]);
    memcpy(prf, F.d, sizeof(double) * a3_size(&F));
    a3_free(&F); a3_free(&C);
    return 0;
}

int orc_true_residual(orc_problem *p, double *fi, const double *rhs, const double *const cs[6],
                      double *out, int maxpass) {
    if (!p) return -1;
    for (int q = 0; q < maxpass; q++)
        if (orc_ghost_fill(p, 1, fi, cs)) return -1;
    return orc_resid(p, 1, fi, rhs, out);
}
