/*
 * abi_check.c -- a C caller of libples_mg.so compiled against
 * include/ples_mg.h, as a binding outside Python would be (test
 * infrastructure, built and run by tests/test_abi_c.py).
 *
 *   abi_check layout : the header's structures against the library's own
 *                      layout (ples_mg_abi_layout): version, sizes and the
 *                      offset of every field; then, without a GPU, that
 *                      ples_mg_create reports PLES_MG_NO_DEVICE
 *   abi_check solve  : one solve on Fortran-layout arrays built here: node
 *                      coordinates (0:jx,0:jy,0:jz) of a sheared channel,
 *                      fi (0:jx+1,0:jy+1,0:jz+1) zero, rhs (1:jx,1:jy,1:jz)
 *                      the divergence of a face-flux field; checks the
 *                      status, ||r||/||b|| <= 1e-10 and that fi came back
 *                      with zero mean over the interior
 * Prints one line per check and exits non-zero on the first failure.
 */
#include <math.h>
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "ples_mg.h"

static int fails = 0;

static void expect(int ok, const char *what, long long got, long long want) {
    printf("%s %s: %lld (want %lld)\n", ok ? "ok  " : "FAIL", what, got, want);
    if (!ok) fails++;
}

static int layout(void) {
    int version = -1;
    long long dsize = 0, ssize = 0, doff[PLES_MG_DESC_FIELDS], soff[PLES_MG_STATS_FIELDS];
    if (ples_mg_abi_layout(&version, &dsize, &ssize, doff, soff) != PLES_MG_OK) return 1;
    const long long mine_d[PLES_MG_DESC_FIELDS] = {
        offsetof(ples_mg_desc, jx), offsetof(ples_mg_desc, jy), offsetof(ples_mg_desc, jz),
        offsetof(ples_mg_desc, ip), offsetof(ples_mg_desc, jp), offsetof(ples_mg_desc, kp),
        offsetof(ples_mg_desc, nlevmax), offsetof(ples_mg_desc, omega), offsetof(ples_mg_desc, precision),
        offsetof(ples_mg_desc, coords_layout), offsetof(ples_mg_desc, x), offsetof(ples_mg_desc, y),
        offsetof(ples_mg_desc, z), offsetof(ples_mg_desc, dt), offsetof(ples_mg_desc, device),
        offsetof(ples_mg_desc, nu_pre), offsetof(ples_mg_desc, nu_post), offsetof(ples_mg_desc, nu_coarse),
        offsetof(ples_mg_desc, inner_cycles), offsetof(ples_mg_desc, smoother), offsetof(ples_mg_desc, coarsening),
        offsetof(ples_mg_desc, solid), offsetof(ples_mg_desc, tipo), offsetof(ples_mg_desc, freesurface)};
    const long long mine_s[PLES_MG_STATS_FIELDS] = {
        offsetof(ples_mg_stats, outer_iterations), offsetof(ples_mg_stats, vcycles),
        offsetof(ples_mg_stats, rel_residual), offsetof(ples_mg_stats, max_residual),
        offsetof(ples_mg_stats, rhs_norm), offsetof(ples_mg_stats, rhs_mean_removed),
        offsetof(ples_mg_stats, seconds), offsetof(ples_mg_stats, status)};
    expect(version == PLES_MG_ABI_VERSION, "abi version", version, PLES_MG_ABI_VERSION);
    expect(dsize == (long long)sizeof(ples_mg_desc), "sizeof(ples_mg_desc)", dsize, (long long)sizeof(ples_mg_desc));
    expect(ssize == (long long)sizeof(ples_mg_stats), "sizeof(ples_mg_stats)", ssize,
           (long long)sizeof(ples_mg_stats));
    char what[64];
    for (int f = 0; f < PLES_MG_DESC_FIELDS; ++f) {
        snprintf(what, sizeof what, "ples_mg_desc field %d offset", f);
        expect(doff[f] == mine_d[f], what, doff[f], mine_d[f]);
    }
    for (int f = 0; f < PLES_MG_STATS_FIELDS; ++f) {
        snprintf(what, sizeof what, "ples_mg_stats field %d offset", f);
        expect(soff[f] == mine_s[f], what, soff[f], mine_s[f]);
    }
    return fails;
}

/* deterministic pseudo-random numbers in [-1, 1) (a 64-bit LCG) */
static double rnd(unsigned long long *s) {
    *s = *s * 6364136223846793005ULL + 1442695040888963407ULL;
    return (double)(*s >> 11) / (double)(1ULL << 52) - 1.0;
}

static int solve(int expect_device) {
    const int jx = 32, jy = 16, jz = 32;
    const double pi = 3.14159265358979323846;
    const size_t nn = (size_t)(jx + 1) * (jy + 1) * (jz + 1);
    double *x = malloc(nn * sizeof *x), *y = malloc(nn * sizeof *y), *z = malloc(nn * sizeof *z);
    /* nodes: x, z uniform and periodic, y stretched over a wavy bottom wall */
    for (int k = 0; k <= jz; ++k)
        for (int j = 0; j <= jy; ++j)
            for (int i = 0; i <= jx; ++i) {
                const size_t q = ((size_t)k * (jy + 1) + j) * (jx + 1) + i;
                const double xs = 2.0 * pi * i / jx, zs = pi * k / jz, eta = (double)j / jy;
                const double y0 = 0.05 * sin(2.0 * xs) * cos(2.0 * zs);
                const double s = 0.5 * (1.0 + tanh(2.0 * (2.0 * eta - 1.0)) / tanh(2.0));
                x[q] = xs;
                z[q] = zs;
                y[q] = y0 + (2.0 - y0) * s;
            }
    /* rhs: divergence of face fluxes (periodic in x and z, zero at the walls) */
    const size_t nr = (size_t)jx * jy * jz, nf = (size_t)(jx + 2) * (jy + 2) * (jz + 2);
    double *uc = malloc(nr * sizeof *uc), *vc = calloc((size_t)jx * (jy + 1) * jz, sizeof *vc),
           *wc = malloc(nr * sizeof *wc), *rhs = malloc(nr * sizeof *rhs), *fi = calloc(nf, sizeof *fi);
    unsigned long long seed = 12345;
    for (size_t q = 0; q < nr; ++q) uc[q] = rnd(&seed);
    for (int k = 0; k < jz; ++k)
        for (int j = 1; j < jy; ++j)
            for (int i = 0; i < jx; ++i) vc[((size_t)k * (jy + 1) + j) * jx + i] = rnd(&seed);
    for (size_t q = 0; q < nr; ++q) wc[q] = rnd(&seed);
    double mean = 0.0;
    for (int k = 0; k < jz; ++k)
        for (int j = 0; j < jy; ++j)
            for (int i = 0; i < jx; ++i) {
                const size_t q = ((size_t)k * jy + j) * jx + i;
                const size_t qw = ((size_t)k * jy + j) * jx + (i + jx - 1) % jx;
                const size_t qb = ((size_t)((k + jz - 1) % jz) * jy + j) * jx + i;
                const double dv = vc[((size_t)k * (jy + 1) + j + 1) * jx + i] - vc[((size_t)k * (jy + 1) + j) * jx + i];
                rhs[q] = (uc[q] - uc[qw]) + dv + (wc[q] - wc[qb]);
                mean += rhs[q];
            }
    mean /= (double)nr;
    for (size_t q = 0; q < nr; ++q) rhs[q] -= mean;

    ples_mg_desc d;
    memset(&d, 0, sizeof d);
    d.jx = jx; d.jy = jy; d.jz = jz;
    d.ip = 0; d.jp = 1; d.kp = 0;
    d.precision = PLES_MG_PREC_MIXED;
    d.coords_layout = PLES_MG_COORDS_NODES;
    d.x = x; d.y = y; d.z = z;
    d.dt = 1.0;
    ples_mg_handle *h = NULL;
    int rc = ples_mg_create(&d, &h);
    if (!expect_device) {
        expect(rc == PLES_MG_NO_DEVICE && h == NULL, "create without a GPU", rc, PLES_MG_NO_DEVICE);
        return fails;
    }
    expect(rc == PLES_MG_OK, "ples_mg_create", rc, PLES_MG_OK);
    if (rc) return fails;
    ples_mg_stats st;
    rc = ples_mg_solve(h, fi, rhs, NULL, 1e-10, 0.0, 100, &st);
    expect(rc == PLES_MG_OK, "ples_mg_solve", rc, PLES_MG_OK);
    expect(st.status == PLES_MG_OK, "stats.status", st.status, PLES_MG_OK);
    printf("%s rel_residual %.3e (want <= 1e-10), %d outer iterations, %d V-cycles\n",
           st.rel_residual <= 1e-10 ? "ok  " : "FAIL", st.rel_residual, st.outer_iterations, st.vcycles);
    if (!(st.rel_residual <= 1e-10)) fails++;
    double s = 0.0, a = 0.0;
    for (int k = 1; k <= jz; ++k)
        for (int j = 1; j <= jy; ++j)
            for (int i = 1; i <= jx; ++i) {
                const double v = fi[((size_t)k * (jy + 2) + j) * (jx + 2) + i];
                s += v;
                a += fabs(v);
            }
    printf("%s interior mean %.3e of mean |fi| %.3e\n", fabs(s) <= 1e-12 * a ? "ok  " : "FAIL", s / (double)nr,
           a / (double)nr);
    if (!(fabs(s) <= 1e-12 * a) || !(a > 0.0)) fails++;
    ples_mg_destroy(h);
    free(x); free(y); free(z); free(uc); free(vc); free(wc); free(rhs); free(fi);
    return fails;
}

int main(int argc, char **argv) {
    if (argc < 2) {
        fprintf(stderr, "usage: abi_check layout|solve|nodevice\n");
        return 2;
    }
    if (!strcmp(argv[1], "layout")) return layout() ? 1 : 0;
    if (!strcmp(argv[1], "nodevice")) return solve(0) ? 1 : 0;
    if (!strcmp(argv[1], "solve")) return (layout() || solve(1)) ? 1 : 0;
    return 2;
}
