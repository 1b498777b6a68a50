// metric.cu -- face metric of every multigrid level, computed on the device
// in FP64 from the fine node coordinates.
//
// A level uses the fine nodes sub-sampled with strides (sx,sy,sz):
//   all 1                 : metrica, fsrc/metrica.f03:85-419
//   sx = sy = sz = 2^(n-1): mul_met, fsrc/multigrid.f03:2520-2988, divided
//                           by pot = 2^(n-1) (inv_div = 1/pot)
//   other strides         : the same formulas along each direction with its
//                           own stride (semi-coarsened levels),
// with the contravariant rows of gprima/gseconda/gterza.f03.  Ghost nodes
// outside [0,jx] x [0,jz] follow cellep.f03:29-99 (periodic shift by the
// domain length along x and z), evaluated on the fly, so any stride whose
// shift stays inside one period works (more than the reference's 8 ghost
// layers).  This file is compiled with -fmad=false: every product and sum is
// rounded as written, matching the CPU restatement bit for bit.
#include <cuda_runtime.h>

#include "mg_device.cuh"
#include "metric.h"

namespace ples {

struct Nodes {
    const double *x, *y, *z;  // (0:jx, 0:jy, 0:jz), i fastest
    int jx, jy, jz;
    int ip, jp, kp;
    __device__ __forceinline__ long long id(int a, int b, int c) const {
        return ((long long)c * (jy + 1) + b) * (jx + 1) + a;
    }
    // cellep.f03:29-40 (x), 77-99 (z); z-ghosts copy x-ghosted planes
    __device__ double X(int a, int b, int c) const {
        if (c < 0) c += jz;
        else if (c > jz) c -= jz;
        if (a < 0) return x[id(0, b, c)] - (x[id(jx, b, c)] - x[id(jx + a, b, c)]);
        if (a > jx) return x[id(jx, b, c)] - (x[id(0, b, c)] - x[id(a - jx, b, c)]);
        return x[id(a, b, c)];
    }
    __device__ double Y(int a, int b, int c) const {
        if (c < 0) c += jz;
        else if (c > jz) c -= jz;
        if (a < 0) a += jx;
        else if (a > jx) a -= jx;
        return y[id(a, b, c)];
    }
    __device__ double Zw(int a, int b, int c) const {  // x-wrapped z, c in range
        if (a < 0) a += jx;
        else if (a > jx) a -= jx;
        return z[id(a, b, c)];
    }
    __device__ double Z(int a, int b, int c) const {
        if (c < 0) return Zw(a, b, 0) - (Zw(a, b, jz) - Zw(a, b, jz + c));
        if (c > jz) return Zw(a, b, jz) - (Zw(a, b, 0) - Zw(a, b, c - jz));
        return Zw(a, b, c);
    }
};

__device__ __forceinline__ double jac(double xcsi, double ycsi, double zcsi, double xeta, double yeta,
                                      double zeta, double xzet, double yzet, double zzet) {
    return xcsi * (yeta * zzet - yzet * zeta) - xeta * (ycsi * zzet - yzet * zcsi) +
           xzet * (ycsi * zeta - yeta * zcsi);
}

// row `row` (0: gprima, 1: gseconda, 2: gterza) of the contravariant metric / J
__device__ void metric_row(int row, double xcsi, double ycsi, double zcsi, double xeta, double yeta,
                           double zeta, double xzet, double yzet, double zzet, double t[3]) {
    const double giac = jac(xcsi, ycsi, zcsi, xeta, yeta, zeta, xzet, yzet, zzet);
    const double csx = yeta * zzet - yzet * zeta;
    const double csy = xzet * zeta - xeta * zzet;
    const double csz = xeta * yzet - xzet * yeta;
    const double etx = yzet * zcsi - ycsi * zzet;
    const double ety = xcsi * zzet - xzet * zcsi;
    const double etz = xzet * ycsi - xcsi * yzet;
    const double ztx = ycsi * zeta - yeta * zcsi;
    const double zty = xeta * zcsi - xcsi * zeta;
    const double ztz = xcsi * yeta - xeta * ycsi;
    if (row == 0) {
        t[0] = (csx * csx + csy * csy + csz * csz) / giac;
        t[1] = (csx * etx + csy * ety + csz * etz) / giac;
        t[2] = (csx * ztx + csy * zty + csz * ztz) / giac;
    } else if (row == 1) {
        t[0] = (etx * csx + ety * csy + etz * csz) / giac;
        t[1] = (etx * etx + ety * ety + etz * etz) / giac;
        t[2] = (etx * ztx + ety * zty + etz * ztz) / giac;
    } else {
        t[0] = (ztx * csx + zty * csy + ztz * csz) / giac;
        t[1] = (ztx * etx + zty * ety + ztz * etz) / giac;
        t[2] = (ztx * ztx + zty * zty + ztz * ztz) / giac;
    }
}

#define AVG_I(F, a, b1, b2, c1, c2) (.25 * (N.F(a, b2, c2) + N.F(a, b2, c1) + N.F(a, b1, c2) + N.F(a, b1, c1)))
#define AVG_J(F, a1, a2, b, c1, c2) (.25 * (N.F(a2, b, c2) + N.F(a2, b, c1) + N.F(a1, b, c1) + N.F(a1, b, c2)))
#define AVG_K(F, a1, a2, b1, b2, c) (.25 * (N.F(a2, b2, c) + N.F(a2, b1, c) + N.F(a1, b1, c) + N.F(a1, b2, c)))

// csi faces i = 0..nx (multigrid.f03:2520-2666 / metrica.f03:85-197)
__global__ void k_metric_csi(Nodes N, Geom g, int sx, int sy, int sz, double inv_pot, double* g11, double* g12,
                             double* g13, double* nx_, double* ny_, double* nz_) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z + 1;
    if (i > g.nx || j > g.ny) return;
    const int j2 = j * sy, j1 = (j - 1) * sy, k2 = k * sz, k1 = (k - 1) * sz, ic = i * sx;
    double xcsi, ycsi, zcsi;
    if (i == 0 && N.ip == 1) {
        const int i1 = sx, i2 = 2 * sx;
        double x2 = AVG_I(X, i2, j1, j2, k1, k2), x1 = AVG_I(X, i1, j1, j2, k1, k2), x0 = AVG_I(X, 0, j1, j2, k1, k2);
        double y2 = AVG_I(Y, i2, j1, j2, k1, k2), y1 = AVG_I(Y, i1, j1, j2, k1, k2), y0 = AVG_I(Y, 0, j1, j2, k1, k2);
        double z2 = AVG_I(Z, i2, j1, j2, k1, k2), z1 = AVG_I(Z, i1, j1, j2, k1, k2), z0 = AVG_I(Z, 0, j1, j2, k1, k2);
        xcsi = .5 * (-3. * x0 + 4. * x1 - x2);
        ycsi = .5 * (-3. * y0 + 4. * y1 - y2);
        zcsi = .5 * (-3. * z0 + 4. * z1 - z2);
    } else if (i == g.nx && N.ip == 1) {
        const int i1 = (i - 1) * sx, i2 = (i - 2) * sx, ie = N.jx;
        double x2 = AVG_I(X, i2, j1, j2, k1, k2), x1 = AVG_I(X, i1, j1, j2, k1, k2), x0 = AVG_I(X, ie, j1, j2, k1, k2);
        double y2 = AVG_I(Y, i2, j1, j2, k1, k2), y1 = AVG_I(Y, i1, j1, j2, k1, k2), y0 = AVG_I(Y, ie, j1, j2, k1, k2);
        double z2 = AVG_I(Z, i2, j1, j2, k1, k2), z1 = AVG_I(Z, i1, j1, j2, k1, k2), z0 = AVG_I(Z, ie, j1, j2, k1, k2);
        xcsi = .5 * (3. * x0 - 4. * x1 + x2);
        ycsi = .5 * (3. * y0 - 4. * y1 + y2);
        zcsi = .5 * (3. * z0 - 4. * z1 + z2);
    } else {
        const int i2 = (i + 1) * sx, i1 = (i - 1) * sx;
        double xdx = AVG_I(X, i2, j1, j2, k1, k2), xsn = AVG_I(X, i1, j1, j2, k1, k2);
        double ydx = AVG_I(Y, i2, j1, j2, k1, k2), ysn = AVG_I(Y, i1, j1, j2, k1, k2);
        double zdx = AVG_I(Z, i2, j1, j2, k1, k2), zsn = AVG_I(Z, i1, j1, j2, k1, k2);
        xcsi = .5 * (xdx - xsn);
        ycsi = .5 * (ydx - ysn);
        zcsi = .5 * (zdx - zsn);
    }
    const double xeta = .5 * (N.X(ic, j2, k2) + N.X(ic, j2, k1)) - .5 * (N.X(ic, j1, k2) + N.X(ic, j1, k1));
    const double yeta = .5 * (N.Y(ic, j2, k2) + N.Y(ic, j2, k1)) - .5 * (N.Y(ic, j1, k2) + N.Y(ic, j1, k1));
    const double zeta = .5 * (N.Z(ic, j2, k2) + N.Z(ic, j2, k1)) - .5 * (N.Z(ic, j1, k2) + N.Z(ic, j1, k1));
    const double xzet = .5 * (N.X(ic, j2, k2) + N.X(ic, j1, k2)) - .5 * (N.X(ic, j2, k1) + N.X(ic, j1, k1));
    const double yzet = .5 * (N.Y(ic, j2, k2) + N.Y(ic, j1, k2)) - .5 * (N.Y(ic, j2, k1) + N.Y(ic, j1, k1));
    const double zzet = .5 * (N.Z(ic, j2, k2) + N.Z(ic, j1, k2)) - .5 * (N.Z(ic, j2, k1) + N.Z(ic, j1, k1));
    const long long q = g.at(i, j, k);
    if (nx_) {  // J(-1) grad(csi) on the face: csx, csy, csz (metrica.f03:158-160)
        nx_[q] = yeta * zzet - yzet * zeta;
        ny_[q] = xzet * zeta - xeta * zzet;
        nz_[q] = xeta * yzet - xzet * yeta;
    }
    if (!g11) return;
    double t[3];
    metric_row(0, xcsi, ycsi, zcsi, xeta, yeta, zeta, xzet, yzet, zzet, t);
    if (sx == 1 && sy == 1 && sz == 1) {
        g11[q] = t[0]; g12[q] = t[1]; g13[q] = t[2];
    } else {
        g11[q] = t[0] * inv_pot; g12[q] = t[1] * inv_pot; g13[q] = t[2] * inv_pot;
    }
}

// eta faces j = 0..ny (multigrid.f03:2675-2827 / metrica.f03:203-294)
__global__ void k_metric_eta(Nodes N, Geom g, int sx, int sy, int sz, double inv_pot, double* g21, double* g22,
                             double* g23, double* nx_, double* ny_, double* nz_) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z + 1;
    if (i > g.nx || j > g.ny) return;
    const int i2 = i * sx, i1 = (i - 1) * sx, k2 = k * sz, k1 = (k - 1) * sz, jc = j * sy;
    double xeta, yeta, zeta;
    if (j == 0 && N.jp == 1) {
        const int j1 = sy, j2 = 2 * sy;
        double x2 = AVG_J(X, i1, i2, j2, k1, k2), x1 = AVG_J(X, i1, i2, j1, k1, k2), x0 = AVG_J(X, i1, i2, 0, k1, k2);
        double y2 = AVG_J(Y, i1, i2, j2, k1, k2), y1 = AVG_J(Y, i1, i2, j1, k1, k2), y0 = AVG_J(Y, i1, i2, 0, k1, k2);
        double z2 = AVG_J(Z, i1, i2, j2, k1, k2), z1 = AVG_J(Z, i1, i2, j1, k1, k2), z0 = AVG_J(Z, i1, i2, 0, k1, k2);
        xeta = .5 * (-3. * x0 + 4. * x1 - x2);
        yeta = .5 * (-3. * y0 + 4. * y1 - y2);
        zeta = .5 * (-3. * z0 + 4. * z1 - z2);
    } else if (j == g.ny && N.jp == 1) {
        const int j1 = (j - 1) * sy, j2 = (j - 2) * sy, je = N.jy;
        double x2 = AVG_J(X, i1, i2, j2, k1, k2), x1 = AVG_J(X, i1, i2, j1, k1, k2), x0 = AVG_J(X, i1, i2, je, k1, k2);
        double y2 = AVG_J(Y, i1, i2, j2, k1, k2), y1 = AVG_J(Y, i1, i2, j1, k1, k2), y0 = AVG_J(Y, i1, i2, je, k1, k2);
        double z2 = AVG_J(Z, i1, i2, j2, k1, k2), z1 = AVG_J(Z, i1, i2, j1, k1, k2), z0 = AVG_J(Z, i1, i2, je, k1, k2);
        xeta = .5 * (3. * x0 - 4. * x1 + x2);
        yeta = .5 * (3. * y0 - 4. * y1 + y2);
        zeta = .5 * (3. * z0 - 4. * z1 + z2);
    } else {
        const int j2 = (j + 1) * sy, j1 = (j - 1) * sy;
        double xsop = AVG_J(X, i1, i2, j2, k1, k2), xsot = AVG_J(X, i1, i2, j1, k1, k2);
        double ysop = AVG_J(Y, i1, i2, j2, k1, k2), ysot = AVG_J(Y, i1, i2, j1, k1, k2);
        double zsop = AVG_J(Z, i1, i2, j2, k1, k2), zsot = AVG_J(Z, i1, i2, j1, k1, k2);
        xeta = .5 * (xsop - xsot);
        yeta = .5 * (ysop - ysot);
        zeta = .5 * (zsop - zsot);
    }
    const double yzet = .5 * (N.Y(i2, jc, k2) + N.Y(i1, jc, k2)) - .5 * (N.Y(i2, jc, k1) + N.Y(i1, jc, k1));
    const double zcsi = .5 * (N.Z(i2, jc, k2) + N.Z(i2, jc, k1)) - .5 * (N.Z(i1, jc, k2) + N.Z(i1, jc, k1));
    const double ycsi = .5 * (N.Y(i2, jc, k2) + N.Y(i2, jc, k1)) - .5 * (N.Y(i1, jc, k2) + N.Y(i1, jc, k1));
    const double zzet = .5 * (N.Z(i2, jc, k2) + N.Z(i1, jc, k2)) - .5 * (N.Z(i2, jc, k1) + N.Z(i1, jc, k1));
    const double xcsi = .5 * (N.X(i2, jc, k2) + N.X(i2, jc, k1)) - .5 * (N.X(i1, jc, k2) + N.X(i1, jc, k1));
    const double xzet = .5 * (N.X(i2, jc, k2) + N.X(i1, jc, k2)) - .5 * (N.X(i2, jc, k1) + N.X(i1, jc, k1));
    const long long q = g.at(i, j, k);
    if (nx_) {  // etx, ety, etz (metrica.f03:272-274)
        nx_[q] = yzet * zcsi - ycsi * zzet;
        ny_[q] = xcsi * zzet - xzet * zcsi;
        nz_[q] = xzet * ycsi - xcsi * yzet;
    }
    if (!g21) return;
    double t[3];
    metric_row(1, xcsi, ycsi, zcsi, xeta, yeta, zeta, xzet, yzet, zzet, t);
    if (sx == 1 && sy == 1 && sz == 1) {
        g21[q] = t[0]; g22[q] = t[1]; g23[q] = t[2];
    } else {
        g21[q] = t[0] * inv_pot; g22[q] = t[1] * inv_pot; g23[q] = t[2] * inv_pot;
    }
}

// zeta faces k = 0..nz (multigrid.f03:2836-2988 / metrica.f03:316-419)
__global__ void k_metric_zet(Nodes N, Geom g, int sx, int sy, int sz, double inv_pot, double* g31, double* g32,
                             double* g33, double* nx_, double* ny_, double* nz_) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z;
    if (i > g.nx || j > g.ny) return;
    const int i2 = i * sx, i1 = (i - 1) * sx, j2 = j * sy, j1 = (j - 1) * sy, kc = k * sz;
    double xzet, yzet, zzet;
    if (k == 0 && N.kp == 1) {
        const int k1 = sz, k2 = 2 * sz;
        double x2 = AVG_K(X, i1, i2, j1, j2, k2), x1 = AVG_K(X, i1, i2, j1, j2, k1), x0 = AVG_K(X, i1, i2, j1, j2, 0);
        double y2 = AVG_K(Y, i1, i2, j1, j2, k2), y1 = AVG_K(Y, i1, i2, j1, j2, k1), y0 = AVG_K(Y, i1, i2, j1, j2, 0);
        double z2 = AVG_K(Z, i1, i2, j1, j2, k2), z1 = AVG_K(Z, i1, i2, j1, j2, k1), z0 = AVG_K(Z, i1, i2, j1, j2, 0);
        xzet = .5 * (-3. * x0 + 4. * x1 - x2);
        yzet = .5 * (-3. * y0 + 4. * y1 - y2);
        zzet = .5 * (-3. * z0 + 4. * z1 - z2);
    } else if (k == g.nz && N.kp == 1) {
        const int k1 = (k - 1) * sz, k2 = (k - 2) * sz, ke = N.jz;
        double x2 = AVG_K(X, i1, i2, j1, j2, k2), x1 = AVG_K(X, i1, i2, j1, j2, k1), x0 = AVG_K(X, i1, i2, j1, j2, ke);
        double y2 = AVG_K(Y, i1, i2, j1, j2, k2), y1 = AVG_K(Y, i1, i2, j1, j2, k1), y0 = AVG_K(Y, i1, i2, j1, j2, ke);
        double z2 = AVG_K(Z, i1, i2, j1, j2, k2), z1 = AVG_K(Z, i1, i2, j1, j2, k1), z0 = AVG_K(Z, i1, i2, j1, j2, ke);
        xzet = .5 * (3. * x0 - 4. * x1 + x2);
        yzet = .5 * (3. * y0 - 4. * y1 + y2);
        zzet = .5 * (3. * z0 - 4. * z1 + z2);
    } else {
        const int k2 = (k + 1) * sz, k1 = (k - 1) * sz;
        double xav = AVG_K(X, i1, i2, j1, j2, k2), xdt = AVG_K(X, i1, i2, j1, j2, k1);
        double yav = AVG_K(Y, i1, i2, j1, j2, k2), ydt = AVG_K(Y, i1, i2, j1, j2, k1);
        double zav = AVG_K(Z, i1, i2, j1, j2, k2), zdt = AVG_K(Z, i1, i2, j1, j2, k1);
        xzet = .5 * (xav - xdt);
        yzet = .5 * (yav - ydt);
        zzet = .5 * (zav - zdt);
    }
    const double ycsi = .5 * (N.Y(i2, j2, kc) + N.Y(i2, j1, kc)) - .5 * (N.Y(i1, j2, kc) + N.Y(i1, j1, kc));
    const double zeta = .5 * (N.Z(i2, j2, kc) + N.Z(i1, j2, kc)) - .5 * (N.Z(i2, j1, kc) + N.Z(i1, j1, kc));
    const double yeta = .5 * (N.Y(i2, j2, kc) + N.Y(i1, j2, kc)) - .5 * (N.Y(i2, j1, kc) + N.Y(i1, j1, kc));
    const double zcsi = .5 * (N.Z(i2, j2, kc) + N.Z(i2, j1, kc)) - .5 * (N.Z(i1, j2, kc) + N.Z(i1, j1, kc));
    const double xcsi = .5 * (N.X(i2, j2, kc) + N.X(i2, j1, kc)) - .5 * (N.X(i1, j2, kc) + N.X(i1, j1, kc));
    const double xeta = .5 * (N.X(i2, j2, kc) + N.X(i1, j2, kc)) - .5 * (N.X(i2, j1, kc) + N.X(i1, j1, kc));
    const long long q = g.at(i, j, k);
    if (nx_) {  // ztx, zty, ztz (the zeta-face normals of metrica.f03)
        nx_[q] = ycsi * zeta - yeta * zcsi;
        ny_[q] = xeta * zcsi - xcsi * zeta;
        nz_[q] = xcsi * yeta - xeta * ycsi;
    }
    if (!g31) return;
    double t[3];
    metric_row(2, xcsi, ycsi, zcsi, xeta, yeta, zeta, xzet, yzet, zzet, t);
    if (sx == 1 && sy == 1 && sz == 1) {
        g31[q] = t[0]; g32[q] = t[1]; g33[q] = t[2];
    } else {
        g31[q] = t[0] * inv_pot; g32[q] = t[1] * inv_pot; g33[q] = t[2] * inv_pot;
    }
}

cudaError_t launch_metric(const double* xn, const double* yn, const double* zn, int jx, int jy, int jz,
                          int ip, int jp, int kp, int sx, int sy, int sz, double inv_div, Geom g,
                          double* const gout[9], cudaStream_t st) {
    Nodes N{xn, yn, zn, jx, jy, jz, ip, jp, kp};
    dim3 blk(32, 4);
    k_metric_csi<<<dim3((g.nx + 1 + 31) / 32, (g.ny + 3) / 4, g.nz), blk, 0, st>>>(
        N, g, sx, sy, sz, inv_div, gout[0], gout[1], gout[2], nullptr, nullptr, nullptr);
    k_metric_eta<<<dim3((g.nx + 31) / 32, (g.ny + 1 + 3) / 4, g.nz), blk, 0, st>>>(
        N, g, sx, sy, sz, inv_div, gout[3], gout[4], gout[5], nullptr, nullptr, nullptr);
    k_metric_zet<<<dim3((g.nx + 31) / 32, (g.ny + 3) / 4, g.nz + 1), blk, 0, st>>>(
        N, g, sx, sy, sz, inv_div, gout[6], gout[7], gout[8], nullptr, nullptr, nullptr);
    return cudaGetLastError();
}

// Cell Jacobian J of the fine grid at cell centres, from the averaged node
// differences of the cell (metrica's giac; the oracle's build_giac).
__global__ void k_giac(Nodes N, Geom g, double* __restrict__ giac) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z + 1;
    if (i > g.nx || j > g.ny) return;
#define C4(F, a, b, c, d) (.25 * (N.F a + N.F b + N.F c + N.F d))
    const double xcsi = C4(X, (i, j, k), (i, j, k - 1), (i, j - 1, k - 1), (i, j - 1, k)) -
                        C4(X, (i - 1, j, k), (i - 1, j, k - 1), (i - 1, j - 1, k - 1), (i - 1, j - 1, k));
    const double ycsi = C4(Y, (i, j, k), (i, j, k - 1), (i, j - 1, k - 1), (i, j - 1, k)) -
                        C4(Y, (i - 1, j, k), (i - 1, j, k - 1), (i - 1, j - 1, k - 1), (i - 1, j - 1, k));
    const double zcsi = C4(Z, (i, j, k), (i, j, k - 1), (i, j - 1, k - 1), (i, j - 1, k)) -
                        C4(Z, (i - 1, j, k), (i - 1, j, k - 1), (i - 1, j - 1, k - 1), (i - 1, j - 1, k));
    const double xeta = C4(X, (i, j, k), (i, j, k - 1), (i - 1, j, k - 1), (i - 1, j, k)) -
                        C4(X, (i, j - 1, k), (i, j - 1, k - 1), (i - 1, j - 1, k - 1), (i - 1, j - 1, k));
    const double yeta = C4(Y, (i, j, k), (i, j, k - 1), (i - 1, j, k - 1), (i - 1, j, k)) -
                        C4(Y, (i, j - 1, k), (i, j - 1, k - 1), (i - 1, j - 1, k - 1), (i - 1, j - 1, k));
    const double zeta = C4(Z, (i, j, k), (i, j, k - 1), (i - 1, j, k - 1), (i - 1, j, k)) -
                        C4(Z, (i, j - 1, k), (i, j - 1, k - 1), (i - 1, j - 1, k - 1), (i - 1, j - 1, k));
    const double xzet = C4(X, (i, j, k), (i, j - 1, k), (i - 1, j - 1, k), (i - 1, j, k)) -
                        C4(X, (i, j, k - 1), (i, j - 1, k - 1), (i - 1, j - 1, k - 1), (i - 1, j, k - 1));
    const double yzet = C4(Y, (i, j, k), (i, j - 1, k), (i - 1, j - 1, k), (i - 1, j, k)) -
                        C4(Y, (i, j, k - 1), (i, j - 1, k - 1), (i - 1, j - 1, k - 1), (i - 1, j, k - 1));
    const double zzet = C4(Z, (i, j, k), (i, j - 1, k), (i - 1, j - 1, k), (i - 1, j, k)) -
                        C4(Z, (i, j, k - 1), (i, j - 1, k - 1), (i - 1, j - 1, k - 1), (i - 1, j, k - 1));
#undef C4
    giac[g.at(i, j, k)] = jac(xcsi, ycsi, zcsi, xeta, yeta, zeta, xzet, yzet, zzet);
}

cudaError_t launch_normals(const double* xn, const double* yn, const double* zn, int jx, int jy, int jz, int ip,
                           int jp, int kp, Geom g, double* const nout[9], double* giac, cudaStream_t st) {
    Nodes N{xn, yn, zn, jx, jy, jz, ip, jp, kp};
    dim3 blk(32, 4);
    k_metric_csi<<<dim3((g.nx + 1 + 31) / 32, (g.ny + 3) / 4, g.nz), blk, 0, st>>>(
        N, g, 1, 1, 1, 1.0, nullptr, nullptr, nullptr, nout[0], nout[1], nout[2]);
    k_metric_eta<<<dim3((g.nx + 31) / 32, (g.ny + 1 + 3) / 4, g.nz), blk, 0, st>>>(
        N, g, 1, 1, 1, 1.0, nullptr, nullptr, nullptr, nout[3], nout[4], nout[5]);
    k_metric_zet<<<dim3((g.nx + 31) / 32, (g.ny + 3) / 4, g.nz + 1), blk, 0, st>>>(
        N, g, 1, 1, 1, 1.0, nullptr, nullptr, nullptr, nout[6], nout[7], nout[8]);
    k_giac<<<dim3((g.nx + 31) / 32, (g.ny + 3) / 4, g.nz), blk, 0, st>>>(N, g, giac);
    return cudaGetLastError();
}

}  // namespace ples
