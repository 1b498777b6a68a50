// mg_device.cuh -- device-side layout and stencil kernels of the GB300
// pressure-Poisson multigrid.
//
// Layout in HBM.  Every per-level field (pressure, right-hand side, each of
// the nine face-coefficient arrays) lives in one "ghosted box": cells
// (i,j,k), i in [0,nx+1], j in [0,ny+1], k in [0,nz+1], i fastest, with the
// row start padded so that i = 1 sits on a 128-byte boundary (FP32) /
// 256-byte boundary (FP64).  Face coefficients are stored at the index of the
// cell on their low side: csi-face i at (i,j,k) for i in [0,nx], eta-face j
// at (i,j,k) for j in [0,ny], zeta-face k at (i,j,k) for k in [0,nz].  One
// index therefore serves all twelve arrays of a cell.
//
// Scaled coefficients.  The reference applies 1/pot to each face flux and
// again to their sum (ppot1 twice, fsrc/resid_sndrcv.f03:85-151) and 0.25 to
// the cross terms.  Both factors are powers of two, so they are folded into
// the stored coefficients exactly:
//   A1 = g11*ppot2,  B12 = g12*ppot2/4,  B13 = g13*ppot2/4   (csi faces)
//   A2 = g22*ppot2,  B21 = g21*ppot2/4,  B23 = g23*ppot2/4   (eta faces)
//   A3 = g33*ppot2,  B31 = g31*ppot2/4,  B32 = g32*ppot2/4   (zeta faces)
// with ppot2 = 4^-(n-1).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace ples {

constexpr int kOX = 31;  // element offset of i = 0 inside a row

struct Geom {
    int nx, ny, nz;
    int sj;          // row pitch (elements)
    long long sk;    // plane pitch (elements)
    long long n;     // elements in the box allocation
    __host__ __device__ __forceinline__ long long at(int i, int j, int k) const {
        return (long long)k * sk + (long long)j * sj + (long long)(i + kOX);
    }
};

inline Geom make_geom(int nx, int ny, int nz) {
    Geom g;
    g.nx = nx; g.ny = ny; g.nz = nz;
    int need = kOX + nx + 2;
    g.sj = (need + 31) / 32 * 32;
    g.sk = (long long)g.sj * (ny + 2);
    g.n = g.sk * (nz + 2);
    return g;
}

template <typename T>
struct Coef {
    T *a1, *b12, *b13;  // csi faces
    T *a2, *b21, *b23;  // eta faces
    T *a3, *b31, *b32;  // zeta faces
};

template <typename T>
__device__ __forceinline__ T ld(const T* p, long long q) { return __ldg(p + q); }

// ---------------------------------------------------------------------------
// L_n(p) - rh at one interior cell: resid_sndrcv.f03:80-151 with the scaled
// coefficients.  The six face fluxes are res_dx, res_sn, res_sop, res_sot,
// res_av, res_ind of the reference.
template <typename T>
__device__ __forceinline__ T cell_residual(const Geom& g, const Coef<T>& c, const T* __restrict__ p,
                                           const T* __restrict__ rh, long long q) {
    const long long sj = g.sj, sk = g.sk;
    const T pc = ld(p, q);
    const T pe = ld(p, q + 1), pw = ld(p, q - 1);
    const T pn = ld(p, q + sj), ps = ld(p, q - sj);
    const T pf = ld(p, q + sk), pb = ld(p, q - sk);
    const T pen = ld(p, q + 1 + sj), pes = ld(p, q + 1 - sj), pwn = ld(p, q - 1 + sj), pws = ld(p, q - 1 - sj);
    const T pef = ld(p, q + 1 + sk), peb = ld(p, q + 1 - sk), pwf = ld(p, q - 1 + sk), pwb = ld(p, q - 1 - sk);
    const T pnf = ld(p, q + sj + sk), pnb = ld(p, q + sj - sk), psf = ld(p, q - sj + sk), psb = ld(p, q - sj - sk);
    T fdx = ld(c.a1, q) * (pe - pc) + ld(c.b12, q) * (pen + pn - pes - ps) + ld(c.b13, q) * (pef + pf - peb - pb);
    T fsn = ld(c.a1, q - 1) * (pc - pw) + ld(c.b12, q - 1) * (pn + pwn - ps - pws) +
            ld(c.b13, q - 1) * (pf + pwf - pb - pwb);
    T fsop = ld(c.a2, q) * (pn - pc) + ld(c.b21, q) * (pen + pe - pwn - pw) + ld(c.b23, q) * (pnf + pf - pnb - pb);
    T fsot = ld(c.a2, q - sj) * (pc - ps) + ld(c.b21, q - sj) * (pe + pes - pw - pws) +
             ld(c.b23, q - sj) * (pf + psf - pb - psb);
    T fav = ld(c.a3, q) * (pf - pc) + ld(c.b31, q) * (pef + pe - pwf - pw) + ld(c.b32, q) * (pnf + pn - psf - ps);
    T find = ld(c.a3, q - sk) * (pc - pb) + ld(c.b31, q - sk) * (pe + peb - pw - pwb) +
             ld(c.b32, q - sk) * (pn + pnb - ps - psb);
    return (fdx - fsn + fsop - fsot + fav - find) - ld(rh, q);
}

// ---------------------------------------------------------------------------
// Periodic ghost shell in x and z (ip = kp = 0): every ghost cell with i or k
// outside the interior copies its periodic image, for all rows j = 0..ny+1
// including the wall ghost rows.  At the fixed point this is exactly the
// reference's x/z copies, corner lines, vertical frame and horizontal square
// (multigrid.f03:1145-1158, 1325-1620).  Sources are never ghosts in x or z,
// so the kernel is race-free.
template <typename T>
__global__ void k_ghost_xz(Geom g, T* __restrict__ p) {
    const int nxg = g.nx + 2, nyg = g.ny + 2;
    const long long nplane = (long long)nxg * nyg;  // cells of one k = 0 / nz+1 plane
    const long long nside = 2LL * nyg * g.nz;       // i = 0 / nx+1 columns, k = 1..nz
    const long long tot = 2 * nplane + nside;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < tot;
         t += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        if (t < 2 * nplane) {
            int side = (int)(t / nplane);
            long long r = t - side * nplane;
            j = (int)(r / nxg);
            i = (int)(r - (long long)j * nxg);
            k = side ? g.nz + 1 : 0;
        } else {
            long long r = t - 2 * nplane;
            int side = (int)(r / ((long long)nyg * g.nz));
            r -= side * (long long)nyg * g.nz;
            k = (int)(r / nyg) + 1;
            j = (int)(r - (long long)(k - 1) * nyg);
            i = side ? g.nx + 1 : 0;
        }
        int si = i == 0 ? g.nx : (i == g.nx + 1 ? 1 : i);
        int sk = k == 0 ? g.nz : (k == g.nz + 1 ? 1 : k);
        p[g.at(i, j, k)] = p[g.at(si, j, sk)];
    }
}

// ---------------------------------------------------------------------------
// eta-line relaxation (the device form of solut_sndrcv_slor,
// multigrid.f03:1939-2290 with tridag.f03).  One thread owns the line (i,k)
// and solves the tridiagonal system over j = 0..ny+1, whose end rows are the
// wall ghost relations (sett.f03:114-143): off-line neighbours and all cross
// terms are explicit, the normal x/z couplings sit on the diagonal.
//   ZEBRA = false: Jacobi over lines, pin -> pout, pout = pin + omega*(x - pin)
//   ZEBRA = true : lines with (i%2, k%2) == colour, in place, SOR factor omega
// The homogeneous wall relation is used (an = 0): this kernel runs on
// corrections only; the FP64 outer loop applies the cs terms.
// Shared memory holds c'(j), d'(j) of the Thomas sweep, [j][thread].
template <typename T, bool ZEBRA>
__global__ void k_line_relax(Geom g, Coef<T> c, const T* pin, T* pout,
                             const T* __restrict__ rh, T omega, int colour) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int nth = blockDim.x * blockDim.y;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    T* sc = reinterpret_cast<T*>(smem_raw);
    T* sd = sc + (size_t)(g.ny + 2) * nth;
    int i, k;
    if (ZEBRA) {
        i = 2 * (blockIdx.x * blockDim.x + threadIdx.x) + 1 + (colour & 1);
        k = 2 * (blockIdx.y * blockDim.y + threadIdx.y) + 1 + (colour >> 1);
    } else {
        i = blockIdx.x * blockDim.x + threadIdx.x + 1;
        k = blockIdx.y * blockDim.y + threadIdx.y + 1;
    }
    if (i > g.nx || k > g.nz) return;
    const int ny = g.ny;
    const long long sj = g.sj, sk = g.sk;
    const T* p = pin;

    // x/z normal couplings of this line's cells go on the diagonal
    // row 0: bottom wall ghost relation (mul_boun_sndrcv :1166-1173, an = 0)
    long long q = g.at(i, 0, k);
    T a2 = ld(c.a2, q);
    T f = ld(c.b21, q) * (ld(p, q + 1 + sj) + ld(p, q + 1) - ld(p, q - 1 + sj) - ld(p, q - 1)) +
          ld(c.b23, q) * (ld(p, q + sj + sk) + ld(p, q + sk) - ld(p, q + sj - sk) - ld(p, q - sk));
    T cp = T(-1);         // c'_0 = c_0 / b_0 = -a2 / a2
    T dp = f / a2;        // d'_0
    sc[tid] = cp;
    sd[tid] = dp;
    T a2m = a2;           // A2 of face j-1
    for (int j = 1; j <= ny; ++j) {
        q += sj;
        const T pc = ld(p, q);
        const T pe = ld(p, q + 1), pw = ld(p, q - 1);
        const T pn = ld(p, q + sj), ps = ld(p, q - sj);
        const T pf = ld(p, q + sk), pb = ld(p, q - sk);
        const T pen = ld(p, q + 1 + sj), pes = ld(p, q + 1 - sj), pwn = ld(p, q - 1 + sj), pws = ld(p, q - 1 - sj);
        const T pef = ld(p, q + 1 + sk), peb = ld(p, q + 1 - sk), pwf = ld(p, q - 1 + sk), pwb = ld(p, q - 1 - sk);
        const T pnf = ld(p, q + sj + sk), pnb = ld(p, q + sj - sk), psf = ld(p, q - sj + sk), psb = ld(p, q - sj - sk);
        const T a1e = ld(c.a1, q), a1w = ld(c.a1, q - 1);
        const T a3f = ld(c.a3, q), a3b = ld(c.a3, q - sk);
        a2 = ld(c.a2, q);
        // off-line explicit part N (cross terms use the old on-line values too)
        T nsum = a1e * pe + a1w * pw + a3f * pf + a3b * pb;
        nsum += ld(c.b12, q) * (pen + pn - pes - ps) - ld(c.b12, q - 1) * (pn + pwn - ps - pws);
        nsum += ld(c.b13, q) * (pef + pf - peb - pb) - ld(c.b13, q - 1) * (pf + pwf - pb - pwb);
        nsum += ld(c.b21, q) * (pen + pe - pwn - pw) - ld(c.b21, q - sj) * (pe + pes - pw - pws);
        nsum += ld(c.b23, q) * (pnf + pf - pnb - pb) - ld(c.b23, q - sj) * (pf + psf - pb - psb);
        nsum += ld(c.b31, q) * (pef + pe - pwf - pw) - ld(c.b31, q - sk) * (pe + peb - pw - pwb);
        nsum += ld(c.b32, q) * (pnf + pn - psf - ps) - ld(c.b32, q - sk) * (pn + pnb - ps - psb);
        f = ld(rh, q) - nsum;
        const T b = -(a2 + a2m + a1e + a1w + a3f + a3b);
        const T m = b - a2m * cp;
        const T inv = T(1) / m;
        cp = a2 * inv;
        dp = (f - a2m * dp) * inv;
        sc[(size_t)j * nth + tid] = cp;
        sd[(size_t)j * nth + tid] = dp;
        a2m = a2;
    }
    // row ny+1: top wall ghost relation (mul_boun_sndrcv :1175-1186, an = 0)
    q += sj;
    {
        const long long qn = q - sj;  // face ny lives at cell (i, ny, k)
        f = -(ld(c.b21, qn) * (ld(p, q + 1) + ld(p, qn + 1) - ld(p, q - 1) - ld(p, qn - 1)) +
              ld(c.b23, qn) * (ld(p, q + sk) + ld(p, qn + sk) - ld(p, q - sk) - ld(p, qn - sk)));
        // a = -A2(ny), b = A2(ny), c = 0
        const T m = a2m - (-a2m) * cp;
        dp = (f + a2m * dp) / m;
    }
    // back substitution and relaxed update, j = ny+1 .. 0
    T xs = dp;
    {
        const T old = ld(p, q);
        pout[q] = old + omega * (xs - old);
    }
    for (int j = ny; j >= 0; --j) {
        q -= sj;
        xs = sd[(size_t)j * nth + tid] - sc[(size_t)j * nth + tid] * xs;
        const T old = ld(p, q);
        pout[q] = old + omega * (xs - old);
    }
}

// ---------------------------------------------------------------------------
// Residual + restriction (resid_sndrcv.f03 followed by restrict_sndrcv.f03:
// 32-53): coarse rh = -(1/8) * sum of the 8 fine residuals L(p) - rh.
template <typename T>
__global__ void k_resid_restrict(Geom gf, Geom gc, Coef<T> c, const T* __restrict__ p,
                                 const T* __restrict__ rh, T* __restrict__ rhc) {
    const int ic = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int jc = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int kc = blockIdx.z + 1;
    if (ic > gc.nx || jc > gc.ny) return;
    T s = T(0);
#pragma unroll
    for (int dk = -1; dk <= 0; ++dk)
#pragma unroll
        for (int dj = -1; dj <= 0; ++dj)
#pragma unroll
            for (int di = -1; di <= 0; ++di)
                s += cell_residual(gf, c, p, rh, gf.at(2 * ic + di, 2 * jc + dj, 2 * kc + dk));
    rhc[gc.at(ic, jc, kc)] = -s * T(0.125);
}

// Plain residual L(p) - rh into out (interior cells).
template <typename T>
__global__ void k_residual(Geom g, Coef<T> c, const T* __restrict__ p, const T* __restrict__ rh,
                           T* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z + 1;
    if (i > g.nx || j > g.ny) return;
    const long long q = g.at(i, j, k);
    out[q] = cell_residual(g, c, p, rh, q);
}

// Restriction alone (restrict_sndrcv.f03:32-53).
template <typename T>
__global__ void k_restrict(Geom gf, Geom gc, const T* __restrict__ r, T* __restrict__ rc) {
    const int ic = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int jc = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int kc = blockIdx.z + 1;
    if (ic > gc.nx || jc > gc.ny) return;
    const int id = 2 * ic, jd = 2 * jc, kd = 2 * kc;
    T v = r[gf.at(id, jd, kd)] + r[gf.at(id - 1, jd, kd)] + r[gf.at(id, jd - 1, kd)] +
          r[gf.at(id - 1, jd - 1, kd)] + r[gf.at(id, jd, kd - 1)] + r[gf.at(id - 1, jd, kd - 1)] +
          r[gf.at(id, jd - 1, kd - 1)] + r[gf.at(id - 1, jd - 1, kd - 1)];
    rc[gc.at(ic, jc, kc)] = -v * T(0.125);
}

// ---------------------------------------------------------------------------
// Prolongation (prolong.f03:64-261): coarse cells i = 0..nxc, j = 0..nyc,
// k = 0..nzc add trilinear (27/9/3/1)/64 corrections into their eight fine
// children (2i+a, 2j+b, 2k+c), which cover every fine cell including ghosts.
template <typename Tf, typename Tc>
__global__ void k_prolong(Geom gf, Geom gc, Tf* __restrict__ pf, const Tc* __restrict__ pc) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i > gc.nx || j > gc.ny) return;
    const long long q = gc.at(i, j, k);
    const long long sj = gc.sj, sk = gc.sk;
    Tc v[8];
    v[0] = pc[q]; v[1] = pc[q + 1]; v[2] = pc[q + sj]; v[3] = pc[q + 1 + sj];
    v[4] = pc[q + sk]; v[5] = pc[q + 1 + sk]; v[6] = pc[q + sj + sk]; v[7] = pc[q + 1 + sj + sk];
#pragma unroll
    for (int cz = 0; cz < 2; ++cz)
#pragma unroll
        for (int cy = 0; cy < 2; ++cy)
#pragma unroll
            for (int cx = 0; cx < 2; ++cx) {
                Tc s = Tc(0);
#pragma unroll
                for (int c = 0; c < 8; ++c) {
                    const int ox = c & 1, oy = (c >> 1) & 1, oz = c >> 2;
                    const Tc w = Tc((ox == cx ? 3 : 1) * (oy == cy ? 3 : 1) * (oz == cz ? 3 : 1));
                    s += w * v[c];
                }
                const long long qf = gf.at(2 * i + cx, 2 * j + cy, 2 * k + cz);
                pf[qf] = pf[qf] + Tf(s * Tc(1.0 / 64.0));
            }
}

}  // namespace ples
