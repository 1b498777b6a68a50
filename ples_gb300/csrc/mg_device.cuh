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
// With the coarse metric t of a level built from nodes sub-sampled by the
// cumulative strides (sx,sy,sz), the stored coefficient is t/(sx*sy*sz):
// for the reference's full coarsening (sx=sy=sz=2^(n-1)) that is exactly
// mul_met's t/pot times ppot2.
//
// Ghost shell.  In a periodic direction (ip = 0 / kp = 0, Geom px / pz)
// ghost cells with i or k outside the interior hold the periodic image of
// the interior, for every row j including the two wall ghost rows; every
// kernel that writes a field keeps those images, so no separate copy pass is
// needed.  In a walled direction the ghosts follow the wall relation and are
// set by the side fill (outer_device.cuh).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace ples {

constexpr int kOX = 31;  // element offset of i = 0 inside a row

// resident CTAs per SM the FP32 line smoother is compiled for (its register
// budget: 65536 / (256 * this)); 4 measured fastest on GB300 (2-6 tried)
#ifndef PLES_LINE_MIN_BLOCKS
#define PLES_LINE_MIN_BLOCKS 4
#endif
// how many of its rows ahead a warp of the line smoother prefetches into L2
#ifndef PLES_LINE_PF_ROWS
#define PLES_LINE_PF_ROWS 1
#endif

struct Geom {
    int nx, ny, nz;
    int sj;          // row pitch (elements)
    long long sk;    // plane pitch (elements)
    long long n;     // elements in the box allocation
    int px, pz;      // 1: periodic in x / z (ghosts are images); 0: walls (ghosts from their relation)
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
    g.px = g.pz = 1;
    return g;
}

template <typename T>
struct Coef {
    T *a1, *b12, *b13;  // csi faces
    T *a2, *b21, *b23;  // eta faces
    T *a3, *b31, *b32;  // zeta faces
};

// Block coordinates of one unit of work.  Every kernel body takes them
// explicitly: a plain launch passes blockIdx/gridDim (hw_blk), a batched
// launch over many grids hands out virtual blocks of each grid's own launch
// shape (batch.cu), so both run the same code.
struct Blk {
    int x, y, z;
    int gx, gy, gz;
};
__device__ __forceinline__ Blk hw_blk() {
    return Blk{(int)blockIdx.x, (int)blockIdx.y, (int)blockIdx.z, (int)gridDim.x, (int)gridDim.y, (int)gridDim.z};
}

template <typename T>
__device__ __forceinline__ T ld(const T* p, long long q) { return __ldg(p + q); }
template <typename T>
__device__ __forceinline__ T ld(const T* p, unsigned q) { return __ldg(p + q); }

// 1: the line smoother loads the arrays it reads once per launch with the
// streaming operator (ld.global.cs: evict-first in L2), so that the rows its
// odd-i pass reads a second time stay in L2; 0: every load plain
#ifndef PLES_LINE_L2HINT
#define PLES_LINE_L2HINT 1
#endif
template <typename T>
__device__ __forceinline__ T ld1(const T* p, unsigned q) {
#if PLES_LINE_L2HINT
    return __ldcs(p + q);
#else
    return __ldg(p + q);
#endif
}

// Every spin-wait on the device is bounded: it gives up after kSpinLimit
// polls (or fewer, when the handle's wait limit says so) or kWaitNs of wall
// time, whichever comes first.
constexpr unsigned kSpinLimit = 1u << 26;              // polls of one wait at most
constexpr unsigned long long kWaitNs = 2000000000ull;  // and 2 s of wall time

// nanoseconds of the GPU's global timer
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// element offset of (i,j,k) in 32 bits: a box has fewer than 2^31 elements
// (checked when a handle is created), so kernels that issue many loads per
// cell form each address with one 32x32->64 multiply-add
__device__ __forceinline__ unsigned at32(const Geom& g, int i, int j, int k) {
    return (unsigned)k * (unsigned)g.sk + (unsigned)j * (unsigned)g.sj + (unsigned)(i + kOX);
}

// hint the L2 to fetch the line holding p[q] (no register, no L1 allocation)
template <typename T>
__device__ __forceinline__ void pf_l2(const T* p, long long q) {
    asm volatile("prefetch.global.L2 [%0];" ::"l"(p + q));
}
template <typename T>
__device__ __forceinline__ void pf_l2(const T* p, unsigned q) {
    asm volatile("prefetch.global.L2 [%0];" ::"l"(p + q));
}

// Store v at interior cell (i,j,k) and at its periodic images in the x/z
// ghost shell (the reference's periodic copies, corner lines, vertical frame
// and horizontal square, multigrid.f03:1145-1158, 1325-1620).
template <typename T>
__device__ __forceinline__ void store_periodic(const Geom& g, T* p, int i, int j, int k, T v) {
    p[g.at(i, j, k)] = v;
    const int gi = !g.px ? -1 : (i == g.nx ? 0 : (i == 1 ? g.nx + 1 : -1));
    const int gk = !g.pz ? -1 : (k == g.nz ? 0 : (k == 1 ? g.nz + 1 : -1));
    if (gi >= 0) p[g.at(gi, j, k)] = v;
    if (gk >= 0) {
        p[g.at(i, j, gk)] = v;
        if (gi >= 0) p[g.at(gi, j, gk)] = v;
    }
    if (g.px && g.nx == 1 && i == 1) {  // a single column is its own image on both sides
        p[g.at(0, j, k)] = v;
        if (gk >= 0) p[g.at(0, j, gk)] = v;
    }
    if (g.pz && g.nz == 1 && k == 1) {
        p[g.at(i, j, 0)] = v;
        if (gi >= 0) p[g.at(gi, j, 0)] = v;
    }
}

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
// Periodic ghost shell refresh: every ghost cell with i or k outside the
// interior in a periodic direction copies its periodic image, rows
// j = 0..ny+1.  Used once on fields that arrive from outside (the caller's fi).
template <typename T>
__device__ __forceinline__ void k_ghost_xz_blk(Geom g, T* __restrict__ p, const Blk& B) {
    const int nxg = g.nx + 2, nyg = g.ny + 2;
    const long long nplane = (long long)nxg * nyg;  // cells of one k = 0 / nz+1 plane
    const long long nside = 2LL * nyg * g.nz;       // i = 0 / nx+1 columns, k = 1..nz
    const long long tot = 2 * nplane + nside;
    for (long long t = B.x * (long long)blockDim.x + threadIdx.x; t < tot;
         t += (long long)B.gx * blockDim.x) {
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
        // walled directions keep their ghosts (set by their relations); at
        // a periodic z plane a wall column takes the image of its own column
        const bool xg = i == 0 || i == g.nx + 1, zg = k == 0 || k == g.nz + 1;
        if ((xg && !g.px && !zg) || (zg && !g.pz)) continue;
        int si = g.px ? (i == 0 ? g.nx : (i == g.nx + 1 ? 1 : i)) : i;
        int sk = k == 0 ? g.nz : (k == g.nz + 1 ? 1 : k);
        p[g.at(i, j, k)] = p[g.at(si, j, sk)];
    }
}
template <typename T>
__global__ void k_ghost_xz(Geom g, T* __restrict__ p) {
    k_ghost_xz_blk<T>(g, p, hw_blk());
}

// ---------------------------------------------------------------------------
// Immersed-boundary mask (no counterpart in the reference's multigrid).  m is
// a byte box of the level: 1 = solid cell; the periodic ghost shell holds the
// images and each wall ghost row the value of the interior cell next to it.
// A face that touches a solid cell carries no flux (Neumann at the immersed
// boundary): its normal and cross coefficients are zeroed.  A cross
// coefficient of a fluid-fluid face is zeroed too when its tangential stencil
// reaches a solid cell, so the operator of the fluid cells reads fluid values
// only and keeps constants in its null space.  A solid cell is left with all
// coefficients zero: the smoothers treat such rows as identity rows.
template <typename T>
__global__ void k_mask_coef(Geom g, Coef<T> c, const uint8_t* __restrict__ m) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i > g.nx || j > g.ny || k > g.nz) return;
    const long long q = g.at(i, j, k), sj = g.sj, sk = g.sk;
    auto S = [&](long long r) { return m[r] != 0; };
    if (j >= 1) {  // csi face i+1/2 of cell (i,j,k)
        if (S(q) || S(q + 1)) {
            c.a1[q] = T(0); c.b12[q] = T(0); c.b13[q] = T(0);
        } else {
            if (S(q + sj) || S(q - sj) || S(q + 1 + sj) || S(q + 1 - sj)) c.b12[q] = T(0);
            if (k >= 1 && (S(q + sk) || S(q - sk) || S(q + 1 + sk) || S(q + 1 - sk))) c.b13[q] = T(0);
        }
    }
    if (i >= 1 && k >= 1) {  // eta face j+1/2
        if (S(q) || S(q + sj)) {
            c.a2[q] = T(0); c.b21[q] = T(0); c.b23[q] = T(0);
        } else {
            if (S(q + 1) || S(q - 1) || S(q + 1 + sj) || S(q - 1 + sj)) c.b21[q] = T(0);
            if (S(q + sk) || S(q - sk) || S(q + sj + sk) || S(q + sj - sk)) c.b23[q] = T(0);
        }
    }
    if (i >= 1 && j >= 1) {  // zeta face k+1/2
        if (S(q) || S(q + sk)) {
            c.a3[q] = T(0); c.b31[q] = T(0); c.b32[q] = T(0);
        } else {
            if (S(q + 1) || S(q - 1) || S(q + 1 + sk) || S(q - 1 + sk)) c.b31[q] = T(0);
            if (S(q + sj) || S(q - sj) || S(q + sj + sk) || S(q - sj + sk)) c.b32[q] = T(0);
        }
    }
}

// zero a field on the solid cells of the mask (the whole box)
template <typename T>
__global__ void k_zero_solid(Geom g, T* __restrict__ p, const uint8_t* __restrict__ m) {
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < g.n;
         q += (long long)gridDim.x * blockDim.x)
        if (m[q]) p[q] = T(0);
}

// ---------------------------------------------------------------------------
// The two first-order recurrences of a Thomas solve with a precomputed LU
// factor, for the 32 lines (lanes) held in shared memory [nj][32]:
//   forward  d(j) = G(j) - AL(j) d(j-1),  d(0) = G(0)
//   backward x(j) = d(j) - CP(j) x(j+1),  x(nj-1) = d(nj-1)  (CP(nj-1) = 0)
// Each is an affine map per row, so the rows are cut into one segment per
// warp: every warp composes its segment's map (offset u, factor v) with the
// incoming value set to zero, the maps are shared through su/sv ([nw][32]),
// each warp folds the maps of the segments before it into its incoming value
// and then runs its own segment again with that value.  The serial depth
// drops from 2 nj to about 4 nj / nw + 2 nw dependent steps.  The solution
// replaces G.  Lanes with mine == false do no arithmetic; every thread must
// call (the function holds __syncthreads).
// RS: row stride of G / AL / CP (lines per tile); slot: this lane's column
// in them (the lane itself when negative).  The folds over the maps of the
// segments before / after a warp's own are unrolled to NWMAX (the most warps
// a CTA has), so their shared-memory loads issue ahead of the FMA chain.
// su2 / sv2: a second map buffer for the backward maps, which saves the
// barrier that otherwise protects the forward maps (null: one buffer).
template <typename T, int RS = 32, int NWMAX = 16>
__device__ __forceinline__ void seg_thomas(T* G, const T* AL, const T* CP, int nj, bool mine, T* su, T* sv,
                                           int slot = -1, T* su2 = nullptr, T* sv2 = nullptr) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int col = slot < 0 ? lane : slot;
    const int len = (nj + nw - 1) / nw;
    const int j0 = min(w * len, nj), j1 = min(j0 + len, nj);
    T u = T(0), v = T(1);
    if (mine)
        for (int j = j0; j < j1; ++j) {
            const T al = AL[j * RS + col];
            u = G[j * RS + col] - al * u;
            v = -al * v;
        }
    su[w * 32 + lane] = u;
    sv[w * 32 + lane] = v;
    __syncthreads();
    if (mine) {
        T d = T(0);
#pragma unroll
        for (int s = 0; s < NWMAX; ++s)
            if (s < w) d = su[s * 32 + lane] + sv[s * 32 + lane] * d;
        for (int j = j0; j < j1; ++j) {
            d = G[j * RS + col] - AL[j * RS + col] * d;
            G[j * RS + col] = d;
        }
    }
    u = T(0);
    v = T(1);
    if (mine)
        for (int j = j1 - 1; j >= j0; --j) {
            const T c = CP[j * RS + col];
            u = G[j * RS + col] - c * u;
            v = -c * v;
        }
    T* bu = su2 ? su2 : su;
    T* bv = su2 ? sv2 : sv;
    if (!su2) __syncthreads();  // the forward maps are read by now
    bu[w * 32 + lane] = u;
    bv[w * 32 + lane] = v;
    __syncthreads();
    if (mine) {
        T x = T(0);
#pragma unroll
        for (int s = NWMAX - 1; s >= 0; --s)
            if (s < nw && s > w) x = bu[s * 32 + lane] + bv[s * 32 + lane] * x;
        for (int j = j1 - 1; j >= j0; --j) {
            x = G[j * RS + col] - CP[j * RS + col] * x;
            G[j * RS + col] = x;
        }
    }
    __syncthreads();
}

// ---------------------------------------------------------------------------
// LU factor of the fixed eta-line operator (sett.f03:114-143 rows, the
// forward sweep of tridag.f03): c'(0) = -1, c'(j) = A2(j) / (b(j) - A2(j-1)
// c'(j-1)).  The operator depends on the coefficients only, so c' is built
// once per level; the smoothers then need one division per row in their
// parallel phase and a pure FMA chain in the sequential one.  With im given,
// the pivot reciprocal 1/m(j) of every row j = 0..ny+1 is stored as well
// (the expressions the line smoothers evaluate, 1 on identity rows), so
// the pair-build smoother needs no division at all.
template <typename T>
__global__ void k_line_lu(Geom g, Coef<T> c, T* __restrict__ cp, T* __restrict__ im) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int k = blockIdx.y + 1;
    if (i > g.nx) return;
    // a row whose coefficients are all zero (a solid cell of an immersed-
    // boundary mask, or the wall row next to one) is an identity row: c' = 0
    const T a20 = ld(c.a2, g.at(i, 0, k));
    T prev = a20 == T(0) ? T(0) : T(-1);
    cp[g.at(i, 0, k)] = prev;
    if (im) im[g.at(i, 0, k)] = a20 == T(0) ? T(1) : T(1) / a20;
    for (int j = 1; j <= g.ny; ++j) {
        const long long q = g.at(i, j, k);
        const T a = ld(c.a2, q - g.sj), cc = ld(c.a2, q);
        // the faces of x / z walls carry no flux in the relaxed equation
        const T ae = !g.px && i == g.nx ? T(0) : ld(c.a1, q), aw = !g.px && i == 1 ? T(0) : ld(c.a1, q - 1);
        const T af = !g.pz && k == g.nz ? T(0) : ld(c.a3, q), ab = !g.pz && k == 1 ? T(0) : ld(c.a3, q - g.sk);
        const T b = -(cc + a + ae + aw + af + ab);
        if (im) im[q] = b == T(0) ? T(1) : T(1) / (b - a * prev);
        prev = b == T(0) ? T(0) : cc / (b - a * prev);
        cp[q] = prev;
    }
    cp[g.at(i, g.ny + 1, k)] = T(0);
    if (im) {  // the top wall row: a2(ny) x(ny+1) - a2(ny) x(ny) = f
        const T as = ld(c.a2, g.at(i, g.ny, k));
        const T a = -as;
        im[g.at(i, g.ny + 1, k)] = as == T(0) ? T(1) : T(1) / (as - a * prev);
    }
}

// ---------------------------------------------------------------------------
// Zebra second half: the odd-i lines of a tile add their six in-plane
// x-neighbour terms, evaluated with the new even-i values (G holds them;
// outside the tile the old field pin), to the scaled right-hand side
// G(j) -= T_x(j) / m(j), where CP(j) held 1/m(j); CP(j) becomes c'(j).
// Rows go in batches of kXB per warp with every load of a batch issued
// before its arithmetic.  Loads of rows 0 and ny+1 that the wall relations
// do not use stay inside the box allocation (k >= 1).
template <typename T, bool ZIN>
__device__ __forceinline__ void odd_x_terms(const Geom& g, const Coef<T>& c, const T* __restrict__ cpa,
                                            const T* __restrict__ pin, T* G, T* CP, int i, int k) {
    constexpr int kXB = 2;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int nj = g.ny + 2, ny = g.ny;
    const long long sj = g.sj, sk = g.sk;
    const bool west_out = lane == 0 || i - 1 < 1;  // i-1 not a lane of this tile
    auto PX = [&](int j, int di, int dj) -> T {
        const int l2 = lane + di;
        if (l2 >= 0 && l2 < 32 && i + di >= 1 && i + di <= g.nx) return G[(j + dj) * 32 + l2];
        return ZIN ? T(0) : ld(pin, g.at(i + di, j + dj, k));
    };
    for (int jb = w; jb < nj; jb += kXB * nw) {
        T a1[kXB], a1w[kXB], b12[kXB], b12w[kXB], b21[kXB], b21s[kXB], b31[kXB], b31b[kXB], cpv[kXB];
        T wm[kXB], w0[kXB], wp[kXB];  // old west neighbours (dj = -1, 0, +1) when outside the tile
#pragma unroll
        for (int u = 0; u < kXB; ++u) {
            const int j = min(jb + u * nw, nj - 1);
            const long long q = g.at(i, j, k);
            a1[u] = ld(c.a1, q); a1w[u] = ld(c.a1, q - 1);
            b12[u] = ld(c.b12, q); b12w[u] = ld(c.b12, q - 1);
            b21[u] = ld(c.b21, q); b21s[u] = ld(c.b21, q - sj);
            b31[u] = ld(c.b31, q); b31b[u] = ld(c.b31, q - sk);
            cpv[u] = ld(cpa, q);
            const bool wl = !ZIN && west_out;
            wm[u] = wl && j > 0 ? ld(pin, q - 1 - sj) : T(0);
            w0[u] = wl ? ld(pin, q - 1) : T(0);
            wp[u] = wl && j < nj - 1 ? ld(pin, q - 1 + sj) : T(0);
        }
#pragma unroll
        for (int u = 0; u < kXB; ++u) {
            const int j = jb + u * nw;
            if (j >= nj) break;
            const T pw = west_out ? w0[u] : PX(j, -1, 0);
            const T pwn = west_out ? wp[u] : (j < nj - 1 ? PX(j, -1, 1) : T(0));
            const T pws = west_out ? wm[u] : (j > 0 ? PX(j, -1, -1) : T(0));
            T tx;
            if (j == 0) {
                tx = -b21[u] * (PX(j, 1, 1) + PX(j, 1, 0) - pwn - pw);
            } else if (j == ny + 1) {
                tx = b21s[u] * (PX(j, 1, 0) + PX(j, 1, -1) - pw - pws);
            } else {
                const T pe = PX(j, 1, 0);
                const T pen = PX(j, 1, 1), pes = PX(j, 1, -1);
                tx = a1[u] * pe + a1w[u] * pw + b12[u] * (pen - pes) - b12w[u] * (pwn - pws) +
                     b21[u] * (pen + pe - pwn - pw) - b21s[u] * (pe + pes - pw - pws) + (b31[u] - b31b[u]) * (pe - pw);
            }
            const T im = CP[j * 32 + lane];
            G[j * 32 + lane] -= tx * im;
            CP[j * 32 + lane] = j == ny + 1 ? T(0) : cpv[u];
        }
    }
}

// the values of the lane beside (i-1 / i+1); lanes 0 and 31 take the column
// just outside the tile, h, which they loaded themselves
template <typename T>
__device__ __forceinline__ T from_west(T v, T h) {
    const T s = __shfl_up_sync(0xffffffffu, v, 1);
    return (threadIdx.x & 31) == 0 ? h : s;
}
template <typename T>
__device__ __forceinline__ T from_east(T v, T h) {
    const T s = __shfl_down_sync(0xffffffffu, v, 1);
    return (threadIdx.x & 31) == 31 ? h : s;
}

// Phase 1 of the plain-load smoother: warp w builds the rows of its own
// segment j0..j1-1 (the one seg_thomas gives it) in order.  The pressure
// rows j-1, j, j+1 of planes k-1, k, k+1 stay in a three-row window and the
// eta-face coefficients of row j-1 are carried, so a step loads one new
// pressure row per plane and the coefficients of row j once; the i-1 / i+1
// values come from the lanes beside, and lanes 0 and 31 load the columns
// just outside the tile.  Every lane up to the east ghost column i = nx+1
// holds its pressure column; the rows and the arithmetic of each equation
// are those of the strided form (same expressions, same order).
// Loads ahead: rows PLES_LINE_PF_ROWS further on are hinted into L2.
// WALLS: x / z walls; as in the reference's line SOR (multigrid.f03:2120-
// 2160, masks i_dx..i_in of sett.f03) a wall face carries no flux in the
// relaxed equation (the correction's wall flux is zero), while the ghost
// cells beyond it still enter the cross terms of the other faces.
// RS, slot: as in seg_thomas; ws / nws: the row segment this warp builds and
// the number of segments (by default the warp's index among the CTA's warps).
// FAST: the pivot reciprocals come from ima (1/m per row, k_line_lu) instead
// of a division per row, and the next rows reach the L2 through one prefetch
// instruction per row step (lane t fetching the line of array t) instead of
// one per array.
template <typename T, bool ZEBRA, bool ZIN, bool WALLS = false, int RS = 32, bool FAST = false>
__device__ __forceinline__ void build_rows(const Geom& g, const Coef<T>& c, const T* __restrict__ cpa,
                                           const T* __restrict__ pin, const T* __restrict__ pk,
                                           const T* __restrict__ rh, T omega, int zk, int i, int k, bool odd, T* G,
                                           T* AL, T* CP, int ws = -1, int nws = 0, int slot = -1,
                                           const T* __restrict__ ima = nullptr) {
    const int lane = threadIdx.x & 31;
    const int w = ws < 0 ? (int)(threadIdx.x >> 5) : ws, nw = ws < 0 ? (int)(blockDim.x >> 5) : nws;
    const int sc = slot < 0 ? lane : slot;
    const int nj = g.ny + 2, ny = g.ny;
    const int len = (nj + nw - 1) / nw;
    const int j0 = min(w * len, nj), j1 = min(j0 + len, nj);
    const unsigned sj = (unsigned)g.sj, sk = (unsigned)g.sk;
    const bool act = i <= g.nx;      // the lane owns a line
    const bool col = i <= g.nx + 1;  // the lane holds a pressure column (the last may be the ghost)
    const bool halo = lane == 0 || (lane == 31 && i + 1 <= g.nx + 1);
    const int hd = lane == 0 ? -1 : 1;
    const bool noneigh = ZIN && (!ZEBRA || zk);  // every old neighbour is zero
    const bool kz = zk || noneigh;               // the k+-1 planes are zero
    auto row = [&](const T* a, int j, unsigned qk, T& v, T& h) {  // qk: offset of (i, 0, plane)
        v = T(0);
        h = T(0);
        if (j < 0 || j > ny + 1) return;
        const unsigned q = qk + (unsigned)j * sj;
        if (col) v = ld(a, q);
        if (halo) h = ld(a, q + hd);
    };
    const unsigned q0 = at32(g, i, 0, k);
    // FAST prefetch: lane t < 18 holds array t of the row (the k-1 zeta faces
    // and the pressure planes offset in advance); one 128-byte line each, the
    // warp's 32 lines starting on a line boundary
    const T* pfa = nullptr;
    if (FAST) {
        const int t = lane;
        const T* b = t == 0 ? c.a1 : t == 1 ? c.b12 : t == 2 ? c.b13 : t == 3 ? c.a2 : t == 4 ? c.b21
                   : t == 5 ? c.b23 : t == 6 || t == 9 ? c.a3 : t == 7 || t == 10 ? c.b31
                   : t == 8 || t == 11 ? c.b32 : t == 12 ? rh : t == 13 ? cpa : t == 14 ? ima
                   : t == 15 ? (ZIN ? nullptr : pin) : t == 16 || t == 17 ? (ZIN && zk ? nullptr : pk) : nullptr;
        const long long off = t >= 9 && t <= 11 ? -(long long)sk
                            : t == 15 ? (long long)sj : t == 16 ? (long long)sk + sj : t == 17 ? (long long)sj - sk : 0LL;
        if (b) pfa = b + off - lane;  // the warp's first line: element q0 - lane
    }
    // window: plane k (P), k+1 (F), k-1 (B); rows j-1 (m), j (0), j+1 (p);
    // h* the halo column of lanes 0 / 31; E*/W* the east / west values of
    // plane k (shuffled once per row and carried)
    T Pm = T(0), P0 = T(0), Pp = T(0);
    T EPm = T(0), EP0 = T(0), EPp = T(0), WPm = T(0), WP0 = T(0), WPp = T(0);
    T Fm = T(0), F0 = T(0), Fp = T(0), hF0 = T(0), hFp = T(0);
    T Bm = T(0), B0 = T(0), Bp = T(0), hB0 = T(0), hBp = T(0);
    if (j0 >= j1) return;
    if (!ZIN) {
        T hP0, hPp;
        row(pin, j0 - 1, q0, P0, hP0);
        row(pin, j0, q0, Pp, hPp);
        EP0 = from_east(P0, hP0);
        WP0 = from_west(P0, hP0);
        EPp = from_east(Pp, hPp);
        WPp = from_west(Pp, hPp);
    }
    if (!kz) {
        T d0, d1;
        row(pk, j0 - 1, q0 + sk, F0, d0);
        row(pk, j0, q0 + sk, Fp, hFp);
        row(pk, j0 - 1, q0 - sk, B0, d1);
        row(pk, j0, q0 - sk, Bp, hBp);
    }
    // eta-face coefficients of row j-1 (a2, b21, b23) and its LU factor c'
    T a2s = T(0), b21s = T(0), b23s = T(0), cps = T(0);
    if (act && j0 >= 1) {
        const unsigned q = q0 + (unsigned)(j0 - 1) * sj;
        a2s = ld(c.a2, q);
        b21s = ld(c.b21, q);
        b23s = ld(c.b23, q);
        cps = ld(cpa, q);
    }
    for (int j = j0; j < j1; ++j) {
        const unsigned q = q0 + (unsigned)j * sj;
        // every load of the step first: the coefficients of row j ...
        T a2v = T(0), b21v = T(0), b23v = T(0), cpv = T(0), imv = T(1);
        if (FAST && act) imv = ld1(ima, q);
        T a1e = T(0), b12v = T(0), b13v = T(0), a1h = T(0), b12h = T(0), b13h = T(0);
        T a3f = T(0), a3b = T(0), b31v = T(0), b31b = T(0), b32v = T(0), b32b = T(0), rhv = T(0);
        // (ld1: arrays this launch reads once; a1, b12, b21, b31 and c' are
        // read again by the odd-i pass and stay plain)
        if (act && j <= ny) {
            a2v = ld1(c.a2, q);
            b21v = ld(c.b21, q);
            b23v = ld1(c.b23, q);
            cpv = ld(cpa, q);
        }
        if (act && j >= 1 && j <= ny) {
            a1e = ld(c.a1, q); b12v = ld(c.b12, q); b13v = ld1(c.b13, q);
            a3f = ld1(c.a3, q); b31v = ld(c.b31, q); b32v = ld1(c.b32, q);
            a3b = ld1(c.a3, q - sk); b31b = ld(c.b31, q - sk); b32b = ld1(c.b32, q - sk);
            rhv = ld1(rh, q);
            if (lane == 0) { a1h = ld(c.a1, q - 1); b12h = ld(c.b12, q - 1); b13h = ld(c.b13, q - 1); }
        }
        // ... then the pressure rows j+1 of the three planes
        Pm = P0; P0 = Pp;
        EPm = EP0; EP0 = EPp; WPm = WP0; WP0 = WPp;
        Fm = F0; F0 = Fp; hF0 = hFp;
        Bm = B0; B0 = Bp; hB0 = hBp;
        T hPp = T(0);
        if (!ZIN) row(pin, j + 1, q0, Pp, hPp);
        if (!kz) {
            row(pk, j + 1, q0 + sk, Fp, hFp);
            row(pk, j + 1, q0 - sk, Bp, hBp);
        }
#if PLES_LINE_PF_ROWS > 0
        if (FAST) {
            if (pfa && j + PLES_LINE_PF_ROWS < j1 && (lane < 15 || j + PLES_LINE_PF_ROWS + 1 < nj))
                pf_l2(pfa, q + PLES_LINE_PF_ROWS * sj);
        } else if (act && j + PLES_LINE_PF_ROWS < j1) {
            const unsigned qn = q + PLES_LINE_PF_ROWS * sj;
            pf_l2(c.a1, qn); pf_l2(c.b12, qn); pf_l2(c.b13, qn);
            pf_l2(c.a2, qn); pf_l2(c.b21, qn); pf_l2(c.b23, qn);
            pf_l2(c.a3, qn); pf_l2(c.b31, qn); pf_l2(c.b32, qn);
            pf_l2(c.a3, qn - sk); pf_l2(c.b31, qn - sk); pf_l2(c.b32, qn - sk);
            pf_l2(rh, qn); pf_l2(cpa, qn);
            if (j + PLES_LINE_PF_ROWS + 1 < nj) {  // the row after stays inside the plane
                if (!ZIN) pf_l2(pin, qn + sj);
                if (!kz) { pf_l2(pk, qn + sj + sk); pf_l2(pk, qn + sj - sk); }
            }
        }
#endif
        if (!ZIN) {
            EPp = from_east(Pp, hPp);
            WPp = from_west(Pp, hPp);
        }
        // the in-plane x-neighbours
        const T pe = EP0, pw = WP0, pes = EPm, pws = WPm, pen = EPp, pwn = WPp;
        T f = T(0), a = T(0), im = T(1), tp = T(0);  // tp = (T p_old)(j), T the line operator
        if (j == 0) {
            if (act) {
                f = noneigh ? T(0) : b23v * (Fp + F0 - Bp - B0);
                if (!odd && !noneigh) f += b21v * (pen + pe - pwn - pw);
                a = T(0);
                im = FAST ? imv : T(1) / a2v;
                tp = a2v * P0 - a2v * Pp;
                if (a2v == T(0)) { im = T(1); f = T(0); tp = P0; }  // wall row above a solid cell
            }
        } else if (j == ny + 1) {
            if (act) {
                f = noneigh ? T(0) : -(b23s * (F0 + Fm - B0 - Bm));
                if (!odd && !noneigh) f -= b21s * (pe + pes - pw - pws);
                a = -a2s;
                im = FAST ? imv : T(1) / (a2s - a * cps);
                tp = a2s * P0 - a2s * Pm;
                if (a2s == T(0)) { im = T(1); f = T(0); tp = P0; }  // wall row below a solid cell
            }
        } else {
            T a1w = from_west(a1e, a1h), b12w = from_west(b12v, b12h), b13w = from_west(b13v, b13h);
            const T pef = from_east(F0, hF0), pwf = from_west(F0, hF0);
            const T peb = from_east(B0, hB0), pwb = from_west(B0, hB0);
            if (WALLS) {  // after the shuffles: the neighbours keep their own faces
                if (!g.px && i == 1) a1w = b12w = b13w = T(0);
                if (!g.px && i == g.nx) a1e = b12v = b13v = T(0);
                if (!g.pz && k == 1) a3b = b31b = b32b = T(0);
                if (!g.pz && k == g.nz) a3f = b31v = b32v = T(0);
            }
            if (act) {
                a = a2s;
                const T b = -(a2v + a + a1e + a1w + a3f + a3b);
                im = FAST ? imv : T(1) / (b - a * cps);
                f = rhv;
                tp = a * Pm + b * P0 + a2v * Pp;
                if (b == T(0)) {  // solid cell of an immersed-boundary mask: identity row
                    im = T(1);
                    f = T(0);
                    a = T(0);
                    tp = P0;
                }
                if (!noneigh) {
                    const T pn = Pp, ps = Pm, pf = F0, pb = B0;
                    const T pnf = Fp, pnb = Bp, psf = Fm, psb = Bm;
                    // every term without an in-plane x-neighbour
                    T rest = a3f * pf + a3b * pb + (b12v - b12w) * (pn - ps);
                    rest += b13v * (pef + pf - peb - pb) - b13w * (pf + pwf - pb - pwb);
                    rest += b23v * (pnf + pf - pnb - pb) - b23s * (pf + psf - pb - psb);
                    rest += b31v * (pef - pwf) - b31b * (peb - pwb);
                    rest += b32v * (pnf + pn - psf - ps) - b32b * (pn + pnb - ps - psb);
                    f -= rest;
                    if (!odd) {  // the in-plane x-neighbour terms, old values
                        const T tx = a1e * pe + a1w * pw + b12v * (pen - pes) - b12w * (pwn - pws) +
                                     b21v * (pen + pe - pwn - pw) - b21s * (pe + pes - pw - pws) +
                                     (b31v - b31b) * (pe - pw);
                        f -= tx;
                    }
                }
            }
        }
        if (act) {
            // the over-relaxation folded into the right-hand side: with T the
            // line operator of row j, T x = omega f + (1 - omega) T p_old
            // gives x = p_old + omega (T^-1 f - p_old) (identity rows keep
            // T p_old = p_old)
            G[j * RS + sc] = (ZIN ? omega * f : omega * f + (T(1) - omega) * tp) * im;
            AL[j * RS + sc] = a * im;
            // odd lanes keep 1/m here until their x-neighbour terms are added
            CP[j * RS + sc] = odd ? im : (j == ny + 1 ? T(0) : cpv);
        }
        a2s = a2v; b21s = b21v; b23s = b23v; cps = cpv;
    }
}

// Zebra second half, plain-load form of odd_x_terms: warp w adds the x-
// neighbour terms to the rows of its own segment, kXR consecutive rows per
// batch with every load of a batch issued first.  The even lanes load a1 and
// b12 for the odd lanes east of them (shuffled across), lane 0 the column
// i0-1 outside the tile (its old pressure rows and the two coefficients),
// and b21 of row j-1 is carried from the previous row.
template <typename T, bool ZIN, bool WALLS = false>
__device__ __forceinline__ void odd_x_rows(const Geom& g, const Coef<T>& c, const T* __restrict__ cpa,
                                           const T* __restrict__ pin, T omega, T* G, T* CP, int i, int k) {
    constexpr int kXR = 2;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int nj = g.ny + 2, ny = g.ny;
    const int len = (nj + nw - 1) / nw;
    const int j0 = min(w * len, nj), j1 = min(j0 + len, nj);
    const unsigned sj = (unsigned)g.sj, sk = (unsigned)g.sk, q0 = at32(g, i, 0, k);
    const bool act = i <= g.nx;
    const bool mine = act && (i & 1);
    const bool east_in = i + 1 <= g.nx;  // i+1 is a lane of this tile (odd lanes are never lane 31)
    // the new value of the east / west neighbour at row jj (old field outside the tile)
    auto EV = [&](int jj) -> T {
        if (east_in) return G[jj * 32 + lane + 1];
        return ZIN ? T(0) : ld(pin, q0 + (unsigned)jj * sj + 1u);
    };
    T b21c = T(0);  // b21 of the row before the batch
    if (mine && j0 >= 1 && j0 < j1) b21c = ld(c.b21, q0 + (unsigned)(j0 - 1) * sj);
    for (int jb = j0; jb < j1; jb += kXR) {
        T a1[kXR], a1h[kXR], b12[kXR], b12h[kXR], b21[kXR], b31[kXR], b31b[kXR], cpv[kXR], wv[kXR + 2];
#pragma unroll
        for (int u = 0; u < kXR; ++u) {
            const int j = min(jb + u, j1 - 1);
            const unsigned q = q0 + (unsigned)j * sj;
            a1[u] = act ? ld1(c.a1, q) : T(0);  // their last read in this launch
            b12[u] = act ? ld1(c.b12, q) : T(0);
            a1h[u] = act && lane == 0 ? ld(c.a1, q - 1) : T(0);
            b12h[u] = act && lane == 0 ? ld(c.b12, q - 1) : T(0);
            b21[u] = mine ? ld1(c.b21, q) : T(0);
            b31[u] = mine ? ld1(c.b31, q) : T(0);
            b31b[u] = mine ? ld1(c.b31, q - sk) : T(0);
            cpv[u] = mine ? ld1(cpa, q) : T(0);
        }
#pragma unroll
        for (int v = 0; v < kXR + 2; ++v) {  // old west column, rows jb-1 .. jb+kXR
            const int jj = jb - 1 + v;
            wv[v] = !ZIN && act && lane == 0 && jj >= 0 && jj <= ny + 1 ? ld(pin, q0 + (unsigned)jj * sj - 1u) : T(0);
        }
#pragma unroll
        for (int u = 0; u < kXR; ++u) {
            const int j = jb + u;
            if (j >= j1) break;
            T a1w = from_west(a1[u], a1h[u]);
            T b12w = from_west(b12[u], b12h[u]);
            const T b21s = u == 0 ? b21c : b21[u - 1];
            if (mine) {
                T a1e = a1[u], b12e = b12[u], b31f = b31[u], b31k = b31b[u];
                if (WALLS) {
                    if (!g.px && i == 1) a1w = b12w = T(0);
                    if (!g.px && i == g.nx) a1e = b12e = T(0);
                    if (!g.pz && k == 1) b31k = T(0);
                    if (!g.pz && k == g.nz) b31f = T(0);
                }
                const bool l0 = lane == 0;
                const T pw = l0 ? wv[u + 1] : G[j * 32 + lane - 1];
                const T pwn = j < nj - 1 ? (l0 ? wv[u + 2] : G[(j + 1) * 32 + lane - 1]) : T(0);
                const T pws = j > 0 ? (l0 ? wv[u] : G[(j - 1) * 32 + lane - 1]) : T(0);
                const T pe = EV(j);
                T tx;
                if (j == 0) {
                    tx = -b21[u] * (EV(j + 1) + pe - pwn - pw);
                } else if (j == ny + 1) {
                    tx = b21s * (pe + EV(j - 1) - pw - pws);
                } else {
                    const T pen = EV(j + 1), pes = EV(j - 1);
                    tx = a1e * pe + a1w * pw + b12e * (pen - pes) - b12w * (pwn - pws) +
                         b21[u] * (pen + pe - pwn - pw) - b21s * (pe + pes - pw - pws) + (b31f - b31k) * (pe - pw);
                }
                const T im = CP[j * 32 + lane];
                G[j * 32 + lane] -= omega * tx * im;
                CP[j * 32 + lane] = j == ny + 1 ? T(0) : cpv[u];
            }
        }
        b21c = b21[kXR - 1];
    }
}

// Phase 3 when the relaxation is folded into the right-hand side (the
// plain-load smoother): G already holds the new values; store the rows
// j = w, w+nw, ... with their periodic images.
template <typename T>
__device__ __forceinline__ void store_rows(const Geom& g, T* pout, const T* G, int i, int k) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int nj = g.ny + 2;
    for (int j = w; j < nj; j += nw) store_periodic(g, pout, i, j, k, G[j * 32 + lane]);
}

// Phase 3: relax the rows j = w, w+nw, ... of this lane's line, keep the
// new value in G (zebra: the odd-i lines read it) and store it with its
// periodic images.  The old values of a batch of kRB rows are loaded first.
template <typename T, bool ZEBRA, bool ZIN>
__device__ __forceinline__ void relax_store(const Geom& g, const T* __restrict__ pin, T* pout, T* G, T omega, int i,
                                            int k) {
    constexpr int kRB = 4;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int nj = g.ny + 2;
    for (int jb = w; jb < nj; jb += kRB * nw) {
        T old[kRB];
#pragma unroll
        for (int u = 0; u < kRB; ++u) {
            const int j = jb + u * nw;
            old[u] = (!ZIN && j < nj) ? ld(pin, g.at(i, j, k)) : T(0);
        }
#pragma unroll
        for (int u = 0; u < kRB; ++u) {
            const int j = jb + u * nw;
            if (j >= nj) break;
            const T x = G[j * 32 + lane];
            const T v = ZIN ? omega * x : old[u] + omega * (x - old[u]);
            if (ZEBRA) G[j * 32 + lane] = v;
            store_periodic(g, pout, i, j, k, v);
        }
    }
}

// ---------------------------------------------------------------------------
// eta-line relaxation (the device form of solut_sndrcv_slor,
// multigrid.f03:1939-2290, with tridag.f03).  A CTA owns 32 consecutive
// lines in i (one per lane) of one plane k, all rows j = 0..ny+1:
//   phase 1: every warp builds the rows of its own segment of the lines'
//            systems (build_rows: coalesced row loads, a sliding window of
//            pressure rows; off-line neighbours and cross terms explicit)
//            and stores g = f'/m, alpha = a/m, c' (m = b - a c'(j-1)), with
//            the over-relaxation folded in: f' = omega f + (1-omega) T p_old
//   phase 2: all warps run the two FMA recurrences per line in shared
//            memory, one row segment each (seg_thomas); the solution is the
//            relaxed line p_old + omega (T^-1 f - p_old)
//   phase 3: every warp writes its rows with the periodic images.
// JACOBI: all lines of all planes from the old field pin -> pout.
// ZEBRA : the lines with one parity of k (launch argument kpar); inside the
//         CTA the even-i lines first, then the odd-i lines, which see the new
//         even-i neighbours of the same tile (Gauss-Seidel in x and z as the
//         reference's lexicographic line SOR, Jacobi only across tile edges).
//         Phase 1 still reads every row once for all 32 lanes: the odd-i
//         lanes keep f without its six in-plane x-neighbour terms, which are
//         added after the even-i update (odd_x_rows: 4 coefficient arrays
//         and c' re-read).
//         Own-plane old values come from pin, k+-1 planes from pk (= pin for
//         the first parity, = pout for the second); output to pout.
// ZIN: pin is identically zero (first sweep of a correction); zk: pk is too.
// Shared memory: 3 arrays [ny+2][32] and the segment maps [4][warps][32].
template <typename T, bool ZEBRA, bool ZIN, bool WALLS = false>
__device__ __forceinline__ void k_line_relax_blk(Geom g, Coef<T> c, const T* __restrict__ cpa,
                                                    const T* __restrict__ pin, const T* __restrict__ pk,
                                                    T* __restrict__ pout, const T* __restrict__ rh, T omega,
                                                    int kpar, int zk, const Blk& B) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int nj = g.ny + 2;
    T* G = reinterpret_cast<T*>(smem_raw);
    T* AL = G + nj * 32;
    T* CP = AL + nj * 32;
    const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    // x: the 32-line tile (fastest, so the tiles of a plane run together and
    // read whole rows), y: the plane
    const int k = ZEBRA ? 2 * B.y + 1 + kpar : B.y + 1;
    if (k > g.nz) return;
    const int i = B.x * 32 + lane + 1;
    const bool act = i <= g.nx;
    const bool odd = ZEBRA && (i & 1);  // updated in the second half
    build_rows<T, ZEBRA, ZIN, WALLS>(g, c, cpa, pin, pk, rh, omega, zk, i, k, odd, G, AL, CP);
    T* SU = CP + nj * 32;  // segment maps of the parallel Thomas solve (forward, backward)
    T* SV = SU + nw * 32;
    T* SU2 = SV + nw * 32;
    T* SV2 = SU2 + nw * 32;
    const int nhalf = ZEBRA ? 2 : 1;
    for (int half = 0; half < nhalf; ++half) {
        const bool mine = act && (!ZEBRA || ((i & 1) == half));
        if (ZEBRA && half == 1) odd_x_rows<T, ZIN, WALLS>(g, c, cpa, pin, omega, G, CP, i, k);
        __syncthreads();
        seg_thomas(G, AL, CP, nj, mine, SU, SV, -1, SU2, SV2);
        if (mine) store_rows(g, pout, G, i, k);
        if (ZEBRA) __syncthreads();
    }
}
// the same smoother with 16 warps per CTA (shorter row segments per warp,
// for coarse levels whose few CTAs leave most SMs idle)
template <typename T, bool ZEBRA, bool ZIN, bool WALLS = false>
__global__ void __launch_bounds__(512, sizeof(T) == 4 ? 2 : 1) k_line_relax_w(Geom g, Coef<T> c, const T* __restrict__ cpa,
                                                    const T* __restrict__ pin, const T* __restrict__ pk,
                                                    T* __restrict__ pout, const T* __restrict__ rh, T omega,
                                                    int kpar, int zk) {
    k_line_relax_blk<T, ZEBRA, ZIN, WALLS>(g, c, cpa, pin, pk, pout, rh, omega, kpar, zk, hw_blk());
}
template <typename T, bool ZEBRA, bool ZIN, bool WALLS = false>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? PLES_LINE_MIN_BLOCKS : 2) k_line_relax(Geom g, Coef<T> c, const T* __restrict__ cpa,
                                                    const T* __restrict__ pin, const T* __restrict__ pk,
                                                    T* __restrict__ pout, const T* __restrict__ rh, T omega,
                                                    int kpar, int zk) {
    k_line_relax_blk<T, ZEBRA, ZIN, WALLS>(g, c, cpa, pin, pk, pout, rh, omega, kpar, zk, hw_blk());
}

// ---------------------------------------------------------------------------
// The zebra smoother on 64-line tiles (FP32, x and z periodic, nx even): the
// same sweep as k_line_relax<float, zebra> with the tile edges, where the x
// coupling is Jacobi, every 64 lines instead of 32.  A CTA of 16 warps owns
// the lines i0..i0+63 of one plane, i0 = 64 b + 1 (odd).  Warps 0-7 build
// the rows of lines i0..i0+31 and warps 8-15 those of i0+32..i0+63 (one
// line per lane, build_rows unchanged).  G / AL / CP hold 64 columns per row:
// the odd-i line i0+2l in column l, the even-i line i0+2l+1 in column 32+l.
// So each half of the zebra has one line per lane of every warp, and all 16
// warps solve it (seg_thomas over 16 row segments) with every lane busy;
// the odd-i lines' x-terms (odd_x_pairs) and the store (one pair per lane,
// 8-byte stores) likewise.

// Second half: lane l adds to line i = i0+2l (column l) its x-neighbour
// terms with the new even-i values beside it, i-1 in column 32+l-1 (lane 0:
// outside the tile, old field) and i+1 in column 32+l (new while i+1 <= nx);
// rows of this warp's segment in order with a sliding window of the
// neighbours' rows j-1, j, j+1.  Then CP(j) changes from 1/m(j) to c'(j).
// Same terms and order as odd_x_rows.
template <bool ZIN>
__device__ __forceinline__ void odd_x_pairs(const Geom& g, const Coef<float>& c, const float* __restrict__ cpa,
                                            const float* __restrict__ pin, float omega, float* G, float* CP,
                                            int i, int k) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int nj = g.ny + 2, ny = g.ny;
    const int len = (nj + nw - 1) / nw;
    const int j0 = min(w * len, nj), j1 = min(j0 + len, nj);
    if (i > g.nx || j0 >= j1) return;
    const unsigned sj = (unsigned)g.sj, sk = (unsigned)g.sk, q0 = at32(g, i, 0, k);
    const bool west_in = lane > 0, east_in = i + 1 <= g.nx;
    const int cw = 32 + lane - 1, ce = 32 + lane;
    auto WV = [&](int jj) -> float {
        if (west_in) return G[jj * 64 + cw];
        return ZIN ? 0.f : ld(pin, q0 + (unsigned)jj * sj - 1u);
    };
    auto EV = [&](int jj) -> float {
        if (east_in) return G[jj * 64 + ce];
        return ZIN ? 0.f : ld(pin, q0 + (unsigned)jj * sj + 1u);
    };
    float wm = j0 > 0 ? WV(j0 - 1) : 0.f, w0 = WV(j0), em = j0 > 0 ? EV(j0 - 1) : 0.f, e0 = EV(j0);
    float b21s = j0 >= 1 ? ld(c.b21, q0 + (unsigned)(j0 - 1) * sj) : 0.f;
    for (int j = j0; j < j1; ++j) {
        const unsigned q = q0 + (unsigned)j * sj;
        const float a1e = ld1(c.a1, q), b12e = ld1(c.b12, q), a1w = ld(c.a1, q - 1u), b12w = ld(c.b12, q - 1u);
        const float b21 = ld1(c.b21, q), b31f = ld1(c.b31, q), b31k = ld1(c.b31, q - sk), cpv = ld1(cpa, q);
        const float wp = j < nj - 1 ? WV(j + 1) : 0.f, ep = j < nj - 1 ? EV(j + 1) : 0.f;
        float tx;
        if (j == 0) {
            tx = -b21 * (ep + e0 - wp - w0);
        } else if (j == ny + 1) {
            tx = b21s * (e0 + em - w0 - wm);
        } else {
            tx = a1e * e0 + a1w * w0 + b12e * (ep - em) - b12w * (wp - wm) + b21 * (ep + e0 - wp - w0) -
                 b21s * (e0 + em - w0 - wm) + (b31f - b31k) * (e0 - w0);
        }
        const float im = CP[j * 64 + lane];
        G[j * 64 + lane] -= omega * tx * im;
        CP[j * 64 + lane] = j == ny + 1 ? 0.f : cpv;
        wm = w0; w0 = wp; em = e0; e0 = ep;
        b21s = b21;
    }
}

// the pair (i, i+1) of row j, plane k (i odd, i+1 <= nx) with its periodic
// images (store_periodic for two cells; nx even, nz >= 2)
__device__ __forceinline__ void store_pair(const Geom& g, float* p, int i, int j, int k, float vo, float ve) {
    const long long q = g.at(i, j, k);
    *reinterpret_cast<float2*>(p + q) = make_float2(vo, ve);
    const int gk = !g.pz ? -1 : (k == g.nz ? 0 : (k == 1 ? g.nz + 1 : -1));
    if (gk >= 0) *reinterpret_cast<float2*>(p + g.at(i, j, gk)) = make_float2(vo, ve);
    if (g.px && i == 1) {
        p[g.at(g.nx + 1, j, k)] = vo;
        if (gk >= 0) p[g.at(g.nx + 1, j, gk)] = vo;
    }
    if (g.px && i + 1 == g.nx) {
        p[g.at(0, j, k)] = ve;
        if (gk >= 0) p[g.at(0, j, gk)] = ve;
    }
}

// Block coordinates: x the 64-line tile, y the plane of this k parity; 16
// warps.  Shared memory: 3 arrays [ny+2][64] and the segment maps [4][16][32].
template <bool ZIN, bool FAST = false>
__device__ __forceinline__ void k_line_relax_x2_blk(Geom g, Coef<float> c, const float* __restrict__ cpa,
                                                    const float* __restrict__ pin, const float* __restrict__ pk,
                                                    float* __restrict__ pout, const float* __restrict__ rh,
                                                    float omega, int kpar, int zk, const Blk& B,
                                                    const float* __restrict__ ima = nullptr) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int nj = g.ny + 2;
    float* G = reinterpret_cast<float*>(smem_raw);
    float* AL = G + nj * 64;
    float* CP = AL + nj * 64;
    float* SU = CP + nj * 64;
    float* SV = SU + 16 * 32;
    float* SU2 = SV + 16 * 32;
    float* SV2 = SU2 + 16 * 32;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int k = 2 * B.y + 1 + kpar;
    if (k > g.nz) return;
    const int i0 = B.x * 64 + 1;
    // phase 1: line L = 32 (w / 8) + lane of the tile, row segment w % 8 of 8
    const int L = 32 * (w >> 3) + lane;
    const int ib = i0 + L;
    const int colb = (L & 1) ? 32 + (L >> 1) : (L >> 1);
    build_rows<float, true, ZIN, false, 64, FAST>(g, c, cpa, pin, pk, rh, omega, zk, ib, k, (ib & 1) != 0, G, AL,
                                                   CP, w & 7, 8, colb, ima);
    // the lane's two lines in the solve phases: io = i0 + 2 lane (odd i,
    // column lane) and io + 1 (even i, column 32 + lane)
    const int io = i0 + 2 * lane;
    __syncthreads();
    seg_thomas<float, 64>(G, AL, CP, nj, io + 1 <= g.nx, SU, SV, 32 + lane, SU2, SV2);  // the even-i lines first
    odd_x_pairs<ZIN>(g, c, cpa, pin, omega, G, CP, io, k);
    __syncthreads();
    seg_thomas<float, 64>(G, AL, CP, nj, io <= g.nx, SU, SV, lane, SU2, SV2);
    if (io <= g.nx)
        for (int j = w; j < nj; j += 16) store_pair(g, pout, io, j, k, G[j * 64 + lane], G[j * 64 + 32 + lane]);
}
template <bool ZIN>
__global__ void __launch_bounds__(512, 2) k_line_relax_x2(Geom g, Coef<float> c, const float* __restrict__ cpa,
                                                          const float* __restrict__ pin, const float* __restrict__ pk,
                                                          float* __restrict__ pout, const float* __restrict__ rh,
                                                          float omega, int kpar, int zk) {
    k_line_relax_x2_blk<ZIN>(g, c, cpa, pin, pk, pout, rh, omega, kpar, zk, hw_blk());
}
// a relaxed load of a counter that other CTAs increment (no L1 invalidation
// per poll, unlike an acquire load: the CTA sharing the SM keeps its cache)
__device__ __forceinline__ int ld_relaxed_gpu(const int* p) {
    int v;
    asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Thread 0 of an even-plane CTA: wait until the counters of the odd planes
// kb and kf reach ntx (relaxed polls with a short sleep, then one acquire
// fence), at most `polls` polls and kWaitNs; 0 and *err = 1 when it gives up.
// Not inlined: its registers are not held across the sweep that follows.
static __device__ __noinline__ int wait_odd_planes(const int* cnt, int kb, int kf, int ntx, unsigned polls, int* err) {
    unsigned long long t0 = 0;
    for (unsigned it = 0;; ++it) {
        if (ld_relaxed_gpu(cnt + kb) >= ntx && ld_relaxed_gpu(cnt + kf) >= ntx) {
            asm volatile("fence.acq_rel.gpu;" ::: "memory");
            return 1;
        }
        const unsigned long long tn = global_ns();
        if (t0 == 0) t0 = tn;
        if (it >= polls || tn - t0 > kWaitNs) {
            atomicExch(err, 1);
            return 0;
        }
        __nanosleep(128);
    }
}

// Thread 0 after the CTA's barrier that follows its stores: release the
// tile of odd plane k (k = 0: none), then count the CTA as finished; true
// for the last CTA of the launch.  The release is cumulative over the
// barrier, so it publishes the stores of every thread of the CTA; the
// acquire-release count orders it before the last CTA's reset.
static __device__ __noinline__ int finish_tile(int* sync, int k, int nblocks) {
    if (k > 0) asm volatile("red.release.gpu.global.add.s32 [%0], 1;" ::"l"(sync + 2 + k) : "memory");
    int old;
    asm volatile("atom.acq_rel.gpu.global.add.s32 %0, [%1], 1;" : "=r"(old) : "l"(sync + 1) : "memory");
    return old == nblocks - 1;
}

// Both k parities of one zebra sweep in a single launch (64-line tiles, the
// FAST row build), 2 ntx ceil(nz/2) CTAs in one dimension.  Each CTA takes a
// ticket from sync[0]: tickets below ntx ceil(nz/2) are the tiles of the
// odd planes (the first launch of the two-launch sweep), the rest those of
// the even planes.  An even-plane tile needs the new values of the odd
// planes k-1 and k+1 (plane 1 for k = nz, whose ghost image it reads): its
// first thread waits (wait_odd_planes) until their counters sync[2 + k']
// reach ntx, each odd-plane CTA adding one after its stores (finish_tile).
// A ticket is only ever held by a resident CTA and odd-plane CTAs wait for
// nothing, so every wait ends; it is bounded all the same, after which the
// CTA sets *err and leaves without writing.  Even-plane CTAs read the odd
// planes only once they are complete and no CTA rewrites them; odd-plane
// CTAs read only pin.  The last CTA to finish (sync[1] counts them) zeroes
// sync[0 .. nz+2] for the next launch.  Same arithmetic as the two launches.
template <bool ZIN>
__global__ void __launch_bounds__(512, 2) k_line_relax_x2m(Geom g, Coef<float> c, const float* __restrict__ cpa,
                                                           const float* __restrict__ ima,
                                                           const float* __restrict__ pin, float* __restrict__ pout,
                                                           const float* __restrict__ rh, float omega, int zk0,
                                                           int* __restrict__ sync, int* __restrict__ err,
                                                           unsigned polls) {
    __shared__ int s_ticket, s_ok;
    if (threadIdx.x == 0) s_ticket = atomicAdd(sync, 1);
    __syncthreads();
    const int ntx = (g.nx + 63) / 64, np0 = (g.nz + 1) / 2;
    const int t = s_ticket;
    const int kpar = t >= ntx * np0 ? 1 : 0;
    const int u = kpar ? t - ntx * np0 : t;
    Blk B;
    B.gx = ntx;
    B.gy = np0;
    B.gz = 1;
    B.x = u % ntx;
    B.y = u / ntx;
    B.z = 0;
    const int k = 2 * B.y + 1 + kpar;
    if (threadIdx.x == 0)
        s_ok = kpar && k <= g.nz ? wait_odd_planes(sync + 2, k - 1, k + 1 <= g.nz ? k + 1 : 1, ntx, polls, err) : 1;
    __syncthreads();
    if (s_ok && k <= g.nz)
        k_line_relax_x2_blk<ZIN, true>(g, c, cpa, pin, kpar ? pout : pin, pout, rh, omega, kpar, kpar ? 0 : zk0, B,
                                       ima);
    __syncthreads();
    if (threadIdx.x == 0) {
        // the ticket again from shared memory: nothing of it stays live across the sweep
        const int t2 = *(volatile int*)&s_ticket;
        const int k2 = t2 < ntx * np0 ? 2 * (t2 / ntx) + 1 : 0;
        s_ok = finish_tile(sync, k2 <= g.nz ? k2 : 0, (int)gridDim.x);
    }
    __syncthreads();
    if (s_ok)  // the last CTA: no other CTA touches the counters any more
        for (int q = threadIdx.x; q < g.nz + 3; q += blockDim.x) sync[q] = 0;
}

// the same with the pivot reciprocals of ima and the lane-parallel prefetch
template <bool ZIN>
__global__ void __launch_bounds__(512, 2) k_line_relax_x2f(Geom g, Coef<float> c, const float* __restrict__ cpa,
                                                           const float* __restrict__ ima,
                                                           const float* __restrict__ pin, const float* __restrict__ pk,
                                                           float* __restrict__ pout, const float* __restrict__ rh,
                                                           float omega, int kpar, int zk) {
    k_line_relax_x2_blk<ZIN, true>(g, c, cpa, pin, pk, pout, rh, omega, kpar, zk, hw_blk(), ima);
}

// ---------------------------------------------------------------------------
// Multicolour point SOR: the device form of solut_sndrcv_sor
// (multigrid.f03:656-1010, selected by islor = 0).  The reference sweeps the
// cells lexicographically and refreshes the ghost rows before every sweep;
// here the cells of one colour -- (i & 1) + 2 (j & 1) + 4 (k & 1) -- are
// updated at once: each of the 18 neighbours of the 19-point stencil differs
// from its cell in the parity of i, j or k, so no two cells of a colour are
// coupled (periodic directions need an even cell count, checked when the
// handle is created).  An interior cell takes pr += omega resi / den with
// resi = L(pr) - rh and den the sum of its six normal coefficients
// (multigrid.f03:840-913, scaled coefficients); a ghost cell of the wall rows
// j = 0 and ny+1 takes its homogeneous relation (mul_boun_sndrcv,
// multigrid.f03:1166-1186) solved for itself, or with FS at the top the
// free-surface relation of :1188-1222 with PrS0 = 0 (the correction's), so
// the ghost rows join the sweep where the reference runs five passes of its
// fill before it.  In place, one launch per colour; identity rows of a mask
// (no coefficients) keep their value.
template <typename T, bool FS>
__global__ void k_point_sor(Geom g, Coef<T> c, T* __restrict__ p, const T* __restrict__ rh, T omega, int colour) {
    const int ci = colour & 1, cj = (colour >> 1) & 1, ck = (colour >> 2) & 1;
    const int i = 2 * (int)(blockIdx.x * blockDim.x + threadIdx.x) + (ci ? 1 : 2);
    const int j = 2 * (int)(blockIdx.y * blockDim.y + threadIdx.y) + cj;
    const int k = 2 * (int)blockIdx.z + (ck ? 1 : 2);
    if (i > g.nx || j > g.ny + 1 || k > g.nz) return;
    const long long q = g.at(i, j, k), sj = g.sj, sk = g.sk;
    T v;
    if (j == 0) {  // bottom wall: flux through face 0 is zero
        const T a2 = c.a2[q];
        if (a2 == T(0)) return;
        const long long q1 = q + sj;
        v = p[q1] + (c.b21[q] * (p[q1 + 1] + p[q + 1] - p[q1 - 1] - p[q - 1]) +
                     c.b23[q] * (p[q1 + sk] + p[q + sk] - p[q1 - sk] - p[q - sk])) / a2;
    } else if (j == g.ny + 1) {  // top: wall (flux through face ny zero) or free surface
        const long long qn = q - sj;
        const T a2 = c.a2[qn];
        if (a2 == T(0)) return;
        const T cross = (c.b21[qn] * (p[q + 1] + p[qn + 1] - p[q - 1] - p[qn - 1]) +
                         c.b23[qn] * (p[q + sk] + p[qn + sk] - p[q - sk] - p[qn - sk])) / a2;
        v = FS ? cross - p[qn] : p[qn] - cross;
    } else {
        const T den = c.a1[q] + c.a1[q - 1] + c.a2[q] + c.a2[q - sj] + c.a3[q] + c.a3[q - sk];
        if (den == T(0)) return;
        v = p[q] + omega * cell_residual(g, c, p, rh, q) / den;
    }
    store_periodic(g, p, i, j, k, v);
}

// ---------------------------------------------------------------------------
// Residual + restriction (resid_sndrcv.f03 followed by restrict_sndrcv.f03:
// 32-53) for a coarsening ratio (rx,ry,rz) in {1,2}^3: coarse rh =
// -(1/(rx*ry*rz)) * sum of the fine residuals L(p) - rh of its children.
template <typename T>
__device__ __forceinline__ void k_resid_restrict_blk(Geom gf, Geom gc, Coef<T> c, const T* __restrict__ p,
                                 const T* __restrict__ rh, T* __restrict__ rhc, int rx, int ry, int rz, const Blk& B) {
    const int ic = B.x * blockDim.x + threadIdx.x + 1;
    const int jc = B.y * blockDim.y + threadIdx.y + 1;
    const int kc = B.z + 1;
    if (ic > gc.nx || jc > gc.ny) return;
    T s = T(0);
    for (int dk = 0; dk < rz; ++dk)
        for (int dj = 0; dj < ry; ++dj)
            for (int di = 0; di < rx; ++di)
                s += cell_residual(gf, c, p, rh, gf.at(rx * ic - di, ry * jc - dj, rz * kc - dk));
    rhc[gc.at(ic, jc, kc)] = -s / T(rx * ry * rz);
}
template <typename T>
__global__ void k_resid_restrict(Geom gf, Geom gc, Coef<T> c, const T* __restrict__ p,
                                 const T* __restrict__ rh, T* __restrict__ rhc, int rx, int ry, int rz) {
    k_resid_restrict_blk<T>(gf, gc, c, p, rh, rhc, rx, ry, rz, hw_blk());
}

// Plain residual L(p) - rh into out (interior cells).
template <typename T>
__device__ __forceinline__ void k_residual_blk(Geom g, Coef<T> c, const T* __restrict__ p, const T* __restrict__ rh,
                           T* __restrict__ out, const Blk& B) {
    const int i = B.x * blockDim.x + threadIdx.x + 1;
    const int j = B.y * blockDim.y + threadIdx.y + 1;
    const int k = B.z + 1;
    if (i > g.nx || j > g.ny) return;
    const long long q = g.at(i, j, k);
    out[q] = cell_residual(g, c, p, rh, q);
}
template <typename T>
__global__ void k_residual(Geom g, Coef<T> c, const T* __restrict__ p, const T* __restrict__ rh,
                           T* __restrict__ out) {
    k_residual_blk<T>(g, c, p, rh, out, hw_blk());
}

// Restriction alone (restrict_sndrcv.f03:32-53), summed in the reference's
// order for full coarsening.
template <typename T>
__device__ __forceinline__ void k_restrict_blk(Geom gf, Geom gc, const T* __restrict__ r, T* __restrict__ rc, int rx, int ry, int rz, const Blk& B) {
    const int ic = B.x * blockDim.x + threadIdx.x + 1;
    const int jc = B.y * blockDim.y + threadIdx.y + 1;
    const int kc = B.z + 1;
    if (ic > gc.nx || jc > gc.ny) return;
    const int id = rx * ic, jd = ry * jc, kd = rz * kc;
    T v;
    if (rx == 2 && ry == 2 && rz == 2) {
        v = r[gf.at(id, jd, kd)] + r[gf.at(id - 1, jd, kd)] + r[gf.at(id, jd - 1, kd)] +
            r[gf.at(id - 1, jd - 1, kd)] + r[gf.at(id, jd, kd - 1)] + r[gf.at(id - 1, jd, kd - 1)] +
            r[gf.at(id, jd - 1, kd - 1)] + r[gf.at(id - 1, jd - 1, kd - 1)];
        rc[gc.at(ic, jc, kc)] = -v * T(0.125);
        return;
    }
    v = T(0);
    for (int dk = 0; dk < rz; ++dk)
        for (int dj = 0; dj < ry; ++dj)
            for (int di = 0; di < rx; ++di) v += r[gf.at(id - di, jd - dj, kd - dk)];
    rc[gc.at(ic, jc, kc)] = -v / T(rx * ry * rz);
}
template <typename T>
__global__ void k_restrict(Geom gf, Geom gc, const T* __restrict__ r, T* __restrict__ rc, int rx, int ry, int rz) {
    k_restrict_blk<T>(gf, gc, r, rc, rx, ry, rz, hw_blk());
}

// ---------------------------------------------------------------------------
// Prolongation (prolong.f03:64-261): every fine cell, ghosts included, adds
// the tensor-product linear interpolation of the coarse correction; along a
// coarsened direction fine 2c gets (3/4, 1/4) of coarse (c, c+1) and fine
// 2c+1 gets (1/4, 3/4) -- the reference's (27/9/3/1)/64 weights for full
// coarsening; along an uncoarsened direction the coarse value is copied.
template <typename Tf, typename Tc>
__device__ __forceinline__ void k_prolong_blk(Geom gf, Geom gc, Tf* __restrict__ pf, const Tc* __restrict__ pc, int rx, int ry,
                          int rz, const Blk& B) {
    const int fi = B.x * blockDim.x + threadIdx.x;
    const int fj = B.y * blockDim.y + threadIdx.y;
    const int fk = B.z;
    if (fi > gf.nx + 1 || fj > gf.ny + 1) return;
    int ci[2], cj[2], ck[2];
    Tc wi[2], wj[2], wk[2];
    int ni = 1, nj = 1, nk = 1;
    if (rx == 2) { ci[0] = fi >> 1; ci[1] = ci[0] + 1; wi[0] = (fi & 1) ? Tc(0.25) : Tc(0.75); wi[1] = Tc(1) - wi[0]; ni = 2; }
    else { ci[0] = fi; wi[0] = Tc(1); }
    if (ry == 2) { cj[0] = fj >> 1; cj[1] = cj[0] + 1; wj[0] = (fj & 1) ? Tc(0.25) : Tc(0.75); wj[1] = Tc(1) - wj[0]; nj = 2; }
    else { cj[0] = fj; wj[0] = Tc(1); }
    if (rz == 2) { ck[0] = fk >> 1; ck[1] = ck[0] + 1; wk[0] = (fk & 1) ? Tc(0.25) : Tc(0.75); wk[1] = Tc(1) - wk[0]; nk = 2; }
    else { ck[0] = fk; wk[0] = Tc(1); }
    Tc s = Tc(0);
    for (int c = 0; c < nk; ++c)
        for (int b = 0; b < nj; ++b)
            for (int a = 0; a < ni; ++a) s += wi[a] * wj[b] * wk[c] * pc[gc.at(ci[a], cj[b], ck[c])];
    const long long q = gf.at(fi, fj, fk);
    pf[q] = pf[q] + Tf(s);
}
template <typename Tf, typename Tc>
__global__ void k_prolong(Geom gf, Geom gc, Tf* __restrict__ pf, const Tc* __restrict__ pc, int rx, int ry,
                          int rz) {
    k_prolong_blk<Tf, Tc>(gf, gc, pf, pc, rx, ry, rz, hw_blk());
}

// Prolongation for a level coarsened in x (rx = 2): one thread makes the
// two fine cells 2c and 2c+1, which interpolate the same coarse pair
// (c, c+1) with weights (3/4, 1/4) and (1/4, 3/4); y and z as in k_prolong.
template <typename T>
__device__ __forceinline__ void k_prolong_x2_blk(Geom gf, Geom gc, T* __restrict__ pf, const T* __restrict__ pc, int ry, int rz, const Blk& B) {
    const int c = B.x * blockDim.x + threadIdx.x;
    const int fj = B.y * blockDim.y + threadIdx.y;
    const int fk = B.z;
    if (c > gc.nx || fj > gf.ny + 1) return;
    const int cj = ry == 2 ? fj >> 1 : fj, ck = rz == 2 ? fk >> 1 : fk;
    const T wj0 = ry == 2 ? ((fj & 1) ? T(0.25) : T(0.75)) : T(1);
    const T wk0 = rz == 2 ? ((fk & 1) ? T(0.25) : T(0.75)) : T(1);
    const long long q = gc.at(c, cj, ck);
    const int oj = (int)gc.sj, ok = (int)gc.sk;
    T a = wj0 * wk0 * pc[q], bb = wj0 * wk0 * pc[q + 1];
    if (ry == 2) {
        const T w = (T(1) - wj0) * wk0;
        a += w * pc[q + oj];
        bb += w * pc[q + oj + 1];
    }
    if (rz == 2) {
        const T w = wj0 * (T(1) - wk0);
        a += w * pc[q + ok];
        bb += w * pc[q + ok + 1];
        if (ry == 2) {
            const T w2 = (T(1) - wj0) * (T(1) - wk0);
            a += w2 * pc[q + oj + ok];
            bb += w2 * pc[q + oj + ok + 1];
        }
    }
    const long long qf = gf.at(2 * c, fj, fk);
    pf[qf] = pf[qf] + (T(0.75) * a + T(0.25) * bb);
    pf[qf + 1] = pf[qf + 1] + (T(0.25) * a + T(0.75) * bb);
}
template <typename T>
__global__ void k_prolong_x2(Geom gf, Geom gc, T* __restrict__ pf, const T* __restrict__ pc, int ry, int rz) {
    k_prolong_x2_blk<T>(gf, gc, pf, pc, ry, rz, hw_blk());
}

// Full coarsening (rx = ry = rz = 2): one thread makes the 2 x 2 x 2 fine
// cells (2c..2c+1, 2cj..2cj+1, 2ck..2ck+1), which all interpolate the same
// eight coarse values (c..c+1, cj..cj+1, ck..ck+1), ghosts included; each
// fine cell gets the expressions of k_prolong_x2 in the same order.  nx, ny
// and nz even, so the pairs cover the box and the coarse reads stay in the
// coarse box.
template <typename T>
__device__ __forceinline__ void k_prolong_222_blk(Geom gf, Geom gc, T* __restrict__ pf, const T* __restrict__ pc,
                                                  const Blk& B) {
    const int c = B.x * blockDim.x + threadIdx.x;
    const int cj = B.y * blockDim.y + threadIdx.y;
    const int ck = B.z;
    if (c > gc.nx || 2 * cj > gf.ny + 1) return;
    const long long q = gc.at(c, cj, ck);
    const int oj = (int)gc.sj, ok = (int)gc.sk;
    const T p000 = pc[q], p100 = pc[q + 1], p010 = pc[q + oj], p110 = pc[q + oj + 1];
    const T p001 = pc[q + ok], p101 = pc[q + ok + 1], p011 = pc[q + oj + ok], p111 = pc[q + oj + ok + 1];
#pragma unroll
    for (int dk = 0; dk < 2; ++dk) {
        const int fk = 2 * ck + dk;
        if (fk > gf.nz + 1) break;
        const T wk0 = dk ? T(0.25) : T(0.75);
#pragma unroll
        for (int dj = 0; dj < 2; ++dj) {
            const int fj = 2 * cj + dj;
            if (fj > gf.ny + 1) break;
            const T wj0 = dj ? T(0.25) : T(0.75);
            T a = wj0 * wk0 * p000, bb = wj0 * wk0 * p100;
            {
                const T w = (T(1) - wj0) * wk0;
                a += w * p010;
                bb += w * p110;
            }
            {
                const T w = wj0 * (T(1) - wk0);
                a += w * p001;
                bb += w * p101;
                const T w2 = (T(1) - wj0) * (T(1) - wk0);
                a += w2 * p011;
                bb += w2 * p111;
            }
            // (scalar accesses: with i = 0 at element kOX = 31 of a row, the
            // pair 2c, 2c+1 starts at an odd element)
            T* f = pf + gf.at(2 * c, fj, fk);
            f[0] = f[0] + (T(0.75) * a + T(0.25) * bb);
            f[1] = f[1] + (T(0.25) * a + T(0.75) * bb);
        }
    }
}
template <typename T>
__global__ void k_prolong_222(Geom gf, Geom gc, T* __restrict__ pf, const T* __restrict__ pc) {
    k_prolong_222_blk<T>(gf, gc, pf, pc, hw_blk());
}

// ---------------------------------------------------------------------------
// Exact solve on the coarsest level: e = S r with S the (pre-computed)
// inverse of the bordered coarse system (interior cells and wall ghost rows
// as unknowns; mean of e zero, incompatible part of r absorbed).  Unknown u
// = ((k-1)*nx + (i-1))*(ny+2) + j.  Each CTA stages r in shared memory; one
// warp per row of S.
template <typename T>
__device__ __forceinline__ void k_dense_solve_blk(Geom g, const T* __restrict__ S, const T* __restrict__ rh, T* __restrict__ p, const Blk& B) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* r = reinterpret_cast<T*>(smem_raw);
    const int nj = g.ny + 2;
    const int n = g.nx * g.nz * nj;
    for (int u = threadIdx.x; u < n; u += blockDim.x) {
        const int j = u % nj, col = u / nj;
        const int i = col % g.nx + 1, k = col / g.nx + 1;
        r[u] = (j == 0 || j == nj - 1) ? T(0) : rh[g.at(i, j, k)];
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int u = B.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (u >= n) return;
    const T* row = S + (long long)u * n;
    T s = T(0);
    if (sizeof(T) == 4 && (n & 3) == 0) {
        // FP32 rows of a multiple of 4 entries start on 16-byte boundaries:
        // 16-byte loads (S is read once per solve: streaming) and four
        // independent accumulators
        const float4* row4 = reinterpret_cast<const float4*>(row);
        const float4* r4 = reinterpret_cast<const float4*>(r);
        float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
        for (int v = lane; v < (n >> 2); v += 32) {
            const float4 a = __ldcs(row4 + v), b = r4[v];
            a0 += a.x * b.x;
            a1 += a.y * b.y;
            a2 += a.z * b.z;
            a3 += a.w * b.w;
        }
        s = T((a0 + a1) + (a2 + a3));
    } else {
        for (int v = lane; v < n; v += 32) s += row[v] * r[v];
    }
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) {
        const int j = u % nj, col = u / nj;
        store_periodic(g, p, col % g.nx + 1, j, col / g.nx + 1, s);
    }
}
template <typename T>
__global__ void k_dense_solve(Geom g, const T* __restrict__ S, const T* __restrict__ rh, T* __restrict__ p) {
    k_dense_solve_blk<T>(g, S, rh, p, hw_blk());
}

}  // namespace ples
