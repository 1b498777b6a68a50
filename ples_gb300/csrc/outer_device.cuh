// outer_device.cuh -- device bodies of the FP64 outer loop (residual with
// norms, wall ghost fill, update, sums) and of the layout conversions, shared
// by the single-grid solver (ples_mg.cu) and the batched engine (batch.cu).
// Each body takes its block coordinates (Blk) explicitly.
#pragma once
#include "mg_device.cuh"

namespace ples {

constexpr int kRedThreads = 256;

__device__ __forceinline__ void block_reduce_sum_max(double& s, double& m) {
    __shared__ double ss[32], sm[32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int o = 16; o; o >>= 1) {
        s += __shfl_xor_sync(0xffffffffu, s, o);
        m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    }
    if (lane == 0) { ss[w] = s; sm[w] = m; }
    __syncthreads();
    const int nw = (blockDim.x + 31) >> 5;
    if (w == 0) {
        s = lane < nw ? ss[lane] : 0.0;
        m = lane < nw ? sm[lane] : 0.0;
        for (int o = 16; o; o >>= 1) {
            s += __shfl_xor_sync(0xffffffffu, s, o);
            m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
        }
    }
}

// Face fluxes of the 19-point operator with the scaled coefficients (the
// bracketed terms of res_dx / res_sop / res_av, resid_sndrcv.f03:85-147):
// flux through csi-face i, eta-face j, zeta-face k of cell (i,j,k).
__device__ __forceinline__ double flux_x(const Geom& g, const Coef<double>& c, const double* __restrict__ p,
                                         long long q) {
    const long long sj = g.sj, sk = g.sk;
    return c.a1[q] * (p[q + 1] - p[q]) + c.b12[q] * (p[q + 1 + sj] + p[q + sj] - p[q + 1 - sj] - p[q - sj]) +
           c.b13[q] * (p[q + 1 + sk] + p[q + sk] - p[q + 1 - sk] - p[q - sk]);
}
__device__ __forceinline__ double flux_y(const Geom& g, const Coef<double>& c, const double* __restrict__ p,
                                         long long q) {
    const long long sj = g.sj, sk = g.sk;
    return c.a2[q] * (p[q + sj] - p[q]) + c.b21[q] * (p[q + 1 + sj] + p[q + 1] - p[q - 1 + sj] - p[q - 1]) +
           c.b23[q] * (p[q + sj + sk] + p[q + sk] - p[q + sj - sk] - p[q - sk]);
}
__device__ __forceinline__ double flux_z(const Geom& g, const Coef<double>& c, const double* __restrict__ p,
                                         long long q) {
    const long long sj = g.sj, sk = g.sk;
    return c.a3[q] * (p[q + sk] - p[q]) + c.b31[q] * (p[q + 1 + sk] + p[q + 1] - p[q - 1 + sk] - p[q - 1]) +
           c.b32[q] * (p[q + sj + sk] + p[q + sj] - p[q - sj + sk] - p[q - sj]);
}

// r = b - L(x) with every face flux evaluated once and shared by its two
// cells: the csi-face flux through the lane shuffle, the eta-face flux
// through shared memory, the zeta-face flux carried while the thread walks
// KC planes in k.  The FP64 pipe is the bound of this kernel, so sharing
// roughly halves its time.  Per-block partial sum of squares and max |r|.
template <typename Ti, int KC>
__device__ __forceinline__ void k_resid_outer2_blk(Geom g, Coef<double> c, const double* __restrict__ x,
                                                      const double* __restrict__ b, Ti* __restrict__ rin,
                                                      double* __restrict__ psq, double* __restrict__ pmax, const Blk& B,
                                                      const uint8_t* __restrict__ tipo = nullptr) {
    __shared__ double sN[8][32];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int i = B.x * 32 + tx + 1, j = B.y * 8 + ty + 1;
    const int k0 = B.z * KC + 1, k1 = min(k0 + KC - 1, g.nz);
    const bool act = i <= g.nx && j <= g.ny;
    const int ic = min(i, g.nx), jc = min(j, g.ny);  // keep idle threads' loads in the box
    double s = 0.0, m = 0.0;
    double fB = flux_z(g, c, x, g.at(ic, jc, k0 - 1));
    for (int k = k0; k <= k1; ++k) {
        const long long q = g.at(ic, jc, k);
        const double fE = flux_x(g, c, x, q);
        double fW = __shfl_up_sync(0xffffffffu, fE, 1);
        if (tx == 0) fW = flux_x(g, c, x, q - 1);
        const double fN = flux_y(g, c, x, q);
        sN[ty][tx] = fN;
        __syncthreads();
        const double fS = ty > 0 ? sN[ty - 1][tx] : flux_y(g, c, x, q - g.sj);
        __syncthreads();
        const double fF = flux_z(g, c, x, q);
        if (act) {
            const double r = b[q] - ((fE - fW) + (fN - fS) + (fF - fB));
            rin[q] = Ti(r);
            s += r * r;
            if (!tipo || tipo[q] == 2) m = fmax(m, fabs(r));  // max over fluid cells (tipo >= 2)
        }
        fB = fF;
    }
    block_reduce_sum_max(s, m);
    if (threadIdx.x == 0) {
        const long long blk = ((long long)B.z * B.gy + B.y) * B.gx + B.x;
        psq[blk] = s;
        pmax[blk] = m;
    }
}
// the same residual when x is zero everywhere in the box: r = b exactly
// (every flux vanishes), written and reduced with the same block layout
template <typename Ti, int KC>
__device__ __forceinline__ void k_resid_zero_blk(Geom g, const double* __restrict__ b, Ti* __restrict__ rin,
                                                 double* __restrict__ psq, double* __restrict__ pmax, const Blk& B,
                                                 const uint8_t* __restrict__ tipo = nullptr) {
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int i = B.x * 32 + tx + 1, j = B.y * 8 + ty + 1;
    const int k0 = B.z * KC + 1, k1 = min(k0 + KC - 1, g.nz);
    double s = 0.0, m = 0.0;
    if (i <= g.nx && j <= g.ny)
        for (int k = k0; k <= k1; ++k) {
            const long long q = g.at(i, j, k);
            const double r = b[q];
            rin[q] = Ti(r);
            s += r * r;
            if (!tipo || tipo[q] == 2) m = fmax(m, fabs(r));
        }
    block_reduce_sum_max(s, m);
    if (threadIdx.x == 0) {
        const long long blk = ((long long)B.z * B.gy + B.y) * B.gx + B.x;
        psq[blk] = s;
        pmax[blk] = m;
    }
}
// flag := 1 if any element of the box is nonzero (flag cleared before)
__device__ __forceinline__ void k_box_nonzero_blk(long long n, const double* __restrict__ x, int* __restrict__ flag,
                                                  const Blk& B) {
    bool nz = false;
    for (long long q = (long long)B.x * blockDim.x + threadIdx.x; q < n; q += (long long)B.gx * blockDim.x)
        nz |= x[q] != 0.0;
    if (__syncthreads_or(nz) && threadIdx.x == 0) *flag = 1;
}
// potenziale_ibm (potenziale_ibm.f03:37-88): a solid cell (tipo 0) takes
// the mean of its IB face neighbours (tipo 1), summed from zero in the order
// i+1, i-1, j+1, j-1, k+1, k-1; with none it keeps its value.  Only solid
// cells are written and only IB cells are read, so cells are independent.
__device__ __forceinline__ void k_potenziale_ibm_blk(Geom g, const uint8_t* __restrict__ tipo, double* __restrict__ fi,
                                                     const Blk& B) {
    const int i = B.x * blockDim.x + threadIdx.x + 1;
    const int j = B.y * blockDim.y + threadIdx.y + 1;
    const int k = B.z + 1;
    if (i > g.nx || j > g.ny) return;
    const long long q = g.at(i, j, k);
    if (tipo[q] != 0) return;
    const long long nb[6] = {q + 1, q - 1, q + g.sj, q - g.sj, q + g.sk, q - g.sk};
    double s = 0.0;
    int cnt = 0;
#pragma unroll
    for (int d = 0; d < 6; ++d)
        if (tipo[nb[d]] == 1) {
            s = s + fi[nb[d]];
            ++cnt;
        }
    if (cnt) fi[q] = s / cnt;
}
// sum / sum of squares of interior cells, per-block partials
__device__ __forceinline__ void k_sum_interior_blk(Geom g, const double* __restrict__ a, int squares, double* __restrict__ psum, const Blk& B) {
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int i = B.x * 32 + tx + 1;
    const int j = B.y * (kRedThreads / 32) + ty + 1;
    const int k = B.z + 1;
    double s = 0.0, m = 0.0;
    if (i <= g.nx && j <= g.ny) {
        const double v = a[g.at(i, j, k)];
        s = squares ? v * v : v;
    }
    block_reduce_sum_max(s, m);
    if (threadIdx.x == 0)
        psum[((long long)B.z * B.gy + B.y) * B.gx + B.x] = s;
}
__device__ __forceinline__ void k_add_interior_blk(Geom g, double* __restrict__ a, double v,
                                                   const uint8_t* __restrict__ solid, const Blk& B) {
    const int i = B.x * blockDim.x + threadIdx.x + 1;
    const int j = B.y * blockDim.y + threadIdx.y + 1;
    const int k = B.z + 1;
    if (i <= g.nx && j <= g.ny) {
        const long long q = g.at(i, j, k);
        if (!solid || !solid[q]) a[q] += v;
    }
}
__device__ __forceinline__ void k_add_box_blk(Geom g, double* __restrict__ a, double v,
                                              const uint8_t* __restrict__ solid, const Blk& B) {
    const int i = B.x * blockDim.x + threadIdx.x;
    const int j = B.y * blockDim.y + threadIdx.y;
    const int k = B.z;
    if (i <= g.nx + 1 && j <= g.ny + 1) {
        const long long q = g.at(i, j, k);
        if (!solid || !solid[q]) a[q] += v;
    }
}
template <typename Te>
__device__ __forceinline__ void k_update_blk(Geom g, double* __restrict__ x, const Te* __restrict__ e, const Blk& B) {
    const int i = B.x * blockDim.x + threadIdx.x;
    const int j = B.y * blockDim.y + threadIdx.y;
    const int k = B.z;
    if (i <= g.nx + 1 && j <= g.ny + 1) {
        const long long q = g.at(i, j, k);
        x[q] += double(e[q]);
    }
}
// FP64 wall ghost rows j = 0 and ny+1 from the current field
// (mul_boun_sndrcv, multigrid.f03:1160-1186, freesurface = 0), written to a
// side buffer so that one pass is a Jacobi step (race-free, deterministic).
__device__ __forceinline__ void k_wall_compute_blk(Geom g, Coef<double> c, const double* __restrict__ p, double* __restrict__ w,
                               const double* __restrict__ cs3, const double* __restrict__ cs4, double an_dt, const Blk& B) {
    const int i = B.x * blockDim.x + threadIdx.x + 1;
    const int k = B.y * blockDim.y + threadIdx.y + 1;
    const int side = B.z;
    if (i > g.nx || k > g.nz) return;
    const long long sj = g.sj, sk = g.sk;
    const long long widx = (long long)side * g.nx * g.nz + (long long)(k - 1) * g.nx + (i - 1);
    if (side == 0) {
        const long long q0 = g.at(i, 0, k), q1 = q0 + sj;
        const double a2 = c.a2[q0];
        if (a2 == 0.0) {  // above a solid cell of an immersed-boundary mask
            w[widx] = 0.0;
            return;
        }
        double v = p[q1];
        if (cs3) v -= an_dt * cs3[(long long)(k - 1) * g.nx + (i - 1)] / a2;
        v += (c.b21[q0] * (p[q1 + 1] + p[q0 + 1] - p[q1 - 1] - p[q0 - 1]) +
              c.b23[q0] * (p[q1 + sk] + p[q0 + sk] - p[q1 - sk] - p[q0 - sk])) / a2;
        w[widx] = v;
    } else {
        const long long qt = g.at(i, g.ny + 1, k), qn = qt - sj;
        const double a2 = c.a2[qn];
        if (a2 == 0.0) {
            w[widx] = 0.0;
            return;
        }
        double v = p[qn];
        if (cs4) v += an_dt * cs4[(long long)(k - 1) * g.nx + (i - 1)] / a2;
        v -= (c.b21[qn] * (p[qt + 1] + p[qn + 1] - p[qt - 1] - p[qn - 1]) +
              c.b23[qn] * (p[qt + sk] + p[qn + sk] - p[qt - sk] - p[qn - sk])) / a2;
        w[widx] = v;
    }
}
// scatter the wall rows, including their periodic x/z images (edges and
// corners of the ghost shell)
__device__ __forceinline__ void k_wall_scatter_blk(Geom g, double* __restrict__ p, const double* __restrict__ w, const Blk& B) {
    const int i = B.x * blockDim.x + threadIdx.x;
    const int k = B.y * blockDim.y + threadIdx.y;
    const int side = B.z;
    if (i > g.nx + 1 || k > g.nz + 1) return;
    const int wi = i == 0 ? g.nx : (i == g.nx + 1 ? 1 : i);
    const int wk = k == 0 ? g.nz : (k == g.nz + 1 ? 1 : k);
    p[g.at(i, side ? g.ny + 1 : 0, k)] = w[(long long)side * g.nx * g.nz + (long long)(wk - 1) * g.nx + (wi - 1)];
}
// compact Fortran arrays <-> ghosted boxes
__device__ __forceinline__ void k_compact_to_box_blk(Geom g, int ghost, const double* __restrict__ src, double* __restrict__ dst, const Blk& B) {
    const int o = ghost ? 0 : 1;
    const int ex = ghost ? g.nx + 2 : g.nx, ey = ghost ? g.ny + 2 : g.ny, ez = ghost ? g.nz + 2 : g.nz;
    const int a = B.x * blockDim.x + threadIdx.x;
    const int b = B.y * blockDim.y + threadIdx.y;
    const int c = B.z;
    if (a >= ex || b >= ey) return;
    dst[g.at(a + o, b + o, c + o)] = src[((long long)c * ey + b) * ex + a];
    (void)ez;
}
__device__ __forceinline__ void k_box_to_compact_blk(Geom g, int ghost, const double* __restrict__ src, double* __restrict__ dst, const Blk& B) {
    const int o = ghost ? 0 : 1;
    const int ex = ghost ? g.nx + 2 : g.nx, ey = ghost ? g.ny + 2 : g.ny;
    const int a = B.x * blockDim.x + threadIdx.x;
    const int b = B.y * blockDim.y + threadIdx.y;
    const int c = B.z;
    if (a >= ex || b >= ey) return;
    dst[((long long)c * ey + b) * ex + a] = src[g.at(a + o, b + o, c + o)];
}

}  // namespace ples
