// outer_device.cuh -- device bodies of the FP64 outer loop (residual with
// norms, wall ghost fill, update, sums) and of the layout conversions, shared
// by the single-grid solver (ples_mg.cu) and the batched engine (batch.cu).
// Each body takes its block coordinates (Blk) explicitly.
#pragma once
#include "dfloat.cuh"
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
// KC planes in k.  The cross terms use the central differences of the cells
// on either side of a face, Dx = p(i+1)-p(i-1), Dy, Dz likewise: the four-
// point bracket p(i+1,j+1)+p(i,j+1)-p(i+1,j-1)-p(i,j-1) of a csi face is
// Dy(i+1) + Dy(i), and so on.  Each cell's three differences are formed
// once and passed to its neighbours (lanes, shared memory, the next plane),
// which takes about a third of the FP64 instructions out; the FP64 pipe is
// the bound of this kernel.  Per-block partial sum of squares and max |r|.
template <typename Ti, int KC>
__device__ __forceinline__ void k_resid_outer2_blk(Geom g, Coef<double> c, const double* __restrict__ x,
                                                      const double* __restrict__ b, Ti* __restrict__ rin,
                                                      double* __restrict__ psq, double* __restrict__ pmax, const Blk& B,
                                                      const uint8_t* __restrict__ tipo = nullptr) {
    __shared__ double sN[2][8][32], sDx[2][8][32], sDz[2][8][32];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int i = B.x * 32 + tx + 1, j = B.y * 8 + ty + 1;
    const int k0 = B.z * KC + 1, k1 = min(k0 + KC - 1, g.nz);
    const bool act = i <= g.nx && j <= g.ny;
    const int ic = min(i, g.nx), jc = min(j, g.ny);  // keep idle threads' loads in the box
    const long long sj = g.sj, sk = g.sk;
    double s = 0.0, m = 0.0;
    // differences of this thread's cell in plane k0 and the flux of its zeta face below
    long long q = g.at(ic, jc, k0);
    double Dx0 = x[q + 1] - x[q - 1], Dy0 = x[q + sj] - x[q - sj], Dz0 = x[q + sk] - x[q - sk];
    double fB;
    {
        const long long qb = q - sk;
        const double DxB = x[qb + 1] - x[qb - 1], DyB = x[qb + sj] - x[qb - sj];
        fB = c.a3[qb] * (x[q] - x[qb]) + c.b31[qb] * (Dx0 + DxB) + c.b32[qb] * (Dy0 + DyB);
    }
    for (int k = k0; k <= k1; ++k) {
        q = g.at(ic, jc, k);
        const int buf = k & 1;
        sDx[buf][ty][tx] = Dx0;
        sDz[buf][ty][tx] = Dz0;
        // the differences of plane k+1 (Dz only where a next step needs it)
        const long long qf = q + sk;
        const double Dx1 = x[qf + 1] - x[qf - 1], Dy1 = x[qf + sj] - x[qf - sj];
        const double Dz1 = k < k1 ? x[qf + sk] - x[q] : 0.0;
        // csi faces: east from the lane beside (lane 31 and the last column
        // form their own), west by shuffle
        double DyE = __shfl_down_sync(0xffffffffu, Dy0, 1), DzE = __shfl_down_sync(0xffffffffu, Dz0, 1);
        if (tx == 31 || i + 1 > g.nx) {  // the lane beside holds no cell of its own
            DyE = x[q + 1 + sj] - x[q + 1 - sj];
            DzE = x[q + 1 + sk] - x[q + 1 - sk];
        }
        const double fE = c.a1[q] * (x[q + 1] - x[q]) + c.b12[q] * (DyE + Dy0) + c.b13[q] * (DzE + Dz0);
        double fW = __shfl_up_sync(0xffffffffu, fE, 1);
        if (tx == 0) {
            const long long qw = q - 1;
            const double DyW = x[qw + sj] - x[qw - sj], DzW = x[qw + sk] - x[qw - sk];
            fW = c.a1[qw] * (x[q] - x[qw]) + c.b12[qw] * (Dy0 + DyW) + c.b13[qw] * (Dz0 + DzW);
        }
        __syncthreads();
        // eta faces: north with the differences of the row above (shared
        // memory; the last warp forms them), south from the warp below
        double DxN, DzN;
        if (ty < 7 && j + 1 <= g.ny) {  // the row above is a cell of this block
            DxN = sDx[buf][ty + 1][tx];
            DzN = sDz[buf][ty + 1][tx];
        } else {
            const long long qn = q + sj;
            DxN = x[qn + 1] - x[qn - 1];
            DzN = x[qn + sk] - x[qn - sk];
        }
        const double fN = c.a2[q] * (x[q + sj] - x[q]) + c.b21[q] * (DxN + Dx0) + c.b23[q] * (DzN + Dz0);
        sN[buf][ty][tx] = fN;
        __syncthreads();
        double fS;
        if (ty > 0) {
            fS = sN[buf][ty - 1][tx];
        } else {
            const long long qs = q - sj;
            const double DxS = x[qs + 1] - x[qs - 1], DzS = x[qs + sk] - x[qs - sk];
            fS = c.a2[qs] * (x[q] - x[qs]) + c.b21[qs] * (Dx0 + DxS) + c.b23[qs] * (Dz0 + DzS);
        }
        // zeta face above
        const double fF = c.a3[q] * (x[qf] - x[q]) + c.b31[q] * (Dx1 + Dx0) + c.b32[q] * (Dy1 + Dy0);
        if (act) {
            const double r = b[q] - ((fE - fW) + (fN - fS) + (fF - fB));
            rin[q] = Ti(r);
            s += r * r;
            if (!tipo || tipo[q] == 2) m = fmax(m, fabs(r));  // max over fluid cells (tipo >= 2)
        }
        fB = fF;
        Dx0 = Dx1;
        Dy0 = Dy1;
        Dz0 = Dz1;
    }
    block_reduce_sum_max(s, m);
    if (threadIdx.x == 0) {
        const long long blk = ((long long)B.z * B.gy + B.y) * B.gx + B.x;
        psq[blk] = s;
        pmax[blk] = m;
    }
}
// The same residual with the products and sums in double-float on the FP32
// pipe (dfloat.cuh): the FP64 pipe takes only the differences of x, which
// are formed in FP64 as above (the same rounding) and split into double-
// floats on the bits.  The coefficients come pre-split (cs: head and tail,
// times 2^oc); the differences are split times 2^ox and b times 2^ob, with
// ob = ox + oc, so every term and r itself are b's scale times 2^ob, near 1.
// The terms are products of a coefficient and a difference, so they are
// carried with about 2^-47 of their own size, against about 2^-53 in FP64:
// the residual agrees with the FP64 kernel's to a few units of 2^-47 of its
// largest terms.  rin = r in Ti; the partial sums of squares and maxima are
// taken in float on the scaled r and returned in FP64, unscaled.  sc[0] =
// ob and sc[1] = ox are read from device memory, so one captured graph
// serves any scaling.
template <typename Ti, int KC>
__device__ __forceinline__ void k_resid_outer2_df_blk(Geom g, Coef<float2> cs, const double* __restrict__ x,
                                                      const double* __restrict__ b, Ti* __restrict__ rin,
                                                      double* __restrict__ psq, double* __restrict__ pmax,
                                                      const Blk& B, const uint8_t* __restrict__ tipo,
                                                      const int* __restrict__ sc) {
    __shared__ dfl sN[2][8][32], sDx[2][8][32], sDz[2][8][32];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int i = B.x * 32 + tx + 1, j = B.y * 8 + ty + 1;
    const int k0 = B.z * KC + 1, k1 = min(k0 + KC - 1, g.nz);
    const bool act = i <= g.nx && j <= g.ny;
    const int ic = min(i, g.nx), jc = min(j, g.ny);  // keep idle threads' loads in the box
    const long long sj = g.sj, sk = g.sk;
    const int ob = sc[0], ox = sc[1];
    auto D = [&](long long qa, long long qz) { return df_from_double(x[qa] - x[qz], ox); };
    auto C = [&](const float2* a, long long qq) {
        const float2 v = a[qq];
        return dfl{v.x, v.y};
    };
    auto shd = [&](dfl v, int d) { return dfl{__shfl_down_sync(0xffffffffu, v.h, d), __shfl_down_sync(0xffffffffu, v.l, d)}; };
    auto shu = [&](dfl v, int d) { return dfl{__shfl_up_sync(0xffffffffu, v.h, d), __shfl_up_sync(0xffffffffu, v.l, d)}; };
    float s = 0.f, m = 0.f;
    long long q = g.at(ic, jc, k0);
    dfl Dx0 = D(q + 1, q - 1), Dy0 = D(q + sj, q - sj), Dz0 = D(q + sk, q - sk);
    dfl fB;
    {
        const long long qb = q - sk;
        const dfl DxB = D(qb + 1, qb - 1), DyB = D(qb + sj, qb - sj);
        fB = df_dot3(C(cs.a3, qb), D(q, qb), C(cs.b31, qb), df_add(Dx0, DxB), C(cs.b32, qb), df_add(Dy0, DyB));
    }
    for (int k = k0; k <= k1; ++k) {
        q = g.at(ic, jc, k);
        // this warp's rows of plane k + 1 into L2, one 128-byte line per
        // lane: lanes 0-17 the nine coefficient pairs, 18-19 b, 20-21 x one
        // plane further (the differences run a plane ahead).  Measured on
        // GB300 at 256x128x256: 394 -> 360 us per launch; two planes ahead
        // gains no more
        if (tx < 22 && k < k1) {
            const long long q0 = g.at(B.x * 32 + 1, jc, k + 1) + (tx & 1) * 16;
            const int u = tx >> 1;
            if (u < 9) {
                const float2* a = u == 0 ? cs.a1 : u == 1 ? cs.b12 : u == 2 ? cs.b13 : u == 3 ? cs.a2
                                : u == 4 ? cs.b21 : u == 5 ? cs.b23 : u == 6 ? cs.a3 : u == 7 ? cs.b31 : cs.b32;
                pf_l2(a, q0);
            } else if (u == 9) {
                pf_l2(b, q0);
            } else {
                pf_l2(x, q0 + sk);
            }
        }
        const int buf = k & 1;
        sDx[buf][ty][tx] = Dx0;
        sDz[buf][ty][tx] = Dz0;
        const long long qf = q + sk;
        const dfl Dx1 = D(qf + 1, qf - 1), Dy1 = D(qf + sj, qf - sj);
        const dfl Dz1 = k < k1 ? D(qf + sk, q) : dfl{0.f, 0.f};
        dfl DyE = shd(Dy0, 1), DzE = shd(Dz0, 1);
        if (tx == 31 || i + 1 > g.nx) {
            DyE = D(q + 1 + sj, q + 1 - sj);
            DzE = D(q + 1 + sk, q + 1 - sk);
        }
        const dfl fE = df_dot3(C(cs.a1, q), D(q + 1, q), C(cs.b12, q), df_add(DyE, Dy0), C(cs.b13, q), df_add(DzE, Dz0));
        dfl fW = shu(fE, 1);
        if (tx == 0) {
            const long long qw = q - 1;
            const dfl DyW = D(qw + sj, qw - sj), DzW = D(qw + sk, qw - sk);
            fW = df_dot3(C(cs.a1, qw), D(q, qw), C(cs.b12, qw), df_add(Dy0, DyW), C(cs.b13, qw), df_add(Dz0, DzW));
        }
        __syncthreads();
        dfl DxN, DzN;
        if (ty < 7 && j + 1 <= g.ny) {
            DxN = sDx[buf][ty + 1][tx];
            DzN = sDz[buf][ty + 1][tx];
        } else {
            const long long qn = q + sj;
            DxN = D(qn + 1, qn - 1);
            DzN = D(qn + sk, qn - sk);
        }
        const dfl fN = df_dot3(C(cs.a2, q), D(q + sj, q), C(cs.b21, q), df_add(DxN, Dx0), C(cs.b23, q), df_add(DzN, Dz0));
        sN[buf][ty][tx] = fN;
        __syncthreads();
        dfl fS;
        if (ty > 0) {
            fS = sN[buf][ty - 1][tx];
        } else {
            const long long qs = q - sj;
            const dfl DxS = D(qs + 1, qs - 1), DzS = D(qs + sk, qs - sk);
            fS = df_dot3(C(cs.a2, qs), D(q, qs), C(cs.b21, qs), df_add(Dx0, DxS), C(cs.b23, qs), df_add(Dz0, DzS));
        }
        const dfl fF = df_dot3(C(cs.a3, q), D(qf, q), C(cs.b31, q), df_add(Dx1, Dx0), C(cs.b32, q), df_add(Dy1, Dy0));
        if (act) {
            const dfl r =
                df_sub(df_from_double(b[q], ob), df_add(df_add(df_sub(fE, fW), df_sub(fN, fS)), df_sub(fF, fB)));
            if constexpr (sizeof(Ti) == 4) {
                rin[q] = df_to_float(r, ob);
            } else {  // FP64 output (the residual entry point): head and tail unscaled exactly
                rin[q] = ((double)r.h + (double)r.l) * (double)pow2f(-ob);
            }
            const float rf = __fadd_rn(r.h, r.l);
            s = __fmaf_rn(rf, rf, s);
            if (!tipo || tipo[q] == 2) m = fmaxf(m, fabsf(rf));  // max over fluid cells (tipo >= 2)
        }
        fB = fF;
        Dx0 = Dx1;
        Dy0 = Dy1;
        Dz0 = Dz1;
    }
    const double un = (double)pow2f(-ob);
    double sd = (double)s * un * un, md = (double)m * un;
    block_reduce_sum_max(sd, md);
    if (threadIdx.x == 0) {
        const long long blk = ((long long)B.z * B.gy + B.y) * B.gx + B.x;
        psq[blk] = sd;
        pmax[blk] = md;
    }
}

// split FP64 coefficients into double-floats times 2^oc
__device__ __forceinline__ void k_split_coef_blk(long long n, Coef<double> c, Coef<float2> o, int oc, const Blk& B) {
    const double* src[9] = {c.a1, c.b12, c.b13, c.a2, c.b21, c.b23, c.a3, c.b31, c.b32};
    float2* dst[9] = {o.a1, o.b12, o.b13, o.a2, o.b21, o.b23, o.a3, o.b31, o.b32};
    for (long long q = (long long)B.x * blockDim.x + threadIdx.x; q < n; q += (long long)B.gx * blockDim.x)
#pragma unroll
        for (int u = 0; u < 9; ++u) {
            const dfl v = df_from_double(src[u][q], oc);
            dst[u][q] = make_float2(v.h, v.l);
        }
}

// the largest biased FP64 exponent of the nine coefficient boxes (atomicMax
// into *out, cleared before)
__device__ __forceinline__ void k_coef_exp_max_blk(long long n, Coef<double> c, int* out, const Blk& B) {
    const double* src[9] = {c.a1, c.b12, c.b13, c.a2, c.b21, c.b23, c.a3, c.b31, c.b32};
    int e = 0;
    for (long long q = (long long)B.x * blockDim.x + threadIdx.x; q < n; q += (long long)B.gx * blockDim.x)
#pragma unroll
        for (int u = 0; u < 9; ++u) {
            const int eb = (__double2hiint(src[u][q]) >> 20) & 0x7FF;
            e = eb == 0x7FF ? e : max(e, eb);
        }
    e = __reduce_max_sync(0xffffffffu, e);
    if ((threadIdx.x & 31) == 0) atomicMax(out, e);
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
// (mul_boun_sndrcv, multigrid.f03:1160-1186), written to a side buffer so
// that one pass is a Jacobi step (race-free, deterministic).  fs: the top
// row takes the free-surface relation of multigrid.f03:1188-1222 instead,
// pr(ny+1) = 2 PrS0 - (pr(ny) - cross terms / r22), PrS0 = prs(i,k)
// ((1:nx,1:nz), or zero when null).
__device__ __forceinline__ void k_wall_compute_blk(Geom g, Coef<double> c, const double* __restrict__ p, double* __restrict__ w,
                               const double* __restrict__ cs3, const double* __restrict__ cs4, double an_dt, const Blk& B,
                               int fs = 0, const double* __restrict__ prs = nullptr) {
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
        const double cross = (c.b21[qn] * (p[qt + 1] + p[qn + 1] - p[qt - 1] - p[qn - 1]) +
                              c.b23[qn] * (p[qt + sk] + p[qn + sk] - p[qt - sk] - p[qn - sk])) / a2;
        if (fs) {
            const double s0 = prs ? prs[(long long)(k - 1) * g.nx + (i - 1)] : 0.0;
            w[widx] = s0 * 2.0 - (p[qn] - cross);
            return;
        }
        double v = p[qn];
        if (cs4) v += an_dt * cs4[(long long)(k - 1) * g.nx + (i - 1)] / a2;
        v -= cross;
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
    // the edge cells of a walled direction follow their own copy rules (side fill)
    if ((!g.px && (i == 0 || i == g.nx + 1)) || (!g.pz && (k == 0 || k == g.nz + 1))) return;
    const int wi = i == 0 ? g.nx : (i == g.nx + 1 ? 1 : i);
    const int wk = k == 0 ? g.nz : (k == g.nz + 1 ? 1 : k);
    p[g.at(i, side ? g.ny + 1 : 0, k)] = w[(long long)side * g.nx * g.nz + (long long)(wk - 1) * g.nx + (wi - 1)];
}
// ---------------------------------------------------------------------------
// Ghost cells of a walled x or z direction (ip = 1 / kp = 1): the face
// relations of mul_boun_sndrcv (multigrid.f03:1111-1158 left/right,
// 1280-1316 back/front; the flux through the wall face equals an*cs/dt) and
// its edge copies (:1360-1742).  k_side_compute evaluates every face ghost
// from the current field into w (Jacobi), k_side_scatter writes them (also
// into p2 when given: the zebra's second launch reads its k+-1 planes from
// the output buffer) with their images in a periodic direction, and
// k_side_edges sets the edge cells.  With zero set the ghosts become 0 (a
// correction that starts from zero).
// w: x walls [side][k-1][j-1] (2 ny nz), then z walls [side][j-1][i-1] (2 nx ny)
__host__ __device__ __forceinline__ long long side_cells(const Geom& g) {
    return (g.px ? 0 : 2LL * g.ny * g.nz) + (g.pz ? 0 : 2LL * g.nx * g.ny);
}
template <typename T>
__device__ __forceinline__ void k_side_compute_blk(Geom g, Coef<T> c, const T* __restrict__ p, T* __restrict__ w,
                                                   const double* __restrict__ cs1, const double* __restrict__ cs2,
                                                   const double* __restrict__ cs5, const double* __restrict__ cs6,
                                                   double an_dt, int zero, const Blk& B) {
    const long long nxw = g.px ? 0 : 2LL * g.ny * g.nz;
    const long long t = (long long)B.x * blockDim.x + threadIdx.x;
    if (t >= side_cells(g)) return;
    if (zero) {
        w[t] = T(0);
        return;
    }
    const long long sj = g.sj, sk = g.sk;
    if (t < nxw) {
        const long long per = (long long)g.ny * g.nz;
        const int side = (int)(t / per);
        const long long r = t - side * per;
        const int k = (int)(r / g.ny) + 1, j = (int)(r % g.ny) + 1;
        const long long ci = (long long)(k - 1) * g.ny + (j - 1);
        if (side == 0) {
            const long long q0 = g.at(0, j, k), q1 = q0 + 1;
            const T a = c.a1[q0];
            T v = p[q1];
            if (cs1) v -= T(an_dt * cs1[ci]) / a;
            v += (c.b12[q0] * (p[q1 + sj] + p[q0 + sj] - p[q1 - sj] - p[q0 - sj]) +
                  c.b13[q0] * (p[q1 + sk] + p[q0 + sk] - p[q1 - sk] - p[q0 - sk])) / a;
            w[t] = v;
        } else {
            const long long qt = g.at(g.nx + 1, j, k), qn = qt - 1;
            const T a = c.a1[qn];
            T v = p[qn];
            if (cs2) v += T(an_dt * cs2[ci]) / a;
            v -= (c.b12[qn] * (p[qt + sj] + p[qn + sj] - p[qt - sj] - p[qn - sj]) +
                  c.b13[qn] * (p[qt + sk] + p[qn + sk] - p[qt - sk] - p[qn - sk])) / a;
            w[t] = v;
        }
    } else {
        const long long per = (long long)g.nx * g.ny, u = t - nxw;
        const int side = (int)(u / per);
        const long long r = u - side * per;
        const int j = (int)(r / g.nx) + 1, i = (int)(r % g.nx) + 1;
        const long long ci = (long long)(j - 1) * g.nx + (i - 1);
        if (side == 0) {
            const long long q0 = g.at(i, j, 0), q1 = q0 + sk;
            const T a = c.a3[q0];
            T v = p[q1];
            if (cs5) v -= T(an_dt * cs5[ci]) / a;
            v += (c.b31[q0] * (p[q1 + 1] + p[q0 + 1] - p[q1 - 1] - p[q0 - 1]) +
                  c.b32[q0] * (p[q1 + sj] + p[q0 + sj] - p[q1 - sj] - p[q0 - sj])) / a;
            w[t] = v;
        } else {
            const long long qt = g.at(i, j, g.nz + 1), qn = qt - sk;
            const T a = c.a3[qn];
            T v = p[qn];
            if (cs6) v += T(an_dt * cs6[ci]) / a;
            v -= (c.b31[qn] * (p[qt + 1] + p[qn + 1] - p[qt - 1] - p[qn - 1]) +
                  c.b32[qn] * (p[qt + sj] + p[qn + sj] - p[qt - sj] - p[qn - sj])) / a;
            w[t] = v;
        }
    }
}
template <typename T>
__device__ __forceinline__ void k_side_scatter_blk(Geom g, T* __restrict__ p, T* __restrict__ p2,
                                                   const T* __restrict__ w, const Blk& B) {
    const long long nxw = g.px ? 0 : 2LL * g.ny * g.nz;
    const long long t = (long long)B.x * blockDim.x + threadIdx.x;
    if (t >= side_cells(g)) return;
    const T v = w[t];
    auto put = [&](int i, int j, int k) {
        const long long q = g.at(i, j, k);
        p[q] = v;
        if (p2) p2[q] = v;
    };
    if (t < nxw) {
        const long long per = (long long)g.ny * g.nz;
        const int side = (int)(t / per);
        const long long r = t - side * per;
        const int k = (int)(r / g.ny) + 1, j = (int)(r % g.ny) + 1;
        const int i = side ? g.nx + 1 : 0;
        put(i, j, k);
        if (g.pz && k == g.nz) put(i, j, 0);
        if (g.pz && k == 1) put(i, j, g.nz + 1);
    } else {
        const long long per = (long long)g.nx * g.ny, u = t - nxw;
        const int side = (int)(u / per);
        const long long r = u - side * per;
        const int j = (int)(r / g.nx) + 1, i = (int)(r % g.nx) + 1;
        const int k = side ? g.nz + 1 : 0;
        put(i, j, k);
        if (g.px && i == g.nx) put(0, j, k);
        if (g.px && i == 1) put(g.nx + 1, j, k);
    }
}
// one CTA; the stages follow the reference's order, each reading what the
// one before wrote
template <typename T>
__device__ __forceinline__ void k_side_edges_blk(Geom g, T* __restrict__ p, T* __restrict__ p2, int zero) {
    auto cp = [&](int i, int j, int k, int si, int sj2, int sk2) {
        const T v = zero ? T(0) : p[g.at(si, sj2, sk2)];
        p[g.at(i, j, k)] = v;
        if (p2) p2[g.at(i, j, k)] = v;
    };
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    if (g.pz) {  // z periodic: the horizontal square of x walls, z images included (:1420-1460)
        if (g.px) return;
        for (int k = threadIdx.x; k <= nz + 1; k += blockDim.x) {
            cp(0, ny + 1, k, 0, ny, k);
            cp(0, 0, k, 0, 1, k);
            cp(nx + 1, ny + 1, k, nx + 1, ny, k);
            cp(nx + 1, 0, k, nx + 1, 1, k);
        }
        return;
    }
    // z walls (:1628-1742): the wall planes' y edges, then their x edges, then
    // the horizontal square of x walls
    for (int t = threadIdx.x; t < 2 * nx; t += blockDim.x) {
        const int i = t % nx + 1, kg = t < nx ? 0 : nz + 1;
        cp(i, 0, kg, i, 1, kg);
        cp(i, ny + 1, kg, i, ny, kg);
    }
    __syncthreads();
    for (int t = threadIdx.x; t < 2 * (ny + 2); t += blockDim.x) {
        const int j = t % (ny + 2), kg = t < ny + 2 ? 0 : nz + 1;
        if (g.px) {
            cp(0, j, kg, nx, j, kg);
            cp(nx + 1, j, kg, 1, j, kg);
        } else {
            cp(0, j, kg, 1, j, kg);
            cp(nx + 1, j, kg, nx, j, kg);
        }
    }
    __syncthreads();
    if (!g.px)
        for (int k = 1 + threadIdx.x; k <= nz; k += blockDim.x) {
            cp(0, ny + 1, k, 1, ny + 1, k);
            cp(0, 0, k, 1, 0, k);
            cp(nx + 1, ny + 1, k, nx, ny + 1, k);
            cp(nx + 1, 0, k, nx, 0, k);
        }
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
