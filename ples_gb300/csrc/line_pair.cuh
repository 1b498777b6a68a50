// line_pair.cuh -- the zebra eta-line smoother on 64-line tiles with its row
// build done two lines per lane.
//
// Same sweep and the same arithmetic as k_line_relax_x2 (mg_device.cuh): a
// CTA owns the lines i0..i0+63 of one plane k (i0 = 64 b + 1), G / AL / CP
// hold 64 columns per row (the odd-i line i0+2l in column l, the even-i line
// i0+2l+1 in column 32+l), the even-i lines are solved first with the old
// odd-i neighbours, then the odd-i lines with the new even-i values beside
// them (odd_x_pairs), and each lane stores its pair with one 8-byte store.
//
// What differs is phase 1.  In k_line_relax_x2 each lane builds one line, so
// every row step of a warp issues one 4-byte load per array and lane, nine
// shuffles for the i-1 / i+1 neighbours and one division per line.  Here
// lane l builds both lines of its pair (i0+2l, i0+2l+1) in the same row
// step, all 64 lines of the tile per warp:
//  * every array is read with one 8-byte load per lane (the pair starts at
//    an even element, i odd and rows padded to 32 elements), so the loads,
//    their address arithmetic and the predicates are shared by two cells;
//  * the neighbour inside the pair is in the lane's own registers; only the
//    west column of the odd line and the east column of the even line come
//    from the lanes beside (eight shuffles per row step for both lines), and
//    lane 0 / the last lane load the columns just outside the tile;
//  * the pivot reciprocal 1/m(j) = 1/(b(j) - a(j) c'(j-1)) depends on the
//    coefficients only: k_line_lu stores it per level next to c', with the
//    same expressions this kernel used to evaluate, so the sweep has no
//    division and its results are bit-identical to k_line_relax_x2's;
//  * the L2 is asked for the arrays' next rows with two prefetch
//    instructions per row step (one cache line per lane) instead of one per
//    array.
// A CTA has 8 warps (each builds a segment of about (ny+2)/8 rows, then the
// same warps run the segmented Thomas solve); two CTAs share an SM.
#pragma once
#include "mg_device.cuh"

namespace ples {

__device__ __forceinline__ float2 ld2(const float* p, unsigned q) {
    return __ldg(reinterpret_cast<const float2*>(p + q));
}
// 8-byte load of an array this launch reads once (evict-first in L2)
__device__ __forceinline__ float2 ld2cs(const float* p, unsigned q) {
#if PLES_LINE_L2HINT
    return __ldcs(reinterpret_cast<const float2*>(p + q));
#else
    return __ldg(reinterpret_cast<const float2*>(p + q));
#endif
}

// rows ahead of the current one that the pair build asks the L2 for
#ifndef PLES_PAIR_PF_ROWS
#define PLES_PAIR_PF_ROWS 1
#endif

// One row equation of an eta line (the expressions and their order are those
// of build_rows): returns G, AL and CP of row j for a line whose values are
// given.  odd: the line's in-plane x-neighbour terms are added later.
struct RowIn {
    float Pm, P0, Pp, Fm, F0, Fp, Bm, B0, Bp;  // own column, rows j-1, j, j+1 of planes k, k+1, k-1
    float pef, pwf, peb, pwb;                  // i+-1 columns of planes k+-1, row j
    float pe, pw, pen, pes, pwn, pws;          // i+-1 columns of plane k (even lines only)
    float a1e, a1w, b12v, b12w, b13v, b13w;    // csi faces i+-1/2
    float a2v, a2s, b21v, b21s, b23v, b23s;    // eta faces j+1/2 (v) and j-1/2 (s)
    float a3f, a3b, b31v, b31b, b32v, b32b;    // zeta faces k+1/2 (f / v) and k-1/2 (b)
    float rhv, imv, cpv;
};

template <bool ZIN, bool ODD>
__device__ __forceinline__ void row_eq(const RowIn& r, int j, int ny, bool noneigh, float omega, float& Go,
                                       float& ALo, float& CPo) {
    float f = 0.f, a = 0.f, im = r.imv, tp = 0.f;
    if (j == 0) {
        f = noneigh ? 0.f : r.b23v * (r.Fp + r.F0 - r.Bp - r.B0);
        if (!ODD && !noneigh) f += r.b21v * (r.pen + r.pe - r.pwn - r.pw);
        a = 0.f;
        tp = r.a2v * r.P0 - r.a2v * r.Pp;
        if (r.a2v == 0.f) { f = 0.f; tp = r.P0; }  // wall row above a solid cell (im is 1)
    } else if (j == ny + 1) {
        f = noneigh ? 0.f : -(r.b23s * (r.F0 + r.Fm - r.B0 - r.Bm));
        if (!ODD && !noneigh) f -= r.b21s * (r.pe + r.pes - r.pw - r.pws);
        a = -r.a2s;
        tp = r.a2s * r.P0 - r.a2s * r.Pm;
        if (r.a2s == 0.f) { f = 0.f; tp = r.P0; }  // wall row below a solid cell
    } else {
        a = r.a2s;
        const float b = -(r.a2v + a + r.a1e + r.a1w + r.a3f + r.a3b);
        f = r.rhv;
        tp = a * r.Pm + b * r.P0 + r.a2v * r.Pp;
        if (b == 0.f) {  // solid cell of an immersed-boundary mask: identity row (im is 1)
            f = 0.f;
            a = 0.f;
            tp = r.P0;
        }
        if (!noneigh) {
            const float pn = r.Pp, ps = r.Pm, pf = r.F0, pb = r.B0;
            const float pnf = r.Fp, pnb = r.Bp, psf = r.Fm, psb = r.Bm;
            float rest = r.a3f * pf + r.a3b * pb + (r.b12v - r.b12w) * (pn - ps);
            rest += r.b13v * (r.pef + pf - r.peb - pb) - r.b13w * (pf + r.pwf - pb - r.pwb);
            rest += r.b23v * (pnf + pf - pnb - pb) - r.b23s * (pf + psf - pb - psb);
            rest += r.b31v * (r.pef - r.pwf) - r.b31b * (r.peb - r.pwb);
            rest += r.b32v * (pnf + pn - psf - ps) - r.b32b * (pn + pnb - ps - psb);
            f -= rest;
            if (!ODD) {
                const float tx = r.a1e * r.pe + r.a1w * r.pw + r.b12v * (r.pen - r.pes) - r.b12w * (r.pwn - r.pws) +
                                 r.b21v * (r.pen + r.pe - r.pwn - r.pw) - r.b21s * (r.pe + r.pes - r.pw - r.pws) +
                                 (r.b31v - r.b31b) * (r.pe - r.pw);
                f -= tx;
            }
        }
    }
    Go = (ZIN ? omega * f : omega * f + (1.f - omega) * tp) * im;
    ALo = a * im;
    CPo = ODD ? im : (j == ny + 1 ? 0.f : r.cpv);
}

// Phase 1: warp w builds the rows of its segment j0..j1-1 for all 64 lines
// of the tile, lane l the pair io = i0 + 2l, ie = io + 1.  pin: the old
// field of plane k; pk: planes k-1 and k+1; ima: 1/m per row; cpa: c'.
template <bool ZIN>
__device__ __forceinline__ void build_pairs(const Geom& g, const Coef<float>& c, const float* __restrict__ cpa,
                                            const float* __restrict__ ima, const float* __restrict__ pin,
                                            const float* __restrict__ pk, const float* __restrict__ rh,
                                            float omega, int zk, int i0, int k, float* G, float* AL, float* CP) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int nj = g.ny + 2, ny = g.ny;
    const int len = (nj + nw - 1) / nw;
    const int j0 = min(w * len, nj), j1 = min(j0 + len, nj);
    const int io = i0 + 2 * lane;
    const bool act = io <= g.nx;  // nx is even: the pair (io, io + 1) is inside the grid
    const bool wh = lane == 0;    // holds the column io - 1 west of the tile
    const bool eh = act && (lane == 31 || io + 1 == g.nx);  // holds the column io + 2 east of its pair
    const bool noneigh = ZIN && zk != 0;  // every old neighbour is zero
    const bool kz = zk != 0;              // the k+-1 planes are zero
    const unsigned sj = (unsigned)g.sj, sk = (unsigned)g.sk;
    const unsigned q0 = at32(g, io, 0, k);
    const unsigned hoff = wh ? 0xffffffffu : 2u;  // element offset of this lane's halo column from q0 (-1 or +2)
    // the L2 prefetch of a row step: lane t asks for cache line t & 1 of
    // array t >> 1 (t < 30), and in a second instruction lanes 0-5 for the
    // two lines of the three pressure planes
    const float* pfa = nullptr;
    {
        const int t = lane >> 1;
        const float* b = t == 0 ? c.a1 : t == 1 ? c.b12 : t == 2 ? c.b13 : t == 3 ? c.a2 : t == 4 ? c.b21
                       : t == 5 ? c.b23 : t == 6 || t == 9 ? c.a3 : t == 7 || t == 10 ? c.b31
                       : t == 8 || t == 11 ? c.b32 : t == 12 ? rh : t == 13 ? ima : t == 14 ? cpa : nullptr;
        if (b) pfa = b + (t >= 9 && t <= 11 ? -(long long)sk : 0LL) + 32 * (lane & 1);
    }
    const float* pfp = nullptr;
    if (lane < 6) {
        const int t = lane >> 1;
        const float* pb = t == 0 ? (ZIN ? nullptr : pin) : (kz ? nullptr : pk);
        if (pb) pfp = pb + (t == 1 ? (long long)sk : (t == 2 ? -(long long)sk : 0LL)) + sj + 32 * (lane & 1);
    }
    if ((lane & 1) && i0 + 32 > g.nx) pfa = pfp = nullptr;  // the tile's second cache line holds no line
    const unsigned qt0 = at32(g, i0, 0, k);  // the tile's row start: element i0 + 31, a multiple of 32
    auto prow = [&](const float* a, int j, unsigned qk, bool halo, float2& v, float& h) {
        v = make_float2(0.f, 0.f);
        h = 0.f;
        if (j < 0 || j > ny + 1) return;
        const unsigned q = qk + (unsigned)j * sj;
        if (act) v = ld2(a, q);
        if (halo) h = ld(a, q + hoff);
    };
    auto east = [&](float x, float h) {  // the value of column io + 2 (the lane beside's odd line)
        const float s = __shfl_down_sync(0xffffffffu, x, 1);
        return eh ? h : s;
    };
    auto west = [&](float y, float h) {  // the value of column io - 1 (the lane beside's even line)
        const float s = __shfl_up_sync(0xffffffffu, y, 1);
        return wh ? h : s;
    };
    if (j0 >= j1) return;
    // window: plane k (P), k+1 (F), k-1 (B); rows j-1 (m), j (0), j+1 (p);
    // EP* the east column of the even line in plane k; h* the halo column
    float2 Pm = {0.f, 0.f}, P0 = {0.f, 0.f}, Pp = {0.f, 0.f};
    float EPm = 0.f, EP0 = 0.f, EPp = 0.f;
    float2 Fm = {0.f, 0.f}, F0 = {0.f, 0.f}, Fp = {0.f, 0.f};
    float2 Bm = {0.f, 0.f}, B0 = {0.f, 0.f}, Bp = {0.f, 0.f};
    float hF0 = 0.f, hFp = 0.f, hB0 = 0.f, hBp = 0.f;
    if (!ZIN) {
        float hP0, hPp;
        prow(pin, j0 - 1, q0, eh, P0, hP0);
        prow(pin, j0, q0, eh, Pp, hPp);
        EP0 = east(P0.x, hP0);
        EPp = east(Pp.x, hPp);
    }
    if (!kz) {
        prow(pk, j0 - 1, q0 + sk, wh || eh, F0, hF0);
        prow(pk, j0, q0 + sk, wh || eh, Fp, hFp);
        prow(pk, j0 - 1, q0 - sk, wh || eh, B0, hB0);
        prow(pk, j0, q0 - sk, wh || eh, Bp, hBp);
    }
    // eta-face coefficients of row j-1
    float2 a2s = {0.f, 0.f}, b21s = {0.f, 0.f}, b23s = {0.f, 0.f};
    if (act && j0 >= 1) {
        const unsigned q = q0 + (unsigned)(j0 - 1) * sj;
        a2s = ld2(c.a2, q);
        b21s = ld2(c.b21, q);
        b23s = ld2(c.b23, q);
    }
    for (int j = j0; j < j1; ++j) {
        const unsigned q = q0 + (unsigned)j * sj;
        // every load of the step first: the coefficients of row j ...
        float2 a2v = {0.f, 0.f}, b21v = {0.f, 0.f}, b23v = {0.f, 0.f}, cpv = {0.f, 0.f}, imv = {0.f, 0.f};
        float2 a1v = {0.f, 0.f}, b12v = {0.f, 0.f}, b13v = {0.f, 0.f}, a3f = {0.f, 0.f}, b31v = {0.f, 0.f};
        float2 b32v = {0.f, 0.f}, a3b = {0.f, 0.f}, b31b = {0.f, 0.f}, b32b = {0.f, 0.f}, rhv = {0.f, 0.f};
        float a1h = 0.f, b12h = 0.f, b13h = 0.f;
        // (ld2cs: arrays this launch reads once; a1, b12, b21, b31 and c'
        // are read again by the odd-i pass and stay plain)
        if (act) imv = ld2cs(ima, q);
        if (act && j <= ny) {
            a2v = ld2cs(c.a2, q);
            b21v = ld2(c.b21, q);
            b23v = ld2cs(c.b23, q);
            cpv = ld2(cpa, q);
        }
        if (act && j >= 1 && j <= ny) {
            a1v = ld2(c.a1, q); b12v = ld2(c.b12, q); b13v = ld2cs(c.b13, q);
            a3f = ld2cs(c.a3, q); b31v = ld2(c.b31, q); b32v = ld2cs(c.b32, q);
            a3b = ld2cs(c.a3, q - sk); b31b = ld2(c.b31, q - sk); b32b = ld2cs(c.b32, q - sk);
            rhv = ld2cs(rh, q);
            if (wh) { a1h = ld(c.a1, q - 1u); b12h = ld(c.b12, q - 1u); b13h = ld(c.b13, q - 1u); }
        }
        // ... then the pressure rows j+1 of the three planes
        Pm = P0; P0 = Pp;
        EPm = EP0; EP0 = EPp;
        Fm = F0; F0 = Fp; hF0 = hFp;
        Bm = B0; B0 = Bp; hB0 = hBp;
        float hPp = 0.f;
        if (!ZIN) prow(pin, j + 1, q0, eh, Pp, hPp);
        if (!kz) {
            prow(pk, j + 1, q0 + sk, wh || eh, Fp, hFp);
            prow(pk, j + 1, q0 - sk, wh || eh, Bp, hBp);
        }
#if PLES_PAIR_PF_ROWS > 0
        if (j + PLES_PAIR_PF_ROWS < j1) {
            const unsigned qn = qt0 + (unsigned)(j + PLES_PAIR_PF_ROWS) * sj;
            if (pfa) pf_l2(pfa, qn);
            if (pfp && j + PLES_PAIR_PF_ROWS + 1 < nj) pf_l2(pfp, qn);
        }
#endif
        if (!ZIN) EPp = east(Pp.x, hPp);
        // the lanes beside: west column of the odd line, east of the even one
        const float a1w_o = west(a1v.y, a1h), b12w_o = west(b12v.y, b12h), b13w_o = west(b13v.y, b13h);
        const float wF0 = west(F0.y, hF0), eF0 = east(F0.x, hF0);
        const float wB0 = west(B0.y, hB0), eB0 = east(B0.x, hB0);
        if (act) {
            RowIn r;
            // the odd-i line io (column lane)
            r.Pm = Pm.x; r.P0 = P0.x; r.Pp = Pp.x;
            r.Fm = Fm.x; r.F0 = F0.x; r.Fp = Fp.x;
            r.Bm = Bm.x; r.B0 = B0.x; r.Bp = Bp.x;
            r.pef = F0.y; r.pwf = wF0; r.peb = B0.y; r.pwb = wB0;
            r.pe = r.pw = r.pen = r.pes = r.pwn = r.pws = 0.f;
            r.a1e = a1v.x; r.a1w = a1w_o; r.b12v = b12v.x; r.b12w = b12w_o; r.b13v = b13v.x; r.b13w = b13w_o;
            r.a2v = a2v.x; r.a2s = a2s.x; r.b21v = b21v.x; r.b21s = b21s.x; r.b23v = b23v.x; r.b23s = b23s.x;
            r.a3f = a3f.x; r.a3b = a3b.x; r.b31v = b31v.x; r.b31b = b31b.x; r.b32v = b32v.x; r.b32b = b32b.x;
            r.rhv = rhv.x; r.imv = imv.x; r.cpv = cpv.x;
            float go, alo, cpo;
            row_eq<ZIN, true>(r, j, ny, noneigh, omega, go, alo, cpo);
            G[j * 64 + lane] = go;
            AL[j * 64 + lane] = alo;
            CP[j * 64 + lane] = cpo;
            // the even-i line io + 1 (column 32 + lane)
            r.Pm = Pm.y; r.P0 = P0.y; r.Pp = Pp.y;
            r.Fm = Fm.y; r.F0 = F0.y; r.Fp = Fp.y;
            r.Bm = Bm.y; r.B0 = B0.y; r.Bp = Bp.y;
            r.pef = eF0; r.pwf = F0.x; r.peb = eB0; r.pwb = B0.x;
            r.pe = EP0; r.pw = P0.x; r.pen = EPp; r.pes = EPm; r.pwn = Pp.x; r.pws = Pm.x;
            r.a1e = a1v.y; r.a1w = a1v.x; r.b12v = b12v.y; r.b12w = b12v.x; r.b13v = b13v.y; r.b13w = b13v.x;
            r.a2v = a2v.y; r.a2s = a2s.y; r.b21v = b21v.y; r.b21s = b21s.y; r.b23v = b23v.y; r.b23s = b23s.y;
            r.a3f = a3f.y; r.a3b = a3b.y; r.b31v = b31v.y; r.b31b = b31b.y; r.b32v = b32v.y; r.b32b = b32b.y;
            r.rhv = rhv.y; r.imv = imv.y; r.cpv = cpv.y;
            row_eq<ZIN, false>(r, j, ny, noneigh, omega, go, alo, cpo);
            G[j * 64 + 32 + lane] = go;
            AL[j * 64 + 32 + lane] = alo;
            CP[j * 64 + 32 + lane] = cpo;
        }
        a2s = a2v; b21s = b21v; b23s = b23v;
    }
}

// Block coordinates: x the 64-line tile, y the plane of this k parity; 8
// warps.  Shared memory: 3 arrays [ny+2][64] and the segment maps
// [4][16][32] (as k_line_relax_x2).
template <bool ZIN>
__device__ __forceinline__ void k_line_relax_p2_blk(Geom g, Coef<float> c, const float* __restrict__ cpa,
                                                    const float* __restrict__ ima, const float* __restrict__ pin,
                                                    const float* __restrict__ pk, float* __restrict__ pout,
                                                    const float* __restrict__ rh, float omega, int kpar, int zk,
                                                    const Blk& B) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int nj = g.ny + 2;
    float* G = reinterpret_cast<float*>(smem_raw);
    float* AL = G + nj * 64;
    float* CP = AL + nj * 64;
    float* SU = CP + nj * 64;
    float* SV = SU + 16 * 32;
    float* SU2 = SV + 16 * 32;
    float* SV2 = SU2 + 16 * 32;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int k = 2 * B.y + 1 + kpar;
    if (k > g.nz) return;
    const int i0 = B.x * 64 + 1;
    build_pairs<ZIN>(g, c, cpa, ima, pin, pk, rh, omega, zk, i0, k, G, AL, CP);
    const int io = i0 + 2 * lane;
    __syncthreads();
    seg_thomas<float, 64>(G, AL, CP, nj, io + 1 <= g.nx, SU, SV, 32 + lane, SU2, SV2);  // the even-i lines first
    odd_x_pairs<ZIN>(g, c, cpa, pin, omega, G, CP, io, k);
    __syncthreads();
    seg_thomas<float, 64>(G, AL, CP, nj, io <= g.nx, SU, SV, lane, SU2, SV2);
    if (io <= g.nx)
        for (int j = w; j < nj; j += nw) store_pair(g, pout, io, j, k, G[j * 64 + lane], G[j * 64 + 32 + lane]);
}
template <bool ZIN>
__global__ void __launch_bounds__(256, 2) k_line_relax_p2(Geom g, Coef<float> c, const float* __restrict__ cpa,
                                                          const float* __restrict__ ima,
                                                          const float* __restrict__ pin, const float* __restrict__ pk,
                                                          float* __restrict__ pout, const float* __restrict__ rh,
                                                          float omega, int kpar, int zk) {
    k_line_relax_p2_blk<ZIN>(g, c, cpa, ima, pin, pk, pout, rh, omega, kpar, zk, hw_blk());
}

}  // namespace ples
