// line_tma.cuh -- the zebra eta-line smoother with its row data staged by TMA.
//
// Same algorithm and arithmetic as k_line_relax<float, true, ZIN>
// (mg_device.cuh): a CTA owns 32 lines in i of one plane k, builds every row
// of their tridiagonal systems, solves them in shared memory and writes the
// relaxed lines.  Here the row build (phase 1) reads shared memory: thread 0
// streams the rows in chunks of kRC with cp.async.bulk.tensor boxes (p of
// planes k-1, k, k+1, the nine face coefficients, rh and the LU factor c')
// into kNB rotating buffers, each completing on its own mbarrier.  The
// copies of the next chunks overlap the arithmetic of the current one and
// about 60 KB per CTA stay in flight without occupying per-thread load
// slots, which is what bounded the plain-load kernel (many outstanding L2
// misses per SM are needed to cover HBM latency).
//
// Box origins in x are element i0+28 (cell i0-3) for the boxes that need the
// i-1 / i+1 neighbours and element i0+32 (cell i0+1) for the others: both
// multiples of 4 floats, so every copy starts on a 16-byte boundary.  Rows
// and planes outside the box (j = -1, j > ny+1, x past the row pitch) read
// as zero and are never used.
#pragma once
#include "mg_device.cuh"
#include "tma.cuh"

namespace ples {

constexpr int kRC = 8;  // rows per chunk (one per warp)
constexpr int kNB = 3;  // chunk buffers in flight

// Tensor maps of one level (3-D: x = element in the padded row, y = j, z = k)
struct LineMaps {
    CUtensorMap pA, pB;        // the level's two pressure buffers, box 40 x (kRC+2) x 1
    CUtensorMap a1, b12, b13;  // csi faces, box 36 x kRC x 1
    CUtensorMap a2, b21, b23;  // eta faces, box 32 x (kRC+1) x 1
    CUtensorMap a3, b31, b32;  // zeta faces, box 32 x kRC x 2 (planes k-1, k)
    CUtensorMap rh;            // box 32 x kRC x 1
    CUtensorMap cp;            // box 32 x (kRC+1) x 1
};

// float offsets of the boxes inside one chunk buffer (each 128-B aligned)
struct ChunkLayout {
    static constexpr int P = 416;  // (kRC+2) x 40 = 400, padded
    static constexpr int X = 288;  // kRC x 36
    static constexpr int Y = 288;  // (kRC+1) x 32
    static constexpr int Z = 512;  // 2 x kRC x 32
    static constexpr int R = 256;  // kRC x 32
    static constexpr int C = 288;  // (kRC+1) x 32
    static constexpr int P0 = 0, PM = P, PP = 2 * P;
    static constexpr int X1 = 3 * P, X2 = X1 + X, X3 = X2 + X;
    static constexpr int Y1 = X3 + X, Y2 = Y1 + Y, Y3 = Y2 + Y;
    static constexpr int Z1 = Y3 + Y, Z2 = Z1 + Z, Z3 = Z2 + Z;
    static constexpr int RH = Z3 + Z, CPB = RH + R;
    static constexpr int SIZE = CPB + C;  // floats per buffer
};
static_assert(ChunkLayout::SIZE % 32 == 0, "chunk buffers must stay 128-B aligned");
static_assert(kRC == 8, "one row per warp of a 256-thread CTA");

// dynamic shared memory of k_line_relax_tma for a level with ny rows
__host__ __device__ constexpr size_t line_tma_smem(int ny) {
    return (size_t)kNB * ChunkLayout::SIZE * 4 + 3 * (size_t)(ny + 2) * 32 * 4 + 8 * kNB;
}

// bytes one chunk's boxes deliver (out-of-range elements count as well)
__host__ __device__ constexpr unsigned line_tma_chunk_bytes(bool zin, bool zk) {
    return (zin ? 0u : 40u * (kRC + 2) * 4u) + (zk ? 0u : 2u * 40u * (kRC + 2) * 4u) + 3u * 36u * kRC * 4u +
           3u * 32u * (kRC + 1) * 4u + 3u * 32u * kRC * 2u * 4u + 32u * kRC * 4u + 32u * (kRC + 1) * 4u;
}

// Zebra half-sweep over the planes k = 2*blockIdx.x + 1 + kpar, 32 lines per
// CTA (blockIdx.y).  pin is the old field (map pA if pin_is_a, else pB), pk
// holds the planes k-1 and k+1 (map by pk_is_a); zk: those planes are zero.
// A transfer that does not complete within the bounded wait (wait_polls
// polls of its mbarrier, and 2 s) sets *err and the CTA leaves without
// writing, after a second bounded wait (the default limits) for the copies
// it still has in flight.
template <bool ZIN>
__global__ void __launch_bounds__(256) k_line_relax_tma(const __grid_constant__ LineMaps maps, Geom g,
                                                        Coef<float> c, const float* __restrict__ cpa,
                                                        const float* __restrict__ pin, float* pout, float omega,
                                                        int kpar, int zk, int pin_is_a, int pk_is_a,
                                                        int* __restrict__ err, unsigned wait_polls) {
    extern __shared__ __align__(128) unsigned char smem_tma[];
    float* buf = reinterpret_cast<float*>(smem_tma);
    const int nj = g.ny + 2, ny = g.ny;
    float* G = buf + kNB * ChunkLayout::SIZE;
    float* AL = G + nj * 32;
    float* CP = AL + nj * 32;
    uint64_t* bar = reinterpret_cast<uint64_t*>(CP + nj * 32);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int k = 2 * blockIdx.x + 1 + kpar;
    if (k > g.nz) return;
    if (*reinterpret_cast<volatile int*>(err)) return;  // an earlier CTA gave up: skip quickly
    if (smem_u32(buf) & 127u) {  // TMA destinations need 128-byte alignment
        if (threadIdx.x == 0) atomicExch(err, 2);
        return;
    }
    const int i0 = blockIdx.y * 32;
    const int i = i0 + lane + 1;
    const bool act = i <= g.nx;
    const bool odd = i & 1;  // updated in the second half
    const int nchunk = (nj + kRC - 1) / kRC;
    const CUtensorMap* mpin = pin_is_a ? &maps.pA : &maps.pB;
    const CUtensorMap* mpk = pk_is_a ? &maps.pA : &maps.pB;
    const unsigned bytes = line_tma_chunk_bytes(ZIN, zk != 0);
    const int xp = i0 + 28, xc = i0 + 32;
    auto issue = [&](int ch) {
        float* b = buf + (ch % kNB) * ChunkLayout::SIZE;
        uint64_t* br = bar + (ch % kNB);
        const int j0 = ch * kRC;
        mbar_arrive_expect_tx(br, bytes);
        if (!ZIN) tma_load_3d(b + ChunkLayout::P0, mpin, xp, j0 - 1, k, br);
        if (!zk) {
            tma_load_3d(b + ChunkLayout::PM, mpk, xp, j0 - 1, k - 1, br);
            tma_load_3d(b + ChunkLayout::PP, mpk, xp, j0 - 1, k + 1, br);
        }
        tma_load_3d(b + ChunkLayout::X1, &maps.a1, xp, j0, k, br);
        tma_load_3d(b + ChunkLayout::X2, &maps.b12, xp, j0, k, br);
        tma_load_3d(b + ChunkLayout::X3, &maps.b13, xp, j0, k, br);
        tma_load_3d(b + ChunkLayout::Y1, &maps.a2, xc, j0 - 1, k, br);
        tma_load_3d(b + ChunkLayout::Y2, &maps.b21, xc, j0 - 1, k, br);
        tma_load_3d(b + ChunkLayout::Y3, &maps.b23, xc, j0 - 1, k, br);
        tma_load_3d(b + ChunkLayout::Z1, &maps.a3, xc, j0, k - 1, br);
        tma_load_3d(b + ChunkLayout::Z2, &maps.b31, xc, j0, k - 1, br);
        tma_load_3d(b + ChunkLayout::Z3, &maps.b32, xc, j0, k - 1, br);
        tma_load_3d(b + ChunkLayout::RH, &maps.rh, xc, j0, k, br);
        tma_load_3d(b + ChunkLayout::CPB, &maps.cp, xc, j0 - 1, k, br);
    };
    if (threadIdx.x == 0) {
        for (int q = 0; q < kNB; ++q) mbar_init(bar + q, 1);
        mbar_fence_init();
    }
    __syncthreads();
    if (threadIdx.x == 0)
        for (int ch = 0; ch < kNB && ch < nchunk; ++ch) issue(ch);
    const bool noneigh = ZIN && zk;  // every old neighbour is zero
    int failed = -1;
    for (int ch = 0; ch < nchunk; ++ch) {
        const float* b = buf + (ch % kNB) * ChunkLayout::SIZE;
        const bool ok = mbar_wait(bar + (ch % kNB), (unsigned)((ch / kNB) & 1), wait_polls);
        if (__syncthreads_or(!ok)) { failed = ch; break; }
        const int jj = w;  // row of this warp inside the chunk
        const int j = ch * kRC + jj;
        if (act && j < nj) {
            const int cx = lane + 4;  // column of cell i in the 40- and 36-wide boxes
            auto P0 = [&](int di, int dj) { return ZIN ? 0.f : b[ChunkLayout::P0 + (jj + 1 + dj) * 40 + cx + di]; };
            auto PM = [&](int di, int dj) { return zk ? 0.f : b[ChunkLayout::PM + (jj + 1 + dj) * 40 + cx + di]; };
            auto PP = [&](int di, int dj) { return zk ? 0.f : b[ChunkLayout::PP + (jj + 1 + dj) * 40 + cx + di]; };
            const float* X1 = b + ChunkLayout::X1 + jj * 36;
            const float* X2 = b + ChunkLayout::X2 + jj * 36;
            const float* X3 = b + ChunkLayout::X3 + jj * 36;
            const float* Y1 = b + ChunkLayout::Y1;
            const float* Y2 = b + ChunkLayout::Y2;
            const float* Y3 = b + ChunkLayout::Y3;
            const float* Z1 = b + ChunkLayout::Z1;
            const float* Z2 = b + ChunkLayout::Z2;
            const float* Z3 = b + ChunkLayout::Z3;
            const int yj = (jj + 1) * 32 + lane, yjm = jj * 32 + lane;   // eta faces j, j-1
            const int zf = (kRC + jj) * 32 + lane, zb = jj * 32 + lane;  // zeta faces k, k-1
            const float cpm = b[ChunkLayout::CPB + jj * 32 + lane];      // c' of row j-1
            float f, a, im;
            if (j == 0) {
                f = noneigh ? 0.f : Y3[yj] * (PP(0, 1) + PP(0, 0) - PM(0, 1) - PM(0, 0));
                if (!odd && !noneigh) f += Y2[yj] * (P0(1, 1) + P0(1, 0) - P0(-1, 1) - P0(-1, 0));
                a = 0.f;
                im = 1.f / Y1[yj];
                if (Y1[yj] == 0.f) { im = 1.f; f = 0.f; }  // wall row above a solid cell
            } else if (j == ny + 1) {
                const float a2 = Y1[yjm];  // face ny
                f = noneigh ? 0.f : -(Y3[yjm] * (PP(0, 0) + PP(0, -1) - PM(0, 0) - PM(0, -1)));
                if (!odd && !noneigh) f -= Y2[yjm] * (P0(1, 0) + P0(1, -1) - P0(-1, 0) - P0(-1, -1));
                a = -a2;
                im = 1.f / (a2 - a * cpm);
                if (a2 == 0.f) { im = 1.f; f = 0.f; }  // wall row below a solid cell
            } else {
                const float a1e = X1[cx], a1w = X1[cx - 1];
                const float a3f = Z1[zf], a3b = Z1[zb];
                const float a2 = Y1[yj];
                a = Y1[yjm];
                const float bd = -(a2 + a + a1e + a1w + a3f + a3b);
                im = 1.f / (bd - a * cpm);
                f = b[ChunkLayout::RH + jj * 32 + lane];
                if (bd == 0.f) {  // solid cell of an immersed-boundary mask: identity row
                    im = 1.f;
                    f = 0.f;
                    a = 0.f;
                }
                if (!noneigh) {
                    const float pn = P0(0, 1), ps = P0(0, -1);
                    const float pf = PP(0, 0), pb = PM(0, 0);
                    const float pef = PP(1, 0), peb = PM(1, 0), pwf = PP(-1, 0), pwb = PM(-1, 0);
                    const float pnf = PP(0, 1), pnb = PM(0, 1), psf = PP(0, -1), psb = PM(0, -1);
                    const float b12 = X2[cx], b12w = X2[cx - 1];
                    const float b31 = Z2[zf], b31b = Z2[zb];
                    // every term without an in-plane x-neighbour
                    float rest = a3f * pf + a3b * pb + (b12 - b12w) * (pn - ps);
                    rest += X3[cx] * (pef + pf - peb - pb) - X3[cx - 1] * (pf + pwf - pb - pwb);
                    rest += Y3[yj] * (pnf + pf - pnb - pb) - Y3[yjm] * (pf + psf - pb - psb);
                    rest += b31 * (pef - pwf) - b31b * (peb - pwb);
                    rest += Z3[zf] * (pnf + pn - psf - ps) - Z3[zb] * (pn + pnb - ps - psb);
                    f -= rest;
                    if (!odd) {  // the in-plane x-neighbour terms, old values
                        const float pe = P0(1, 0), pw = P0(-1, 0);
                        const float pen = P0(1, 1), pes = P0(1, -1), pwn = P0(-1, 1), pws = P0(-1, -1);
                        const float b21 = Y2[yj], b21s = Y2[yjm];
                        const float tx = a1e * pe + a1w * pw + b12 * (pen - pes) - b12w * (pwn - pws) +
                                         b21 * (pen + pe - pwn - pw) - b21s * (pe + pes - pw - pws) +
                                         (b31 - b31b) * (pe - pw);
                        f -= tx;
                    }
                }
            }
            G[j * 32 + lane] = f * im;
            AL[j * 32 + lane] = a * im;
            // odd lanes keep 1/m here until their x-neighbour terms are added
            CP[j * 32 + lane] = odd ? im : (j == ny + 1 ? 0.f : b[ChunkLayout::CPB + (jj + 1) * 32 + lane]);
        }
        __syncthreads();  // every thread is done with buffer ch % kNB
        if (threadIdx.x == 0 && ch + kNB < nchunk) {
            fence_proxy_async();
            issue(ch + kNB);
        }
    }
    if (failed >= 0) {
        // chunks failed .. failed+kNB-1 may still be in flight: wait for them
        // (bounded) before the shared memory is released, then report
        if (threadIdx.x == 0) {
            for (int ch = failed; ch < nchunk && ch < failed + kNB; ++ch)
                mbar_wait(bar + (ch % kNB), (unsigned)((ch / kNB) & 1));
            atomicExch(err, 1);
        }
        return;
    }
    float* SU = buf;  // segment maps of the parallel Thomas solve (chunk buffers are free now)
    float* SV = SU + nw * 32;
    for (int half = 0; half < 2; ++half) {
        const bool mine = act && ((i & 1) == half);
        if (half == 1 && mine) odd_x_terms<float, ZIN>(g, c, cpa, pin, G, CP, i, k);
        __syncthreads();
        seg_thomas(G, AL, CP, nj, mine, SU, SV);
        if (mine) relax_store<float, true, ZIN>(g, pin, pout, G, omega, i, k);
        __syncthreads();
    }
}

}  // namespace ples
