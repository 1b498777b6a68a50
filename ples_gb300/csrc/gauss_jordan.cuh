// gauss_jordan.cuh -- dense inverse of the coarsest level by blocked
// Gauss-Jordan elimination with partial pivoting.
//
// K (m x m, row-major) is reduced to a row-permuted diagonal while the same
// row operations build the inverse.  The pivot rows stay where they are and
// unscaled: row p_c keeps its pivot K(p_c, c), and the inverse's row c is
// row p_c of the result over that pivot (k_gj_extract).  S holds the result
// with its columns in pivot order: before elimination step c, S(:, c) is the
// unit vector of row p_c.  Step c takes, for every row r other than p_c,
// f = K(r, c) / K(p_c, c) and row r -= f row p_c (in K and S alike).
//
// Blocked by panels of B pivot columns [c0, c1).  A panel's steps are run on
// its own K columns only (k_gjb_panel, one CTA, the panel in shared memory),
// recording the multipliers F(r, c - c0) (zero for the step's pivot row).
// The product T of the panel's B eliminations is then applied to every other
// column v at once: T v = v - F w, with w_c = v(p_c) - sum_{c' < c}
// F(p_c, c' - c0) w_c' (the pivot row's value when step c reads it), a unit
// lower-triangular solve (at the end of k_gjb_panel) and a rank-B update
// (k_gjb_update).  The
// columns it applies to are those of S up to c1 (the panel's own start as
// the unit vectors of their pivot rows: T leaves a unit vector alone until
// its step) and those of K from c1 on: column index d < c1 in S, d >= c1 in
// K.  The pivots are those of the unblocked elimination (each panel column
// is fully updated before its pivot is chosen); only the rounding order of
// the updates differs.
//
// The pivot of column c is the unused row with the largest |K(r, c)|, ties
// to the lowest row; none above zero marks the system singular (*bad = 1).
#pragma once
#include <cuda_runtime.h>

namespace ples {

// panel width: FP32 panels of up to 3073 rows fit the 227 KB of shared
// memory of one CTA at 16 columns, FP64 at 8
template <typename R>
struct GjPanel {
    static constexpr int B = sizeof(R) == 4 ? 16 : 8;
};

template <typename R>
__host__ __device__ constexpr size_t gjb_panel_smem(int m) {
    return (size_t)m * (GjPanel<R>::B + 1) * sizeof(R);
}

// The panel's B steps in one CTA of 1024 threads: K(:, c0 .. c0+nb) into
// shared memory (rows padded to B + 1), thread t owning rows t + 1024 k.
// Each step eliminates its column and, in the same pass, every owner offers
// its unused rows' |K(r, c + 1)| for the next pivot; a warp reduces its
// offers, and after one barrier every warp reduces the 32 warp offers
// itself (the offer buffers alternate between steps, so one barrier per
// step suffices).  Then: the multipliers in F (B x m, F(r, c) at c m + r),
// the panel back in K, used[] and pivrow[] updated, S(p_c, c) = 1 for the
// panel's columns (S is zero there), and w = L^-1 v(p_c0 .. p_c1-1) for
// every column d < m (S below c1, K from c1 on) into W (B x m),
// L(c, c') = F(p_c, c') for c' < c.
constexpr int kGjThreads = 1024, kGjRows = 4;  // rows per thread: m <= 4096
template <typename R>
__global__ void __launch_bounds__(kGjThreads, 1) k_gjb_panel(R* __restrict__ K, R* __restrict__ S, R* __restrict__ F,
                                                          R* __restrict__ W, int m, int c0, int nb,
                                                          int* __restrict__ used, int* __restrict__ pivrow,
                                                          int* __restrict__ bad) {
    constexpr int B = GjPanel<R>::B, LD = B + 1;
    extern __shared__ __align__(16) unsigned char smem_gj[];
    R* P = reinterpret_cast<R*>(smem_gj);
    __shared__ R s_best[2][32];
    __shared__ int s_row[2][32];
    __shared__ int s_p[B];
    __shared__ R s_L[B][B];
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    for (int e = tid; e < m * nb; e += kGjThreads) {
        const int r = e / nb, c = e - r * nb;
        P[r * LD + c] = K[(size_t)r * m + c0 + c];
    }
    unsigned um = 0;  // bit k: row tid + 1024 k is a pivot row already
#pragma unroll
    for (int k = 0; k < kGjRows; ++k) {
        const int r = tid + k * kGjThreads;
        if (r < m && used[r]) um |= 1u << k;
    }
    auto better = [](R v2, int r2, R v, int r) { return r2 >= 0 && (r < 0 || v2 > v || (v2 == v && r2 < r)); };
    // the block's pivot for a column from every thread's offer (best, br)
    auto reduce = [&](R best, int br, int buf) {
        for (int o = 16; o; o >>= 1) {
            const R v2 = __shfl_xor_sync(0xffffffffu, best, o);
            const int r2 = __shfl_xor_sync(0xffffffffu, br, o);
            if (better(v2, r2, best, br)) { best = v2; br = r2; }
        }
        if (lane == 0) { s_best[buf][wid] = best; s_row[buf][wid] = br; }
        __syncthreads();
        constexpr int nw = kGjThreads / 32;
        best = lane < nw ? s_best[buf][lane] : R(0);
        br = lane < nw ? s_row[buf][lane] : -1;
        for (int o = 16; o; o >>= 1) {
            const R v2 = __shfl_xor_sync(0xffffffffu, best, o);
            const int r2 = __shfl_xor_sync(0xffffffffu, br, o);
            if (better(v2, r2, best, br)) { best = v2; br = r2; }
        }
        return br;
    };
    __syncthreads();
    int p;
    {
        R best = R(0);
        int br = -1;
#pragma unroll
        for (int k = 0; k < kGjRows; ++k) {
            const int r = tid + k * kGjThreads;
            if (r < m && !(um >> k & 1u)) {
                const R v = fabs(P[r * LD]);
                if (v > best) { best = v; br = r; }
            }
        }
        p = reduce(best, br, 0);
    }
    for (int c = 0; c < nb; ++c) {
        if (p < 0) {  // singular: the host reports it (pivrow stays in range)
            if (tid == 0) *bad = 1;
            return;
        }
        if (tid == 0) {
            s_p[c] = p;
            used[p] = 1;
            pivrow[c0 + c] = p;
        }
        if (p % kGjThreads == tid) um |= 1u << (p / kGjThreads);
        const R piv = P[p * LD + c];
        R best = R(0);
        int br = -1;
#pragma unroll
        for (int k = 0; k < kGjRows; ++k) {
            const int r = tid + k * kGjThreads;
            if (r >= m) continue;
            R f = R(0);
            if (r != p) {
                f = P[r * LD + c] / piv;
                if (f != R(0))
                    for (int cc = c + 1; cc < nb; ++cc) P[r * LD + cc] -= f * P[p * LD + cc];
            }
            F[(size_t)c * m + r] = f;
            if (c + 1 < nb && !(um >> k & 1u)) {
                const R v = fabs(P[r * LD + c + 1]);
                if (v > best) { best = v; br = r; }
            }
        }
        if (c + 1 < nb) p = reduce(best, br, (c + 1) & 1);
    }
    __syncthreads();  // the panel, F and s_p are complete
    for (int e = tid; e < m * nb; e += kGjThreads) {
        const int r = e / nb, c = e - r * nb;
        K[(size_t)r * m + c0 + c] = P[r * LD + c];
    }
    if (tid < nb) S[(size_t)s_p[tid] * m + c0 + tid] = R(1);
    if (tid < B * B) {  // zero beyond a short last panel
        const int c = tid / B, cp = tid - c * B;
        s_L[c][cp] = c < nb && cp < nb ? F[(size_t)cp * m + s_p[c]] : R(0);
    }
    __syncthreads();  // S's unit entries and L are in place
    const int c1 = c0 + nb;
    // L read from shared memory at each use (volatile): held in registers
    // across the columns, its 120 entries would spill
    const volatile R(*Lv)[B] = s_L;
    for (int d = tid; d < m; d += kGjThreads) {
        const R* V = d < c1 ? S : K;
        R w[B];
#pragma unroll
        for (int c = 0; c < B; ++c) {
            R v = c < nb ? V[(size_t)s_p[c] * m + d] : R(0);
#pragma unroll
            for (int cp = 0; cp < c; ++cp) v -= Lv[c][cp] * w[cp];
            w[c] = v;
        }
#pragma unroll
        for (int c = 0; c < B; ++c)
            if (c < nb) W[(size_t)c * m + d] = w[c];
    }
}

// V -= F W over 64 x 64 tiles (rows r, columns d; V = S below c1, K from c1
// on): 8 warps, warp y taking rows y + 8 i and lane x columns x + 32 j, so
// each access of a warp is 32 consecutive elements of one row
template <typename R>
__global__ void __launch_bounds__(256, 4) k_gjb_update(R* __restrict__ K, R* __restrict__ S, const R* __restrict__ F,
                                                    const R* __restrict__ W, int m, int c0, int nb) {
    constexpr int B = GjPanel<R>::B;
    __shared__ R sF[64][B + 1];
    __shared__ R sW[B][64];
    const int r0 = blockIdx.y * 64, d0 = blockIdx.x * 64;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    for (int e = threadIdx.x; e < 64 * B; e += 256) {
        const int c = e >> 6, rr = e & 63, r = r0 + rr;
        sF[rr][c] = r < m && c < nb ? F[(size_t)c * m + r] : R(0);
    }
    for (int e = threadIdx.x; e < B * 64; e += 256) {
        const int c = e >> 6, dd = e & 63, d = d0 + dd;
        sW[c][dd] = d < m && c < nb ? W[(size_t)c * m + d] : R(0);
    }
    __syncthreads();
    R acc[8][2];
#pragma unroll
    for (int i = 0; i < 8; ++i) acc[i][0] = acc[i][1] = R(0);
#pragma unroll
    for (int c = 0; c < B; ++c) {
        const R w0 = sW[c][tx], w1 = sW[c][tx + 32];
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const R a = sF[ty + 8 * i][c];
            acc[i][0] += a * w0;
            acc[i][1] += a * w1;
        }
    }
    const int c1 = c0 + nb;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const int r = r0 + ty + 8 * i;
        if (r >= m) continue;
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const int d = d0 + tx + 32 * j;
            if (d >= m) continue;
            R* v = (d < c1 ? S : K) + (size_t)r * m + d;
            *v -= acc[i][j];
        }
    }
}

}  // namespace ples
