// handle.h -- the state behind a ples_mg_handle (one grid's coefficient
// hierarchy and work buffers on one device), shared by the single-grid
// solver (ples_mg.cu) and the batched engine (batch.cu).  Internal: not part
// of the C ABI.
#pragma once
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <string>
#include <vector>

#include "line_pair.cuh"
#include "line_tma.cuh"
#include "mg_device.cuh"
#include "ples_mg.h"

constexpr int kMaxLev = 12;

struct LevelData {
    ples::Geom g;
    int rx = 1, ry = 1, rz = 1;  // coarsening ratio from the finer level
    int sx = 1, sy = 1, sz = 1;  // cumulative node strides relative to level 1
    double inv_div = 1.0;        // raw metric = t * inv_div
    double post = 1.0;           // stored coefficient = raw * post (x 1/4 on cross terms)
    void* p = nullptr;           // inner-precision fields (T boxes)
    void* p2 = nullptr;
    void* rh = nullptr;
    void* cp = nullptr;          // LU factor c' of the eta-line operator (T box)
    void* im = nullptr;          // pivot reciprocals 1/m of that operator (FP32 box, 64-line-tile levels)
    ples::Coef<float> cf{};             // FP32 scaled coefficients (mixed)
    ples::Coef<double> cd{};            // FP64 scaled coefficients (level 1 always; all levels in FP64 mode)
    ples::Coef<float2> cs{};            // the FP64 ones split into double-floats x 2^oc (level 1, mixed)
    bool has_cf = false, has_cd = false, has_cs = false;
    // TMA-staged zebra smoother (FP32): tensor maps of this level's fields;
    // pA/pB are the buffers behind maps.pA/pB (p and p2 swap every sweep)
    // form of the eta-line smoother: 128, 256 or 512 threads on 32-line
    // tiles, 1024 for the 64-line-tile form (512 threads, k_line_relax_x2),
    // 2048 for the 64-line tiles with the pair build (256 threads,
    // k_line_relax_p2), 4096 for the 64-line tiles with both k parities in
    // one launch (512 threads, k_line_relax_x2m); autotuned
    int line_threads = 256;
    bool x2_ok = false;  // the 64-line-tile form applies (FP32, x and z periodic, nx even, nz >= 2)
    bool tma = false;
    void *pA = nullptr, *pB = nullptr;
    ples::LineMaps maps{};
};

struct ples_mg_handle {
    ples_mg_desc d{};
    int dev = 0;
    cudaStream_t st = nullptr;
    int nlev = 0;
    LevelData L[kMaxLev];
    double *xn = nullptr, *yn = nullptr, *zn = nullptr;  // fine nodes (0:jx,0:jy,0:jz)
    double *x = nullptr, *b = nullptr;                   // FP64 solution / rhs boxes (level 1)
    double* wbuf = nullptr;                              // 2*nx*nz wall rows
    void* sbuf = nullptr;                                // ghosts of walled x/z directions (side_cells, 8 B each)
    bool walls_xz = false;                               // ip = 1 or kp = 1
    bool fs = false;                                     // free surface at the top wall (desc.freesurface)
    double* prs = nullptr;                               // its surface pressure PrS0 (1:jx,1:jz), device
    double *part_a = nullptr, *part_b = nullptr;         // block partials
    long long npart = 0;
    double* red = nullptr;                               // 2 doubles on the device (+ dflag)
    int* dflag = nullptr;                                // bounded-wait error flag, inside red
    int* dscale = nullptr;                               // ob, ox of the double-float residual (inside red)
    int oc = 0;                                          // power-of-two scale of the split coefficients
    bool probe_fallback = false;                         // the default settings diverged on this grid (earlier defaults taken)
    int* x2sync = nullptr;                               // tickets and plane counters of k_line_relax_x2m (nz + 3)
    unsigned wait_polls = ples::kSpinLimit;              // polls of a bounded device wait before it gives up
    double* h_red = nullptr;                             // pinned host copy
    double* norm_scratch = nullptr;  // device address of the library's fixed residual scratch (this device)
    double *fi_c = nullptr, *rhs_c = nullptr;            // compact staging
    uint8_t* tipo = nullptr;  // level-1 cell types (0 solid, 1 IB, 2 fluid, 3 other), or null
    double* cs_c[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};   // this call's wall fluxes
    double* cs_buf[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr}; // their device buffers
    // projection step (diver / gradie / vel_up), allocated on first use:
    // contravariant face velocities, Cartesian cell velocities, face normals
    // csx..ztz and the cell Jacobian
    double *d_uc = nullptr, *d_vc = nullptr, *d_wc = nullptr;
    double *d_u = nullptr, *d_v = nullptr, *d_w = nullptr;
    double* nrm[9] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    double* giac = nullptr;
    void* coarse_S = nullptr;                            // dense inverse of the coarsest system (T)
    int coarse_n = 0;
    // immersed-boundary mask: byte box per level (1 = solid), fluid cells of level 1
    bool masked = false;
    uint8_t* mask[kMaxLev] = {};
    long long nfluid = 0;
    int wall_passes = 3;
    double wall_q = 0.0;
    int nu_pre = 2, nu_post = 2, nu_coarse = 40, inner_cycles = 3, smoother = 0;
    double omega = 0.8;
    std::vector<void*> allocs;
    std::string err;
    long long bytes = 0;
    // instrumentation: kernels launched, and optional CUDA-event timing of
    // one kernel kind at one level (pairs are read back after each solve)
    long long launches = 0;
    int timed_kind = -1, timed_level = 0;
    std::vector<cudaEvent_t> ev_pool;
    size_t ev_used = 0;
    double timed_ms = 0.0;
    long long timed_launches = 0;
    // CUDA graph of one outer iteration (V-cycles, update, wall fill, FP64
    // residual, reduction and its copy to the host), replayed while the
    // settings it was captured with hold
    cudaGraphExec_t iter_exec = nullptr;
    std::vector<long long> iter_key;
    long long iter_launches = 0;
    bool use_graphs = true;
    bool capturing = false;            // timing events go into the graph
    std::vector<cudaEvent_t> ev_graph; // the graph's timing event pairs
    size_t g_used = 0;
    bool graph_pending = false;        // a replay ran since the last collect
};

inline int fail(ples_mg_handle* h, int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (h) h->err = buf;
    return code;
}

#define CK(call)                                                                               \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess)                                                                 \
            return fail(h, e_ == cudaErrorMemoryAllocation ? PLES_MG_OOM : PLES_MG_CUDA_ERROR, \
                        "%s failed: %s", #call, cudaGetErrorString(e_));                       \
    } while (0)

namespace ples {
// single-grid solve from the resident boxes, no wall fluxes (ples_mg.cu)
int solve_resident(ples_mg_handle* h, double rel_tol, double abs_tol, int max_cycles, ples_mg_stats* st);
}  // namespace ples
