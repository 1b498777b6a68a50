// batch.cu -- many grids solved together on one GPU: batched solves
// (ples_mg_batch_*) and the request server with continuous batching
// (ples_srv_*), both declared in include/ples_mg.h.
//
// Every member grid keeps its own handle: coefficient hierarchy, LU factors,
// dense coarse inverse and work buffers stay resident, and a member's last
// solution stays in its FP64 box as the warm start of its next solve.
//
// One outer iteration of the solve of every active member is a fixed list of
// steps: the FP64 wall fill passes, the FP64 residual with its norm, the
// per-member convergence decision, the inner V-cycles level by level, and the
// update.  Each step is ONE launch of a persistent kernel (about one CTA
// per SM slot) whose CTAs claim work items from that step's queue with an
// atomic counter until it is empty; an item is a (member, level, tile)
// triple -- a tile being one block of the kernel's own single-grid launch
// shape (Blk), so the item runs the same device body as a single-grid solve.
// Members of different sizes and depths share every launch; a member takes
// no part in the steps of levels it does not have, and members that are
// idle, converged or not yet admitted skip their items.  The step list,
// with the prologue (periodic ghosts of the initial guess, compatibility
// projection of the right-hand side and its norm) and the epilogue (zero
// mean) of the members whose phase asks for them, is captured once into a
// CUDA graph; one replay is one outer iteration for all members, and every
// phase change (admission, convergence, completion) is made on the device or
// between replays, so the same graph serves any mix of requests.
//
// Within a V-cycle the two field buffers of a level swap roles every sweep;
// the roles are fixed by the step list, which is generated by following the
// swaps once on the host (a member's sweep count per outer iteration is
// even, so each replay starts from the same roles).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "handle.h"
#include "mg_device.cuh"
#include "outer_device.cuh"

using namespace ples;

namespace {

enum Phase { PH_IDLE = 0, PH_PRO = 1, PH_ITER = 2, PH_EPI = 3, PH_DONE = 4 };
enum RedMode { RED_SHIFT = 0, RED_BNORM = 1, RED_DECIDE = 2, RED_MEAN = 3, RED_FINISH = 4 };

// per-member solve state, resident on the device and mirrored after each replay
struct InstState {
    int phase, it, status, vcycles;
    int max_cycles, inner, pad0, pad1;
    double rel_tol, abs_tol;
    double bn2, bnorm, shift, mean, rel, rmax, rel0;
};

// every task starts with the member, its first virtual block and its launch shape
struct TaskHead {
    int inst, blk0;
    int gx, gy, gz;
};
struct GhostTask { TaskHead h; Geom g; double* p; };
struct SumTask { TaskHead h; Geom g; const double* a; double* part; int squares; };
struct RedTask { TaskHead h; int mode; const double* pa; const double* pb; long long n; double ncell; int* sc; int oc; };
struct AddTask { TaskHead h; Geom g; double* a; int box; int use_mean; const uint8_t* solid; };
struct ZeroTask { TaskHead h; Geom g; double* a; const uint8_t* solid; };
struct WallCTask { TaskHead h; Geom g; Coef<double> c; const double* p; double* w; };
struct WallSTask { TaskHead h; Geom g; double* p; const double* w; };
struct RoutTask { TaskHead h; Geom g; Coef<float2> cs; const int* sc; const double* x; const double* b; float* rin; double* psq; double* pmax; const uint8_t* tipo; };
struct LineTask { TaskHead h; Geom g; Coef<float> c; const float* cp; const float* pin; const float* pk; float* pout; const float* rh; float omega; int kpar; int zk; int wide; };
struct RRTask { TaskHead h; Geom gf, gc; Coef<float> c; const float* p; const float* rh; float* rhc; int rx, ry, rz; };
struct DenseTask { TaskHead h; Geom g; const float* S; const float* rh; float* p; };
struct ProlTask { TaskHead h; Geom gf, gc; float* pf; const float* pc; int ry, rz; int b222; };
struct UpdTask { TaskHead h; Geom g; double* x; const float* e; };

// Claim virtual blocks of one step until its queue is empty.  The binary
// search finds the task (member, level) a block belongs to; blocks of members
// in another phase are skipped.
template <class Task, class F>
__device__ __forceinline__ void walk(const Task* __restrict__ tasks, int ntask, int total, int* ctr,
                                     const InstState* st, int phase, F&& f) {
    __shared__ int s_vb;
    const bool lead = threadIdx.x == 0 && threadIdx.y == 0;
    for (;;) {
        __syncthreads();  // the previous item is done with shared memory and s_vb
        if (lead) s_vb = atomicAdd(ctr, 1);
        __syncthreads();
        const int vb = s_vb;
        if (vb >= total) return;
        int lo = 0, hi = ntask - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (tasks[mid].h.blk0 <= vb) lo = mid;
            else hi = mid - 1;
        }
        const Task& t = tasks[lo];
        if (st[t.h.inst].phase != phase) continue;
        const int l = vb - t.h.blk0;
        Blk B;
        B.gx = t.h.gx;
        B.gy = t.h.gy;
        B.gz = t.h.gz;
        B.x = l % t.h.gx;
        B.y = (l / t.h.gx) % t.h.gy;
        B.z = l / (t.h.gx * t.h.gy);
        f(t, B);
    }
}

#define WALK_ARGS const T* t, int n, int total, int* ctr, InstState* st, int ph

template <class T>
__global__ void kb_ghost(WALK_ARGS) {
    walk(t, n, total, ctr, st, ph, [](const GhostTask& k, const Blk& B) { k_ghost_xz_blk<double>(k.g, k.p, B); });
}
template <class T>
__global__ void kb_sum(WALK_ARGS) {
    walk(t, n, total, ctr, st, ph,
         [](const SumTask& k, const Blk& B) { k_sum_interior_blk(k.g, k.a, k.squares, k.part, B); });
}
template <class T>
__global__ void kb_add(WALK_ARGS) {
    walk(t, n, total, ctr, st, ph, [st](const AddTask& k, const Blk& B) {
        const InstState& S = st[k.h.inst];
        const double v = -(k.use_mean ? S.mean : S.shift);
        if (k.box) k_add_box_blk(k.g, k.a, v, k.solid, B);
        else k_add_interior_blk(k.g, k.a, v, k.solid, B);
    });
}
// a field set to zero on the solid cells of a member's immersed-boundary mask
template <class T>
__global__ void kb_zero(WALK_ARGS) {
    walk(t, n, total, ctr, st, ph, [](const ZeroTask& k, const Blk& B) {
        for (long long q = (long long)B.x * blockDim.x + threadIdx.x; q < k.g.n; q += (long long)B.gx * blockDim.x)
            if (k.solid[q]) k.a[q] = 0.0;
    });
}
template <class T>
__global__ void kb_wallc(WALK_ARGS) {
    walk(t, n, total, ctr, st, ph, [](const WallCTask& k, const Blk& B) {
        k_wall_compute_blk(k.g, k.c, k.p, k.w, nullptr, nullptr, 0.0, B);
    });
}
template <class T>
__global__ void kb_walls(WALK_ARGS) {
    walk(t, n, total, ctr, st, ph, [](const WallSTask& k, const Blk& B) { k_wall_scatter_blk(k.g, k.p, k.w, B); });
}
// the outer residual of the (mixed) members in double-float, as the
// single-grid solve forms it
template <class T>
__global__ void __launch_bounds__(256, 4) kb_rout(WALK_ARGS) {
    walk(t, n, total, ctr, st, ph, [](const RoutTask& k, const Blk& B) {
        k_resid_outer2_df_blk<float, 8>(k.g, k.cs, k.x, k.b, k.rin, k.psq, k.pmax, B, k.tipo, k.sc);
    });
}
template <class T, bool ZIN>
__global__ void __launch_bounds__(256, 3) kb_line(WALK_ARGS) {
    walk(t, n, total, ctr, st, ph, [](const LineTask& k, const Blk& B) {
        k_line_relax_blk<float, true, ZIN>(k.g, k.c, k.cp, k.pin, k.pk, k.pout, k.rh, k.omega, k.kpar, k.zk, B);
    });
}
// a sweep step with 64-line tiles: 16 warps per CTA; the tasks of members
// whose level does not take them run the 32-line body with the same warps
template <class T, bool ZIN>
__global__ void __launch_bounds__(512, 2) kb_line_wide(WALK_ARGS) {
    walk(t, n, total, ctr, st, ph, [](const LineTask& k, const Blk& B) {
        if (k.wide)
            k_line_relax_x2_blk<ZIN>(k.g, k.c, k.cp, k.pin, k.pk, k.pout, k.rh, k.omega, k.kpar, k.zk, B);
        else
            k_line_relax_blk<float, true, ZIN>(k.g, k.c, k.cp, k.pin, k.pk, k.pout, k.rh, k.omega, k.kpar, k.zk, B);
    });
}
template <class T>
__global__ void kb_rr(WALK_ARGS) {
    walk(t, n, total, ctr, st, ph, [](const RRTask& k, const Blk& B) {
        k_resid_restrict_blk<float>(k.gf, k.gc, k.c, k.p, k.rh, k.rhc, k.rx, k.ry, k.rz, B);
    });
}
template <class T>
__global__ void kb_dense(WALK_ARGS) {
    walk(t, n, total, ctr, st, ph, [](const DenseTask& k, const Blk& B) { k_dense_solve_blk<float>(k.g, k.S, k.rh, k.p, B); });
}
template <class T>
__global__ void kb_prol(WALK_ARGS) {
    walk(t, n, total, ctr, st, ph, [](const ProlTask& k, const Blk& B) {
        if (k.b222)
            k_prolong_222_blk<float>(k.gf, k.gc, k.pf, k.pc, B);
        else
            k_prolong_x2_blk<float>(k.gf, k.gc, k.pf, k.pc, k.ry, k.rz, B);
    });
}
template <class T>
__global__ void kb_upd(WALK_ARGS) {
    walk(t, n, total, ctr, st, ph, [](const UpdTask& k, const Blk& B) { k_update_blk<float>(k.g, k.x, k.e, B); });
}

// Per-member reductions of block partials and the phase changes they drive
// (the host decisions of the single-grid solve, made on the device).
template <class T>
__global__ void kb_red(WALK_ARGS) {
    walk(t, n, total, ctr, st, ph, [st](const RedTask& k, const Blk&) {
        double s = 0.0, m = 0.0;
        for (long long q = threadIdx.x; q < k.n; q += blockDim.x) {
            s += k.pa[q];
            if (k.pb) m = fmax(m, k.pb[q]);
        }
        block_reduce_sum_max(s, m);
        if (threadIdx.x != 0) return;
        InstState& S = st[k.h.inst];
        switch (k.mode) {
            case RED_SHIFT: S.shift = s / k.ncell; break;
            case RED_BNORM:
                S.bn2 = s;
                S.bnorm = s > 0.0 ? sqrt(s) : 1.0;
                if (k.sc) {  // scale of the double-float residual: b's RMS into [1, 2)
                    const double rms = sqrt(s / k.ncell);
                    const int ob = rms > 0.0 && isfinite(rms) ? min(100, max(-100, -ilogb(rms))) : 0;
                    k.sc[0] = ob;
                    k.sc[1] = ob - k.oc;
                }
                S.it = 0;
                S.vcycles = 0;
                S.rel0 = -1.0;
                S.status = PLES_MG_NOT_CONVERGED;
                S.phase = PH_ITER;
                break;
            case RED_DECIDE: {
                const double rel = sqrt(s) / S.bnorm;
                S.rel = rel;
                S.rmax = m;
                if (!isfinite(rel)) {
                    S.status = PLES_MG_DIVERGED;
                    S.phase = PH_EPI;
                    break;
                }
                if (S.rel0 < 0.0) S.rel0 = rel;
                if ((S.rel_tol > 0.0 && rel <= S.rel_tol) || (S.abs_tol > 0.0 && m < S.abs_tol) || S.bn2 == 0.0) {
                    S.status = PLES_MG_OK;
                    S.phase = PH_EPI;
                } else if (rel > 1e6 * S.rel0 && rel > 1.0) {
                    S.status = PLES_MG_DIVERGED;
                    S.phase = PH_EPI;
                } else if (S.it >= S.max_cycles) {
                    S.status = PLES_MG_NOT_CONVERGED;
                    S.phase = PH_EPI;
                } else {
                    S.it += 1;
                    S.vcycles += S.inner;
                }
                break;
            }
            case RED_MEAN: S.mean = s / k.ncell; break;
            case RED_FINISH: S.phase = PH_DONE; break;
        }
    });
}
#undef WALK_ARGS

__global__ void k_to_box(Geom g, int ghost, const double* __restrict__ src, double* __restrict__ dst) {
    k_compact_to_box_blk(g, ghost, src, dst, hw_blk());
}
__global__ void k_from_box(Geom g, int ghost, const double* __restrict__ src, double* __restrict__ dst) {
    k_box_to_compact_blk(g, ghost, src, dst, hw_blk());
}
dim3 cgrid(const Geom& g, int ghost) {
    return ghost ? dim3((g.nx + 2 + 31) / 32, (g.ny + 2 + 3) / 4, g.nz + 2) : dim3((g.nx + 31) / 32, (g.ny + 3) / 4, g.nz);
}

enum Kind { K_GHOST, K_SUM, K_RED, K_ADD, K_WALLC, K_WALLS, K_ROUT, K_LINE0, K_LINE1, K_RR, K_DENSE, K_PROL, K_UPD,
            K_ZERO };

struct Step {
    int kind, phase;
    int ntask = 0, total = 0;
    size_t off = 0;    // byte offset of the task array in the table buffer
    int threads = 0;   // CTA width of a smoother step (the tuned width of its largest grid)
    bool wide = false; // a smoother step with 64-line tiles (kb_line_wide, 512 threads)
};

}  // namespace

// ---------------------------------------------------------------------------
// The engine: members, their step list, the task tables and the graph.
struct ples_mg_batch {
    std::vector<ples_mg_handle*> mem;
    // members the step list does not cover (x / z walls, FP64, another
    // smoother, semi-coarsening, no dense coarsest level): solved one after
    // another by the single-grid solver within the same call
    std::vector<char> solo;
    int dev = 0, nsm = 0;
    cudaStream_t st = nullptr;
    InstState* d_state = nullptr;
    InstState* h_state = nullptr;  // pinned mirror
    int* d_ctr = nullptr;
    unsigned char* d_tab = nullptr;
    std::vector<unsigned char> tab;
    std::vector<Step> steps;
    size_t smem_line = 0, smem_dense = 0, smem_wide = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::string err;
    long long replays = 0;
};

namespace {

int bfail(ples_mg_batch* b, int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (b) b->err = buf;
    return code;
}
#define BK(call)                                                                                          \
    do {                                                                                                  \
        cudaError_t e_ = (call);                                                                          \
        if (e_ != cudaSuccess)                                                                            \
            return bfail(b, e_ == cudaErrorMemoryAllocation ? PLES_MG_OOM : PLES_MG_CUDA_ERROR, "%s: %s", \
                         #call, cudaGetErrorString(e_));                                                  \
    } while (0)

// Step builder: tasks of one step are appended with their virtual-block prefix.
struct Builder {
    ples_mg_batch* b;
    Step cur{};
    template <class Task>
    void begin(int kind, int phase) {
        cur = Step{};
        cur.kind = kind;
        cur.phase = phase;
        size_t o = (b->tab.size() + 255) & ~size_t(255);
        b->tab.resize(o);
        cur.off = o;
    }
    template <class Task>
    void add(Task t, dim3 grid) {
        if (b->solo[t.h.inst]) return;  // solved outside the step list
        t.h.blk0 = cur.total;
        t.h.gx = (int)grid.x;
        t.h.gy = (int)grid.y;
        t.h.gz = (int)grid.z;
        const size_t o = b->tab.size();
        b->tab.resize(o + sizeof(Task));
        std::memcpy(b->tab.data() + o, &t, sizeof(Task));
        cur.ntask += 1;
        cur.total += (int)(grid.x * grid.y * grid.z);
    }
    void end() {
        if (cur.ntask > 0) b->steps.push_back(cur);
    }
};

dim3 line_grid(const Geom& g) { return dim3((g.nx + 31) / 32, (g.nz + 1) / 2, 1); }
dim3 rr_grid(const Geom& gc) { return dim3((gc.nx + 31) / 32, (gc.ny + 3) / 4, gc.nz); }
dim3 prol_grid(const Geom& gf, const Geom& gc) { return dim3((gc.nx + 1 + 31) / 32, (gf.ny + 2 + 3) / 4, gf.nz + 2); }
dim3 box_grid2(const Geom& g) { return dim3((g.nx + 2 + 31) / 32, (g.ny + 2 + 3) / 4, g.nz + 2); }
dim3 red_grid2(const Geom& g) { return dim3((g.nx + 31) / 32, (g.ny + kRedThreads / 32 - 1) / (kRedThreads / 32), g.nz); }
dim3 rout_grid(const Geom& g) { return dim3((g.nx + 31) / 32, (g.ny + 7) / 8, (g.nz + 7) / 8); }

int build_steps(ples_mg_batch* b) {
    const int nm = (int)b->mem.size();
    Builder B{b};
    // kb_line_wide runs the 64-line form or the 32-line form with 16 warps:
    // its shared memory is the larger of the two over all members' levels
    for (int i = 0; i < nm; ++i)
        for (int n = 0; n < b->mem[i]->nlev && !b->solo[i]; ++n) {
            const size_t ny2 = (size_t)b->mem[i]->L[n].g.ny + 2;
            b->smem_wide = std::max(b->smem_wide, std::max(3 * ny2 * 64 + 4 * 16 * 32, (3 * ny2 + 4 * 16) * 32) *
                                                      sizeof(float));
        }
    const bool allow_wide = b->smem_wide <= 227 * 1024;
    // buffer roles per member and level: 0 -> (p, p2), 1 -> (p2, p)
    std::vector<std::vector<int>> cur(nm);
    int lmax = 0, numax = 0, nupmax = 0, inmax = 0, wmax = 0;
    for (int i = 0; i < nm; ++i) {
        ples_mg_handle* h = b->mem[i];
        cur[i].assign(h->nlev, 0);
        if (b->solo[i]) continue;
        lmax = std::max(lmax, h->nlev);
        numax = std::max(numax, h->nu_pre);
        nupmax = std::max(nupmax, h->nu_post);
        inmax = std::max(inmax, h->inner_cycles);
        wmax = std::max(wmax, h->wall_passes);
    }
    auto P = [&](int i, int n, int which) -> float* {
        const LevelData& L = b->mem[i]->L[n];
        return (float*)((cur[i][n] ^ which) ? L.p2 : L.p);
    };
    auto sum_step = [&](int phase, bool on_x, int squares) {
        B.begin<SumTask>(K_SUM, phase);
        for (int i = 0; i < nm; ++i) {
            ples_mg_handle* h = b->mem[i];
            SumTask t{};
            t.h.inst = i;
            t.g = h->L[0].g;
            t.a = on_x ? h->x : h->b;
            t.part = h->part_a;
            t.squares = squares;
            B.add(t, red_grid2(t.g));
        }
        B.end();
    };
    auto red_step = [&](int phase, int mode, int src) {  // src 0: sum partials, 1: residual partials, 2: none
        B.begin<RedTask>(K_RED, phase);
        for (int i = 0; i < nm; ++i) {
            ples_mg_handle* h = b->mem[i];
            const Geom& g = h->L[0].g;
            RedTask t{};
            t.h.inst = i;
            t.mode = mode;
            if (mode == RED_BNORM && h->L[0].has_cs) {
                t.sc = h->dscale;
                t.oc = h->oc;
            }
            t.ncell = h->masked ? (double)h->nfluid : (double)g.nx * g.ny * g.nz;
            if (src == 0) {
                const dim3 r = red_grid2(g);
                t.pa = h->part_a;
                t.n = (long long)r.x * r.y * r.z;
            } else if (src == 1) {
                const dim3 r = rout_grid(g);
                t.pa = h->part_a;
                t.pb = h->part_b;
                t.n = (long long)r.x * r.y * r.z;
            }
            B.add(t, dim3(1, 1, 1));
        }
        B.end();
    };
    auto add_step = [&](int phase, bool on_x) {
        B.begin<AddTask>(K_ADD, phase);
        for (int i = 0; i < nm; ++i) {
            ples_mg_handle* h = b->mem[i];
            AddTask t{};
            t.h.inst = i;
            t.g = h->L[0].g;
            t.a = on_x ? h->x : h->b;
            t.box = on_x;
            t.use_mean = on_x;
            t.solid = h->masked ? h->mask[0] : nullptr;
            B.add(t, on_x ? box_grid2(t.g) : dim3((t.g.nx + 31) / 32, (t.g.ny + 3) / 4, t.g.nz));
        }
        B.end();
    };
    auto zero_step = [&](int phase, bool on_x) {  // masked members: the field vanishes on solid cells
        B.begin<ZeroTask>(K_ZERO, phase);
        for (int i = 0; i < nm; ++i) {
            ples_mg_handle* h = b->mem[i];
            if (!h->masked) continue;
            ZeroTask t{};
            t.h.inst = i;
            t.g = h->L[0].g;
            t.a = on_x ? h->x : h->b;
            t.solid = h->mask[0];
            B.add(t, dim3((unsigned)std::min<long long>((t.g.n + 255) / 256, 4096), 1, 1));
        }
        B.end();
    };
    // one sweep of level n for the members in it (s: the sweep's index among
    // the pre-smoothing sweeps, or the post-smoothing ones when post)
    auto line_steps = [&](int c, int n, int s, bool zin, bool post) {
        for (int par = 0; par < 2; ++par) {
            B.begin<LineTask>(zin ? K_LINE1 : K_LINE0, PH_ITER);
            long long big = -1;
            for (int i = 0; i < nm; ++i) {
                ples_mg_handle* h = b->mem[i];
                if (c >= h->inner_cycles || n > h->nlev - 2 || s >= (post ? h->nu_post : h->nu_pre)) continue;
                const LevelData& L = h->L[n];
                LineTask t{};
                t.h.inst = i;
                t.g = L.g;
                t.c = L.cf;
                t.cp = (const float*)L.cp;
                t.pin = P(i, n, 0);
                t.pout = P(i, n, 1);
                t.pk = par == 0 ? t.pin : t.pout;
                t.rh = (const float*)L.rh;
                t.omega = (float)h->omega;
                t.kpar = par;
                t.zk = (zin && par == 0) ? 1 : 0;
                // 64-line tiles where they apply and fill at least one tile
                t.wide = allow_wide && L.x2_ok && L.g.nx >= 64 ? 1 : 0;
                B.add(t, t.wide ? dim3((L.g.nx + 63) / 64, (L.g.nz + 1) / 2, 1) : line_grid(L.g));
                if (t.wide) B.cur.wide = true;
                const long long cells = (long long)L.g.nx * L.g.ny * L.g.nz;
                if (cells > big) {
                    big = cells;
                    B.cur.threads = std::min(L.line_threads, 256);  // kb_line is built for 256
                }
            }
            B.end();
        }
        for (int i = 0; i < nm; ++i) {
            ples_mg_handle* h = b->mem[i];
            if (c >= h->inner_cycles || n > h->nlev - 2 || s >= (post ? h->nu_post : h->nu_pre)) continue;
            cur[i][n] ^= 1;
        }
    };

    // ---- prologue: solid cells of masked members zeroed, periodic ghosts of
    // fi, compatibility projection, |b|
    zero_step(PH_PRO, true);
    zero_step(PH_PRO, false);
    B.begin<GhostTask>(K_GHOST, PH_PRO);
    for (int i = 0; i < nm; ++i) {
        ples_mg_handle* h = b->mem[i];
        GhostTask t{};
        t.h.inst = i;
        t.g = h->L[0].g;
        t.p = h->x;
        const long long tot = 2LL * (t.g.nx + 2) * (t.g.ny + 2) + 2LL * (t.g.ny + 2) * t.g.nz;
        B.add(t, dim3((unsigned)std::min<long long>((tot + 255) / 256, 4096), 1, 1));
    }
    B.end();
    sum_step(PH_PRO, false, 0);
    red_step(PH_PRO, RED_SHIFT, 0);
    add_step(PH_PRO, false);
    sum_step(PH_PRO, false, 1);
    red_step(PH_PRO, RED_BNORM, 0);

    // ---- one outer iteration
    for (int pass = 0; pass < wmax; ++pass) {
        B.begin<WallCTask>(K_WALLC, PH_ITER);
        for (int i = 0; i < nm; ++i) {
            ples_mg_handle* h = b->mem[i];
            if (pass >= h->wall_passes) continue;
            WallCTask t{};
            t.h.inst = i;
            t.g = h->L[0].g;
            t.c = h->L[0].cd;
            t.p = h->x;
            t.w = h->wbuf;
            B.add(t, dim3((t.g.nx + 31) / 32, (t.g.nz + 3) / 4, 2));
        }
        B.end();
        B.begin<WallSTask>(K_WALLS, PH_ITER);
        for (int i = 0; i < nm; ++i) {
            ples_mg_handle* h = b->mem[i];
            if (pass >= h->wall_passes) continue;
            WallSTask t{};
            t.h.inst = i;
            t.g = h->L[0].g;
            t.p = h->x;
            t.w = h->wbuf;
            B.add(t, dim3((t.g.nx + 2 + 31) / 32, (t.g.nz + 2 + 3) / 4, 2));
        }
        B.end();
    }
    B.begin<RoutTask>(K_ROUT, PH_ITER);
    for (int i = 0; i < nm; ++i) {
        ples_mg_handle* h = b->mem[i];
        RoutTask t{};
        t.h.inst = i;
        t.g = h->L[0].g;
        t.cs = h->L[0].cs;
        t.sc = h->dscale;
        t.x = h->x;
        t.b = h->b;
        t.rin = (float*)h->L[0].rh;
        t.psq = h->part_a;
        t.pmax = h->part_b;
        t.tipo = h->tipo;
        B.add(t, rout_grid(t.g));
    }
    B.end();
    red_step(PH_ITER, RED_DECIDE, 1);
    for (int c = 0; c < inmax; ++c) {
        for (int n = 0; n + 1 < lmax; ++n) {
            for (int s = 0; s < numax; ++s) line_steps(c, n, s, s == 0 && (n > 0 || c == 0), false);
            B.begin<RRTask>(K_RR, PH_ITER);
            for (int i = 0; i < nm; ++i) {
                ples_mg_handle* h = b->mem[i];
                if (c >= h->inner_cycles || n > h->nlev - 2) continue;
                const LevelData& F = h->L[n];
                const LevelData& C = h->L[n + 1];
                RRTask t{};
                t.h.inst = i;
                t.gf = F.g;
                t.gc = C.g;
                t.c = F.cf;
                t.p = P(i, n, 0);
                t.rh = (const float*)F.rh;
                t.rhc = (float*)C.rh;
                t.rx = C.rx;
                t.ry = C.ry;
                t.rz = C.rz;
                B.add(t, rr_grid(C.g));
            }
            B.end();
        }
        B.begin<DenseTask>(K_DENSE, PH_ITER);
        for (int i = 0; i < nm; ++i) {
            ples_mg_handle* h = b->mem[i];
            if (c >= h->inner_cycles) continue;
            const int nc = h->nlev - 1;
            const LevelData& C = h->L[nc];
            DenseTask t{};
            t.h.inst = i;
            t.g = C.g;
            t.S = (const float*)h->coarse_S;
            t.rh = (const float*)C.rh;
            t.p = P(i, nc, 0);
            B.add(t, dim3((h->coarse_n + 7) / 8, 1, 1));
        }
        B.end();
        for (int n = lmax - 2; n >= 0; --n) {
            B.begin<ProlTask>(K_PROL, PH_ITER);
            for (int i = 0; i < nm; ++i) {
                ples_mg_handle* h = b->mem[i];
                if (c >= h->inner_cycles || n > h->nlev - 2) continue;
                const LevelData& F = h->L[n];
                const LevelData& C = h->L[n + 1];
                ProlTask t{};
                t.h.inst = i;
                t.gf = F.g;
                t.gc = C.g;
                t.pf = P(i, n, 0);
                t.pc = P(i, n + 1, 0);
                t.ry = C.ry;
                t.rz = C.rz;
                // eight fine cells per thread under full coarsening of even sizes
                t.b222 = C.ry == 2 && C.rz == 2 && F.g.nx % 2 == 0 && F.g.ny % 2 == 0 && F.g.nz % 2 == 0;
                B.add(t, t.b222 ? dim3((C.g.nx + 1 + 31) / 32, (F.g.ny + 10) / 8, (F.g.nz + 3) / 2)
                                : prol_grid(F.g, C.g));
            }
            B.end();
            for (int s = 0; s < nupmax; ++s) line_steps(c, n, s, false, true);
        }
    }
    B.begin<UpdTask>(K_UPD, PH_ITER);
    for (int i = 0; i < nm; ++i) {
        ples_mg_handle* h = b->mem[i];
        UpdTask t{};
        t.h.inst = i;
        t.g = h->L[0].g;
        t.x = h->x;
        t.e = P(i, 0, 0);
        B.add(t, box_grid2(t.g));
    }
    B.end();

    // ---- epilogue: solid cells reset (the prolongation may have touched
    // them), zero mean over the fluid cells, then done
    zero_step(PH_EPI, true);
    sum_step(PH_EPI, true, 0);
    red_step(PH_EPI, RED_MEAN, 0);
    add_step(PH_EPI, true);
    red_step(PH_EPI, RED_FINISH, 2);

    for (int i = 0; i < nm; ++i)
        for (int n = 0; n < (int)cur[i].size() && !b->solo[i]; ++n)
            if (cur[i][n] != 0)
                return bfail(b, PLES_MG_BAD_ARG, "member %d: odd sweep count per outer iteration on level %d", i,
                             n + 1);
    for (int i = 0; i < nm; ++i) {
        ples_mg_handle* h = b->mem[i];
        if (b->solo[i]) continue;
        for (int n = 0; n < h->nlev; ++n)
            b->smem_line = std::max(b->smem_line, (3 * (size_t)(h->L[n].g.ny + 2) + 4 * 8) * 32 * sizeof(float));
        b->smem_dense = std::max(b->smem_dense, (size_t)h->coarse_n * sizeof(float));
    }
    return PLES_MG_OK;
}

template <class K>
int occupancy_grid(ples_mg_batch* b, K kernel, int threads, size_t smem, int total, int* grid) {
    int per = 0;
    BK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, threads, smem));
    if (per < 1) return bfail(b, PLES_MG_BAD_ARG, "a batched kernel does not fit on an SM");
    *grid = std::max(1, std::min(total, per * b->nsm));
    return PLES_MG_OK;
}

template <class Task, class K>
int launch_step(ples_mg_batch* b, const Step& s, int idx, K kernel, dim3 block, size_t smem) {
    int grid = 0;
    int rc = occupancy_grid(b, kernel, (int)(block.x * block.y * block.z), smem, s.total, &grid);
    if (rc) return rc;
    kernel<<<grid, block, smem, b->st>>>((const Task*)(b->d_tab + s.off), s.ntask, s.total, b->d_ctr + idx,
                                         b->d_state, s.phase);
    BK(cudaGetLastError());
    return PLES_MG_OK;
}

int record_steps(ples_mg_batch* b) {
    BK(cudaMemsetAsync(b->d_ctr, 0, sizeof(int) * b->steps.size(), b->st));
    const dim3 b1(256), b2(32, 4);
    for (size_t q = 0; q < b->steps.size(); ++q) {
        const Step& s = b->steps[q];
        const int i = (int)q;
        int rc = 0;
        switch (s.kind) {
            case K_GHOST: rc = launch_step<GhostTask>(b, s, i, kb_ghost<GhostTask>, b1, 0); break;
            case K_SUM: rc = launch_step<SumTask>(b, s, i, kb_sum<SumTask>, dim3(kRedThreads), 0); break;
            case K_RED: rc = launch_step<RedTask>(b, s, i, kb_red<RedTask>, b1, 0); break;
            case K_ADD: rc = launch_step<AddTask>(b, s, i, kb_add<AddTask>, b2, 0); break;
            case K_WALLC: rc = launch_step<WallCTask>(b, s, i, kb_wallc<WallCTask>, b2, 0); break;
            case K_WALLS: rc = launch_step<WallSTask>(b, s, i, kb_walls<WallSTask>, b2, 0); break;
            case K_ROUT: rc = launch_step<RoutTask>(b, s, i, kb_rout<RoutTask>, b1, 0); break;
            case K_LINE0:
                rc = s.wide ? launch_step<LineTask>(b, s, i, kb_line_wide<LineTask, false>, dim3(512), b->smem_wide)
                            : launch_step<LineTask>(b, s, i, kb_line<LineTask, false>, dim3(s.threads), b->smem_line);
                break;
            case K_LINE1:
                rc = s.wide ? launch_step<LineTask>(b, s, i, kb_line_wide<LineTask, true>, dim3(512), b->smem_wide)
                            : launch_step<LineTask>(b, s, i, kb_line<LineTask, true>, dim3(s.threads), b->smem_line);
                break;
            case K_RR: rc = launch_step<RRTask>(b, s, i, kb_rr<RRTask>, b2, 0); break;
            case K_DENSE: rc = launch_step<DenseTask>(b, s, i, kb_dense<DenseTask>, b1, b->smem_dense); break;
            case K_PROL: rc = launch_step<ProlTask>(b, s, i, kb_prol<ProlTask>, b2, 0); break;
            case K_UPD: rc = launch_step<UpdTask>(b, s, i, kb_upd<UpdTask>, b2, 0); break;
            case K_ZERO: rc = launch_step<ZeroTask>(b, s, i, kb_zero<ZeroTask>, b1, 0); break;
        }
        if (rc) return rc;
    }
    BK(cudaMemcpyAsync(b->h_state, b->d_state, sizeof(InstState) * b->mem.size(), cudaMemcpyDeviceToHost, b->st));
    return PLES_MG_OK;
}

int batch_create(ples_mg_handle* const* members, int n, ples_mg_batch* b) {
    if (!members || n < 1) return bfail(b, PLES_MG_BAD_ARG, "no members");
    for (int i = 0; i < n; ++i) {
        ples_mg_handle* h = members[i];
        if (!h) return bfail(b, PLES_MG_BAD_ARG, "member %d is null", i);
        if (h->dev != members[0]->dev) return bfail(b, PLES_MG_BAD_ARG, "members live on different devices");
        // the step list covers mixed precision, the zebra smoother, full
        // coarsening in x, periodic x and z and a dense coarsest level
        bool solo = h->d.precision != PLES_MG_PREC_MIXED || h->smoother != 0 || h->d.coarsening != 0 ||
                    !h->coarse_S || h->walls_xz;
        for (int l = 1; l < h->nlev; ++l) solo = solo || h->L[l].rx != 2;
        b->mem.push_back(h);
        b->solo.push_back(solo ? 1 : 0);
    }
    b->dev = members[0]->dev;
    BK(cudaSetDevice(b->dev));
    BK(cudaDeviceGetAttribute(&b->nsm, cudaDevAttrMultiProcessorCount, b->dev));
    BK(cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking));
    int rc = build_steps(b);
    if (rc) return rc;
    BK(cudaMalloc((void**)&b->d_state, sizeof(InstState) * n));
    BK(cudaMallocHost((void**)&b->h_state, sizeof(InstState) * n));
    std::memset(b->h_state, 0, sizeof(InstState) * n);
    BK(cudaMemcpyAsync(b->d_state, b->h_state, sizeof(InstState) * n, cudaMemcpyHostToDevice, b->st));
    BK(cudaMalloc((void**)&b->d_ctr, sizeof(int) * std::max<size_t>(1, b->steps.size())));
    BK(cudaMalloc((void**)&b->d_tab, std::max<size_t>(256, b->tab.size())));
    BK(cudaMemcpyAsync(b->d_tab, b->tab.data(), b->tab.size(), cudaMemcpyHostToDevice, b->st));
    if (b->smem_line > 227 * 1024 || b->smem_dense > 227 * 1024)
        return bfail(b, PLES_MG_BAD_ARG, "a member's lines are too long for shared memory");
    for (auto& s : b->steps)  // (no step is wide when smem_wide does not fit)
        if (s.wide) {
            BK(cudaFuncSetAttribute(kb_line_wide<LineTask, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)b->smem_wide));
            BK(cudaFuncSetAttribute(kb_line_wide<LineTask, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)b->smem_wide));
            break;
        }
    BK(cudaFuncSetAttribute(kb_line<LineTask, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b->smem_line));
    BK(cudaFuncSetAttribute(kb_line<LineTask, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b->smem_line));
    BK(cudaFuncSetAttribute(kb_dense<DenseTask>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                            (int)std::max<size_t>(b->smem_dense, 1)));
    BK(cudaStreamSynchronize(b->st));
    BK(cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal));
    rc = record_steps(b);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(b->st, &g);
    if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess) return bfail(b, PLES_MG_CUDA_ERROR, "graph capture: %s", cudaGetErrorString(e));
    b->graph = g;
    BK(cudaGraphInstantiate(&b->exec, b->graph, 0));
    return PLES_MG_OK;
}

void batch_free(ples_mg_batch* b) {
    if (!b) return;
    cudaSetDevice(b->dev);
    if (b->st) cudaStreamSynchronize(b->st);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    if (b->d_state) cudaFree(b->d_state);
    if (b->h_state) cudaFreeHost(b->h_state);
    if (b->d_ctr) cudaFree(b->d_ctr);
    if (b->d_tab) cudaFree(b->d_tab);
    if (b->st) cudaStreamDestroy(b->st);
    delete b;
}

// upload the state mirror after host-side phase changes
int push_state(ples_mg_batch* b) {
    BK(cudaMemcpyAsync(b->d_state, b->h_state, sizeof(InstState) * b->mem.size(), cudaMemcpyHostToDevice, b->st));
    return PLES_MG_OK;
}

// one outer iteration of every active member; the mirror is current afterwards
int replay(ples_mg_batch* b) {
    BK(cudaGraphLaunch(b->exec, b->st));
    BK(cudaStreamSynchronize(b->st));
    ++b->replays;
    return PLES_MG_OK;
}

// member i: host fi (may be null: keep the resident solution) and rhs into its boxes
int stage_in(ples_mg_batch* b, int i, const double* fi, const double* rhs, bool device_ptrs) {
    ples_mg_handle* h = b->mem[i];
    const Geom& g = h->L[0].g;
    const size_t nfi = (size_t)(g.nx + 2) * (g.ny + 2) * (g.nz + 2), nrh = (size_t)g.nx * g.ny * g.nz;
    const cudaMemcpyKind kind = device_ptrs ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    if (fi) {
        BK(cudaMemcpyAsync(h->fi_c, fi, 8 * nfi, kind, b->st));
        k_to_box<<<cgrid(g, 1), dim3(32, 4), 0, b->st>>>(g, 1, h->fi_c, h->x);
    }
    BK(cudaMemcpyAsync(h->rhs_c, rhs, 8 * nrh, kind, b->st));
    k_to_box<<<cgrid(g, 0), dim3(32, 4), 0, b->st>>>(g, 0, h->rhs_c, h->b);
    BK(cudaGetLastError());
    return PLES_MG_OK;
}

// member i's solution box into fi (host or device), with its ghost layer
int stage_out(ples_mg_batch* b, int i, double* fi, bool device_ptrs) {
    ples_mg_handle* h = b->mem[i];
    const Geom& g = h->L[0].g;
    const size_t nfi = (size_t)(g.nx + 2) * (g.ny + 2) * (g.nz + 2);
    k_from_box<<<cgrid(g, 1), dim3(32, 4), 0, b->st>>>(g, 1, h->x, h->fi_c);
    BK(cudaGetLastError());
    BK(cudaMemcpyAsync(fi, h->fi_c, 8 * nfi, device_ptrs ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, b->st));
    return PLES_MG_OK;
}

void admit(ples_mg_batch* b, int i, double rel_tol, double abs_tol, int max_cycles) {
    InstState& S = b->h_state[i];
    std::memset(&S, 0, sizeof S);
    S.phase = PH_PRO;
    S.rel_tol = rel_tol;
    S.abs_tol = abs_tol;
    S.max_cycles = max_cycles;
    S.inner = b->mem[i]->inner_cycles;
    S.status = PLES_MG_NOT_CONVERGED;
}

void to_stats(const InstState& S, ples_mg_stats* o) {
    std::memset(o, 0, sizeof *o);
    o->outer_iterations = S.it;
    o->vcycles = S.vcycles;
    o->rel_residual = S.rel;
    o->max_residual = S.rmax;
    o->rhs_norm = std::sqrt(S.bn2);
    o->rhs_mean_removed = S.shift;
    o->status = S.status;
}

int batch_solve(ples_mg_batch* b, double* const* fi, const double* const* rhs, double rel_tol, double abs_tol,
                int max_cycles, ples_mg_stats* stats, bool device_ptrs) {
    nvtxRangePushA("ples_mg batch solve");
    struct Pop {
        ~Pop() { nvtxRangePop(); }
    } pop;
    const int nm = (int)b->mem.size();
    auto t0 = std::chrono::steady_clock::now();
    BK(cudaSetDevice(b->dev));
    for (int i = 0; i < nm; ++i) {
        if (!rhs[i]) return bfail(b, PLES_MG_BAD_ARG, "rhs of member %d is null", i);
        if (b->solo[i]) continue;
        int rc = stage_in(b, i, fi ? fi[i] : nullptr, rhs[i], device_ptrs);
        if (rc) return rc;
        admit(b, i, rel_tol, abs_tol, max_cycles);
    }
    int rc = push_state(b);
    if (rc) return rc;
    bool any = false;
    for (int i = 0; i < nm; ++i) any = any || !b->solo[i];
    for (long long r = 0; any && r < (long long)max_cycles + 3; ++r) {
        if ((rc = replay(b))) return rc;
        bool all = true;
        for (int i = 0; i < nm; ++i) all = all && (b->solo[i] || b->h_state[i].phase == PH_DONE);
        if (all) break;
    }
    int worst = PLES_MG_OK;
    auto fold = [&](int s) {
        if (s == PLES_MG_DIVERGED) worst = s;
        else if (s == PLES_MG_NOT_CONVERGED && worst == PLES_MG_OK) worst = s;
    };
    // the members outside the step list, one after another
    for (int i = 0; i < nm; ++i) {
        if (!b->solo[i]) continue;
        ples_mg_handle* h = b->mem[i];
        if ((rc = stage_in(b, i, fi ? fi[i] : nullptr, rhs[i], device_ptrs))) return rc;
        BK(cudaStreamSynchronize(b->st));
        ples_mg_stats st{};
        const int s = solve_resident(h, rel_tol, abs_tol, max_cycles, &st);
        if (s != PLES_MG_OK && s != PLES_MG_NOT_CONVERGED && s != PLES_MG_DIVERGED)
            return bfail(b, s, "member %d: %s", i, h->err.c_str());
        BK(cudaStreamSynchronize(h->st));
        if (fi && fi[i] && (rc = stage_out(b, i, fi[i], device_ptrs))) return rc;
        if (stats) stats[i] = st;
        fold(s);
    }
    for (int i = 0; i < nm; ++i) {
        if (b->solo[i]) continue;
        if (b->h_state[i].phase != PH_DONE)
            return bfail(b, PLES_MG_CUDA_ERROR, "member %d did not finish (phase %d)", i, b->h_state[i].phase);
        if (fi && fi[i] && (rc = stage_out(b, i, fi[i], device_ptrs))) return rc;
        if (stats) to_stats(b->h_state[i], &stats[i]);
        fold(b->h_state[i].status);
        b->h_state[i].phase = PH_IDLE;
    }
    if ((rc = push_state(b))) return rc;
    BK(cudaStreamSynchronize(b->st));
    const double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (stats)
        for (int i = 0; i < nm; ++i) stats[i].seconds = sec;
    return worst;
}

}  // namespace

// ---------------------------------------------------------------------------
// The request server: a worker thread owns the engine.  Requests wait in a
// FIFO; a request is admitted when its member has no request in flight (a
// member's buffers are its slot): its right-hand side goes through the
// member's pinned staging buffer to the device and the member enters the
// prologue at the next replay, while the other members keep iterating.
// After a replay the members that finished start their copy-out (device box
// -> pinned buffer); the next replay is launched at once and the host
// completes those requests (pinned buffer -> caller's array) while it runs.
struct ples_srv {
    ples_mg_batch* eng = nullptr;
    std::thread worker;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    bool stop = false;
    struct Req {
        long long ticket;
        int member;
        std::vector<double> rhs;
        double* fi_out;
        double rel_tol;
        int max_cycles;
        std::chrono::steady_clock::time_point t_sub;
        ples_mg_stats st{};
        int rc = 0;
        bool done = false;
    };
    std::deque<std::shared_ptr<Req>> pending;
    std::vector<std::shared_ptr<Req>> inflight;  // per member: admitted, solving
    std::vector<std::shared_ptr<Req>> prepared;  // per member: next request, its rhs in pin_rhs
    std::vector<std::shared_ptr<Req>> handing;   // per member: finished, solution being copied out
    std::vector<std::shared_ptr<Req>> finished;  // not yet collected by wait
    std::vector<double*> pin_rhs, pin_fi;        // per-member pinned staging
    cudaEvent_t ev_out = nullptr;
    long long next_ticket = 1;
    std::vector<double> lat_ms;
    long long completed = 0;
    double bytes = 0.0;
    int fatal = 0;
    std::string err;
    std::chrono::steady_clock::time_point t_first{};
    bool started = false;
};

namespace {

size_t box_count(const Geom& g) { return (size_t)(g.nx + 2) * (g.ny + 2) * (g.nz + 2); }
size_t rhs_count(const Geom& g) { return (size_t)g.nx * g.ny * g.nz; }

void srv_fail_all(ples_srv* s, int rc) {  // under s->mu
    s->fatal = rc;
    s->err = s->eng->err;
    for (auto* v : {&s->inflight, &s->prepared, &s->handing})
        for (auto& r : *v)
            if (r) {
                r->rc = rc;
                r->done = true;
                s->finished.push_back(r);
                r.reset();
            }
    for (auto& r : s->pending) {
        r->rc = rc;
        r->done = true;
        s->finished.push_back(r);
    }
    s->pending.clear();
    s->stop = true;
    s->cv_done.notify_all();
}

// The worker.  Per member: inflight (admitted, solving), prepared (its
// right-hand side already in the member's pinned buffer, admitted as soon as
// the member finishes) and handing (finished, its solution being copied
// out).  One pass: admit requests of idle members, replay once, and while
// the replay runs hand out the solutions copied before it and copy the next
// requests' right-hand sides into pinned memory; after it, a finished
// member's solution is queued for copy-out and its prepared request admitted
// at once, so it joins the next replay (warm-started from the solution just
// copied out: the copy is queued first on the same stream).
void srv_loop(ples_srv* s) {
    ples_mg_batch* b = s->eng;
    const int nm = (int)b->mem.size();
    cudaSetDevice(b->dev);
    std::vector<int> out_pending;  // copy-out enqueued before the current replay
    std::vector<ples_mg_stats> snap(nm);
    // a stage-in from pin_rhs[i] is queued and may not have run yet (cleared
    // by the stream synchronisation after each replay)
    std::vector<char> rhs_busy(nm, 0);
    bool dirty = false;            // host-side phase changes not yet on the device
    auto finish = [&](const std::shared_ptr<ples_srv::Req>& r, const ples_mg_stats& st, int rc,
                      std::chrono::steady_clock::time_point now) {  // under s->mu
        r->st = st;
        r->st.seconds = std::chrono::duration<double>(now - r->t_sub).count();
        r->rc = rc;
        r->done = true;
        s->lat_ms.push_back(r->st.seconds * 1e3);
        ++s->completed;
        s->finished.push_back(r);
    };
    for (;;) {
        std::vector<std::shared_ptr<ples_srv::Req>> admit_now;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            auto busy = [&] {
                for (int i = 0; i < nm; ++i)
                    if (s->inflight[i] || s->handing[i] || s->prepared[i]) return true;
                return false;
            };
            s->cv_work.wait(lk, [&] { return s->stop || !s->pending.empty() || busy(); });
            if (s->stop && !busy()) return;
            for (auto it = s->pending.begin(); it != s->pending.end();) {
                if (!s->inflight[(*it)->member]) {
                    s->inflight[(*it)->member] = *it;
                    admit_now.push_back(*it);
                    it = s->pending.erase(it);
                } else {
                    ++it;
                }
            }
        }
        int rc = 0;
        for (auto& r : admit_now) {
            const int i = r->member;
            std::memcpy(s->pin_rhs[i], r->rhs.data(), sizeof(double) * r->rhs.size());
            if ((rc = stage_in(b, i, nullptr, s->pin_rhs[i], false))) break;
            rhs_busy[i] = 1;
            if (b->solo[i]) {  // outside the step list: solved now, warm-started from its last solution
                ples_mg_handle* h = b->mem[i];
                if (cudaStreamSynchronize(b->st) != cudaSuccess) { rc = PLES_MG_CUDA_ERROR; break; }
                ples_mg_stats st{};
                const int sr = solve_resident(h, r->rel_tol, 0.0, r->max_cycles, &st);
                if (sr != PLES_MG_OK && sr != PLES_MG_NOT_CONVERGED && sr != PLES_MG_DIVERGED) { rc = sr; break; }
                if (cudaStreamSynchronize(h->st) != cudaSuccess || (rc = stage_out(b, i, s->pin_fi[i], false)) ||
                    cudaStreamSynchronize(b->st) != cudaSuccess) {
                    rc = rc ? rc : PLES_MG_CUDA_ERROR;
                    break;
                }
                const auto now = std::chrono::steady_clock::now();
                std::lock_guard<std::mutex> lk(s->mu);
                if (r->fi_out) std::memcpy(r->fi_out, s->pin_fi[i], sizeof(double) * box_count(h->L[0].g));
                finish(r, st, sr, now);
                s->inflight[i].reset();
                s->cv_done.notify_all();
                continue;
            }
            admit(b, i, r->rel_tol, 0.0, r->max_cycles);
            dirty = true;
        }
        if (!rc && dirty) {
            rc = push_state(b);
            dirty = false;
        }
        bool active = false;
        for (int i = 0; i < nm; ++i) {
            const int ph = b->h_state[i].phase;
            active = active || ph == PH_PRO || ph == PH_ITER || ph == PH_EPI;
        }
        if (!rc && active && cudaGraphLaunch(b->exec, b->st) != cudaSuccess) rc = PLES_MG_CUDA_ERROR;
        // while the replay runs: hand out the results copied before it ...
        if (!rc && !out_pending.empty()) {
            if (cudaEventSynchronize(s->ev_out) != cudaSuccess) rc = PLES_MG_CUDA_ERROR;
            const auto now = std::chrono::steady_clock::now();
            std::lock_guard<std::mutex> lk(s->mu);
            for (int i : out_pending) {
                auto r = s->handing[i];
                if (!rc && r->fi_out) std::memcpy(r->fi_out, s->pin_fi[i], sizeof(double) * box_count(b->mem[i]->L[0].g));
                finish(r, snap[i], rc ? rc : snap[i].status, now);
                s->handing[i].reset();
            }
            s->cv_done.notify_all();
            out_pending.clear();
        }
        // ... and stage the next request of each busy member in pinned memory
        if (!rc) {
            std::vector<std::shared_ptr<ples_srv::Req>> prep;
            {
                std::lock_guard<std::mutex> lk(s->mu);
                for (auto it = s->pending.begin(); it != s->pending.end();) {
                    const int i = (*it)->member;
                    if (!b->solo[i] && s->inflight[i] && !s->prepared[i] && !rhs_busy[i]) {
                        s->prepared[i] = *it;
                        prep.push_back(*it);
                        it = s->pending.erase(it);
                    } else {
                        ++it;
                    }
                }
            }
            for (auto& r : prep) std::memcpy(s->pin_rhs[r->member], r->rhs.data(), sizeof(double) * r->rhs.size());
        }
        if (!rc && cudaStreamSynchronize(b->st) != cudaSuccess) rc = PLES_MG_CUDA_ERROR;
        if (!rc && active) ++b->replays;
        if (!rc) {
            std::fill(rhs_busy.begin(), rhs_busy.end(), 0);
            std::lock_guard<std::mutex> lk(s->mu);
            for (int i = 0; i < nm && !rc; ++i)
                if (b->h_state[i].phase == PH_DONE) {
                    to_stats(b->h_state[i], &snap[i]);
                    const Geom& g = b->mem[i]->L[0].g;
                    k_from_box<<<cgrid(g, 1), dim3(32, 4), 0, b->st>>>(g, 1, b->mem[i]->x, b->mem[i]->fi_c);
                    if (cudaMemcpyAsync(s->pin_fi[i], b->mem[i]->fi_c, sizeof(double) * box_count(g),
                                        cudaMemcpyDeviceToHost, b->st) != cudaSuccess)
                        rc = PLES_MG_CUDA_ERROR;
                    s->handing[i] = s->inflight[i];
                    s->inflight[i].reset();
                    b->h_state[i].phase = PH_IDLE;
                    dirty = true;
                    out_pending.push_back(i);
                    if (!rc && s->prepared[i]) {  // the member's next request joins the next replay
                        auto r = s->prepared[i];
                        s->prepared[i].reset();
                        s->inflight[i] = r;
                        if ((rc = stage_in(b, i, nullptr, s->pin_rhs[i], false))) break;
                        rhs_busy[i] = 1;
                        admit(b, i, r->rel_tol, 0.0, r->max_cycles);
                    }
                }
            if (!rc && !out_pending.empty() && cudaEventRecord(s->ev_out, b->st) != cudaSuccess) rc = PLES_MG_CUDA_ERROR;
        }
        if (rc) {  // a device error ends the server: fail everything in flight
            std::lock_guard<std::mutex> lk(s->mu);
            srv_fail_all(s, rc);
            return;
        }
    }
}

double pct(std::vector<double> v, double p) {
    if (v.empty()) return 0.0;
    std::sort(v.begin(), v.end());
    const double pos = p / 100.0 * (double)(v.size() - 1);
    const size_t lo = (size_t)std::floor(pos), hi = std::min(v.size() - 1, lo + 1);
    return v[lo] + (pos - (double)lo) * (v[hi] - v[lo]);
}

}  // namespace

extern "C" {

int ples_mg_batch_create(ples_mg_handle* const* members, int n, ples_mg_batch** out) {
    if (!out) return PLES_MG_BAD_ARG;
    *out = nullptr;
    ples_mg_batch* b = new ples_mg_batch();
    int rc = batch_create(members, n, b);
    if (rc) {
        std::fprintf(stderr, "ples_mg_batch_create: %s\n", b->err.c_str());
        batch_free(b);
        return rc;
    }
    *out = b;
    return PLES_MG_OK;
}

int ples_mg_batch_solve(ples_mg_batch* b, double* const* fi, const double* const* rhs, double rel_tol,
                        int max_cycles, ples_mg_stats* stats) {
    if (!b || !rhs || max_cycles < 0) return b ? bfail(b, PLES_MG_BAD_ARG, "bad argument") : PLES_MG_BAD_ARG;
    return batch_solve(b, fi, rhs, rel_tol, 0.0, max_cycles, stats, false);
}

int ples_mg_batch_solve_device(ples_mg_batch* b, double* const* d_fi, const double* const* d_rhs, double rel_tol,
                               int max_cycles, ples_mg_stats* stats) {
    if (!b || !d_rhs || max_cycles < 0) return b ? bfail(b, PLES_MG_BAD_ARG, "bad argument") : PLES_MG_BAD_ARG;
    return batch_solve(b, d_fi, d_rhs, rel_tol, 0.0, max_cycles, stats, true);
}

int ples_mg_batch_info(const ples_mg_batch* b, int* steps, long long* replays) {
    if (!b) return PLES_MG_BAD_ARG;
    if (steps) *steps = (int)b->steps.size();
    if (replays) *replays = b->replays;
    return PLES_MG_OK;
}

const char* ples_mg_batch_last_error(const ples_mg_batch* b) { return b ? b->err.c_str() : "null batch"; }

void ples_mg_batch_destroy(ples_mg_batch* b) { batch_free(b); }

int ples_srv_create(ples_mg_handle* const* members, int n, double hbm_budget_bytes, ples_srv** out) {
    if (!out || !members || n < 1) return PLES_MG_BAD_ARG;
    *out = nullptr;
    double bytes = 0.0;
    for (int i = 0; i < n; ++i) {
        if (!members[i]) return PLES_MG_BAD_ARG;
        bytes += (double)members[i]->bytes;
    }
    if (hbm_budget_bytes > 0.0 && bytes > hbm_budget_bytes) {
        std::fprintf(stderr, "ples_srv_create: members hold %.3g bytes, over the budget of %.3g\n", bytes,
                     hbm_budget_bytes);
        return PLES_MG_OOM;
    }
    ples_mg_batch* b = new ples_mg_batch();
    int rc = batch_create(members, n, b);
    if (rc) {
        std::fprintf(stderr, "ples_srv_create: %s\n", b->err.c_str());
        batch_free(b);
        return rc;
    }
    ples_srv* s = new ples_srv();
    s->eng = b;
    s->inflight.resize(n);
    s->prepared.resize(n);
    s->handing.resize(n);
    s->bytes = bytes;
    bool ok = cudaEventCreateWithFlags(&s->ev_out, cudaEventDisableTiming) == cudaSuccess;
    for (int i = 0; i < n && ok; ++i) {
        const Geom& g = members[i]->L[0].g;
        double *pr = nullptr, *pf = nullptr;
        ok = cudaMallocHost((void**)&pr, sizeof(double) * rhs_count(g)) == cudaSuccess;
        if (ok) ok = cudaMallocHost((void**)&pf, sizeof(double) * box_count(g)) == cudaSuccess;
        s->pin_rhs.push_back(pr);
        s->pin_fi.push_back(pf);
    }
    if (!ok) {
        ples_srv_destroy(s);
        return PLES_MG_OOM;
    }
    s->worker = std::thread(srv_loop, s);
    *out = s;
    return PLES_MG_OK;
}

int ples_srv_submit(ples_srv* s, int member, const double* rhs, double* fi_out, double rel_tol, int max_cycles,
                    long long* ticket) {
    if (!s || !rhs || member < 0 || member >= (int)s->inflight.size() || max_cycles < 0) return PLES_MG_BAD_ARG;
    auto r = std::make_shared<ples_srv::Req>();
    const Geom& g = s->eng->mem[member]->L[0].g;
    r->rhs.assign(rhs, rhs + rhs_count(g));
    r->member = member;
    r->fi_out = fi_out;
    r->rel_tol = rel_tol;
    r->max_cycles = max_cycles;
    r->t_sub = std::chrono::steady_clock::now();
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->fatal) return s->fatal;
    r->ticket = s->next_ticket++;
    if (ticket) *ticket = r->ticket;
    if (!s->started) {
        s->started = true;
        s->t_first = r->t_sub;
    }
    s->pending.push_back(r);
    s->cv_work.notify_one();
    return PLES_MG_OK;
}

int ples_srv_wait(ples_srv* s, long long ticket, ples_mg_stats* stats) {
    if (!s) return PLES_MG_BAD_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    for (;;) {
        for (auto it = s->finished.begin(); it != s->finished.end(); ++it)
            if ((*it)->ticket == ticket) {
                auto r = *it;
                s->finished.erase(it);
                if (stats) *stats = r->st;
                return r->rc;
            }
        bool known = false;
        for (auto& r : s->pending) known = known || r->ticket == ticket;
        for (auto* v : {&s->inflight, &s->prepared, &s->handing})
            for (auto& r : *v) known = known || (r && r->ticket == ticket);
        if (!known) return PLES_MG_BAD_ARG;
        s->cv_done.wait(lk);
    }
}

int ples_srv_report(ples_srv* s, double* p50_ms, double* p99_ms, double* p999_ms, long long* completed,
                    double* solves_per_s) {
    if (!s) return PLES_MG_BAD_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    if (p50_ms) *p50_ms = pct(s->lat_ms, 50.0);
    if (p99_ms) *p99_ms = pct(s->lat_ms, 99.0);
    if (p999_ms) *p999_ms = pct(s->lat_ms, 99.9);
    if (completed) *completed = s->completed;
    if (solves_per_s) {
        const double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - s->t_first).count();
        *solves_per_s = s->started && sec > 0.0 ? (double)s->completed / sec : 0.0;
    }
    return PLES_MG_OK;
}

void ples_srv_destroy(ples_srv* s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        s->cv_work.notify_all();
    }
    if (s->worker.joinable()) s->worker.join();
    batch_free(s->eng);
    for (double* p : s->pin_rhs)
        if (p) cudaFreeHost(p);
    for (double* p : s->pin_fi)
        if (p) cudaFreeHost(p);
    if (s->ev_out) cudaEventDestroy(s->ev_out);
    delete s;
}

}  // extern "C"
