#!/usr/bin/env python
"""Benchmark: pressure-Poisson solves per second to ||r||/||b|| <= 1e-10.

Workload: the wavy-wall channel at 256x128x256 (8.4M cells, wall amplitude
0.1, y-stretch 2.5, RHS seed 1), seeded synthetic inputs.  One step is one
complete solve from a zero initial guess on the GPU-resident grid through
the C ABI (ples_mg_solve_device): mixed precision, FP32 V-cycles inside the
FP64 defect-correction loop.  `value` is whole-job solves/s (K steps x N
replicas / max over ranks of the CUDA-event time on the solve stream).
Inputs stay larger than L2 (the FP64 fields and coefficients are ~1.9 GB),
so no L2 flush is needed between steps.

Extra fields: the plain-FP64 solve rate on the same grid and the mixed/FP64
ratio; `e2e` times the host-buffer entry point ples_mg_solve (pinned host
fi/rhs, H2D and D2H inside the timed region); `roofline` measures the
dominant kernel (the level-1 FP32 eta-line smoother) with CUDA events
around each of its launches inside the timed region; `cpu_baseline` times
the CPU oracle (the restated reference algorithm, line SOR, emulated MPI
ranks as threads) on a bounded sample.

`--impl reference` times the reference's algorithm on the host cores (the
CPU oracle: the Fortran reference cannot be built here) and prints the same
line with "impl": "reference".
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Poisson solves/s to rel-resid 1e-10"
UNIT = "solves/s"
# algorithmic bytes per cell of one FP32 eta-line sweep (both k-parity
# launches of the zebra smoother together): read p, rhs and the nine face
# coefficients, write p (12 x 4 B)
LINE_BYTES_PER_CELL = 48
# DRAM bytes (read + written) of one level-1 sweep of the smoother, from one
# ncu capture (`ncu --set full --clock-control none -k regex:k_line_relax_x2f
# -s 12 -c 2` of `python bench.py --steps 1 --warmup 3 --fp64-steps 0
# --e2e-steps 0 --no-cpu-baseline --batch-steps 0 --serve-requests 0
# --ib-steps 0`): dram__bytes_read.sum + dram__bytes_write.sum over the two
# launches of one sweep; keyed by workload and the kernel that capture timed,
# and reported only when the bench times that same kernel
LINE_TRAFFIC = {
    ("channel_256x128x256", "k_line_relax_x2f"): 335541504 + 335393792,
}
# the level-1 smoother form (threads per CTA as ples_mg_set_line_threads
# takes them) -> the kernel it launches
LINE_KERNELS = {2048: "k_line_relax_p2", 1024: "k_line_relax_x2f", 512: "k_line_relax_w", 256: "k_line_relax",
                128: "k_line_relax"}


def _workload_config(w):
    """The keys that define a workload, shared by both arms' `config`."""
    return {"workload": w.name, "grid": f"{w.jx}x{w.jy}x{w.jz}", "cells": w.cells,
            "wall_amplitude": w.amp, "y_stretch": w.beta, "rhs_seed": w.seed,
            "tolerance": "||r||2/||b||2 <= 1e-10", "data": "seeded synthetic grid and RHS",
            "l2": "inputs larger than L2 (no flush)"}


def _ranks_for(w, cores):
    """Emulated MPI ranks of the reference solver: the most threads up to
    `cores` that divide jz at every one of its 4 levels (jz / 8)."""
    for p in range(cores, 0, -1):
        if (w.jz // 8) % p == 0:
            return p
    return 1


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [v.strip() for v in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def replica_throughput(t_local, steps, world_size, dist=None, device="cpu"):
    """Whole-job throughput of independent replicas: every rank timed its own
    `steps` solves in t_local seconds; the job's time is the slowest rank's
    (max over ranks) and the job solved steps x world_size grids.  Returns
    (t_max, solves per second)."""
    t = t_local
    if dist is not None and world_size > 1:
        import torch
        tt = torch.tensor([t_local], dtype=torch.float64, device=device)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t = float(tt.item())
    return t, steps * world_size / t


def cpu_baseline(workload, threads_cap=None):
    """Reference algorithm on the host: the CPU oracle (line SOR as in the
    reference's islor=1 option, 4 levels, kss 5/10, omega 1.6) with nproc
    emulated MPI ranks as threads, one complete solve from zero to
    ||r||/||b|| <= 1e-10 on the full grid, timed whole (no extrapolation)."""
    from oracle.oracle import Oracle
    from ples_gb300 import synthetic as S
    w = S.WORKLOADS[workload]
    x, y, z = w.grid()
    rhs = w.rhs()
    cores = os.cpu_count() or 1
    if threads_cap:
        cores = min(cores, threads_cap)
    nproc = _ranks_for(w, cores)
    o = Oracle(x, y, z, islor=1, nproc=nproc)
    t0 = time.perf_counter()
    _, cyc, _, rr = o.multi(rhs, eps=1e-10, ficycle=400)
    dt = time.perf_counter() - t0
    return {"value": 1.0 / dt, "unit": UNIT, "cores": nproc, "kind": "port",
            "sample": (f"one complete solve of the restated reference solver (line SOR, {nproc} emulated "
                       f"MPI ranks as threads) on the full {workload} grid from zero to "
                       f"||r||/||b|| = {rr:.2e}: {cyc} V-cycles in {dt:.1f} s"),
            "vcycles": cyc, "seconds_per_solve": dt}


def run_reference(args):
    """The reference arm: the restated reference solver on the host cores
    (the Fortran+MPI reference cannot be built on either machine).  One
    complete solve from zero counts the V-cycles it needs to reach
    ||r||/||b|| <= 1e-10 with this run's rank count; then each of the
    warm-up and timed steps is one V-cycle of the same solve, and
    value = 1 / (mean timed V-cycle x that count).  ms_per_step is the timed
    step (one V-cycle)."""
    ws, rank, local = _dist()
    if rank != 0:
        return
    steps, warm = args.steps, args.warmup
    from oracle.oracle import Oracle
    from ples_gb300 import synthetic as S
    w = S.WORKLOADS[args.workload]
    x, y, z = w.grid()
    rhs = w.rhs()
    nproc = _ranks_for(w, os.cpu_count() or 1)
    o = Oracle(x, y, z, islor=1, nproc=nproc)
    t0 = time.perf_counter()
    _, ncyc, _, rr = o.multi(rhs, eps=1e-10, ficycle=400)
    t_solve = time.perf_counter() - t0
    times = []
    for s in range(warm + steps):
        t0 = time.perf_counter()
        o.multi(rhs, eps=1e-30, ficycle=1)
        if s >= warm:
            times.append(time.perf_counter() - t0)
    t_cycle = sum(times) / len(times)
    value = 1.0 / (t_cycle * ncyc)
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": steps,
        "warmup": warm, "ms_per_step": t_cycle * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "impl": "reference",
        "config": _workload_config(w),
        "solver": {"kind": "restated reference multi: line SOR (islor=1), omega 1.6, kss 5/10, 4 levels, "
                           f"{nproc} emulated MPI ranks as threads",
                   "step": "one V-cycle; value = 1 / (ms_per_step x vcycles_to_tolerance)",
                   "vcycles_to_tolerance": ncyc, "rel_residual_reached": rr,
                   "full_solve_seconds": t_solve},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nproc, "kind": "port",
                         "sample": (f"{steps} timed V-cycles ({t_cycle:.2f} s each) x {ncyc} V-cycles to 1e-10 "
                                    f"counted in this run by one complete solve ({t_solve:.1f} s)")},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="channel_256x128x256")
    ap.add_argument("--fp64-steps", type=int, default=3)
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--smoother", type=int, default=0)
    ap.add_argument("--nu", type=int, default=0)
    ap.add_argument("--inner", type=int, default=0)
    ap.add_argument("--omega", type=float, default=0.0)
    ap.add_argument("--batch-steps", type=int, default=3,
                    help="timed repetitions of the 64-grid batched solve (0: skip that leg)")
    ap.add_argument("--serve-requests", type=int, default=400,
                    help="requests of the served-ensemble leg (0: skip that leg)")
    ap.add_argument("--serve-rate", type=float, default=2000.0)
    ap.add_argument("--ib-steps", type=int, default=2,
                    help="timed solves of the 512x256x512 immersed-boundary case (0: skip that leg)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
        return

    import numpy as np
    import torch
    from ples_gb300 import mg
    from ples_gb300 import synthetic as S

    ws, rank, local = _dist()
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    w = S.WORKLOADS[args.workload]
    x, y, z = w.grid()
    rhs = w.rhs()
    kw = dict(device=local, smoother=args.smoother, nu_pre=args.nu, nu_post=args.nu,
              inner_cycles=args.inner, omega=args.omega)
    m = mg.Multigrid(x, y, z, precision="mixed", **kw)
    nfi = (w.jx + 2) * (w.jy + 2) * (w.jz + 2)
    d_fi = torch.zeros(nfi, dtype=torch.float64, device="cuda")
    d_rhs = torch.from_numpy(np.ascontiguousarray(rhs.ravel(order="F"))).cuda()
    stream = torch.cuda.current_stream()
    sh = stream.cuda_stream

    def step():
        d_fi.zero_()
        return m.solve_device(d_fi.data_ptr(), d_rhs.data_ptr(), rel_tol=1e-10, max_cycles=200, stream=sh)

    for _ in range(args.warmup):
        st = step()
    torch.cuda.synchronize()
    if st["status"] != mg.OK:
        raise RuntimeError(f"warm-up solve did not converge: {st}")
    m.time_kernel("line", 1)
    n0 = m.counters()["launches"]
    clocks = ClockSampler(local)
    clocks.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    stats = []
    for _ in range(args.steps):
        stats.append(step())
    e1.record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clk = clocks.stop()
    t = e0.elapsed_time(e1) / 1e3
    launches = m.counters()["launches"] - n0
    kms, kn = m.kernel_time()
    m.time_kernel(None)
    t, value = replica_throughput(t, args.steps, ws, dist, device="cuda")
    ms_per_step = t / args.steps * 1e3
    outer = statistics.mean(s["outer_iterations"] for s in stats)
    relres = max(s["rel_residual"] for s in stats)

    # plain FP64 on the same grid
    t64, st64, err_vs_fp64 = None, {"outer_iterations": None}, None
    if args.fp64_steps > 0:
        t64, st64, err_vs_fp64 = fp64_leg(args, x, y, z, w, nfi, d_fi, d_rhs, local, sh)

    # end to end through the host-buffer entry point with pinned buffers
    e2e_value = None
    if args.e2e_steps > 0:
        e2e_value = e2e_leg(args, m, rhs, w, nfi) * ws
    extra = {}
    if args.batch_steps > 0:
        extra["batch"] = batch_leg(args, local)
    if args.serve_requests > 0:
        extra["serve"] = serve_leg(args, local)
    if args.ib_steps > 0:
        extra["ib"] = ib_leg(args, local)
    _report(args, m, w, ws, rank, dist, value, ms_per_step, outer, relres, t64, st64, err_vs_fp64,
            e2e_value, nfi, launches, kms, kn, clk, extra)


def fp64_leg(args, x, y, z, w, nfi, d_fi, d_rhs, local, sh):
    import numpy as np
    import torch
    from ples_gb300 import mg
    m64 = mg.Multigrid(x, y, z, precision="fp64", device=local, smoother=args.smoother,
                       nu_pre=args.nu, nu_post=args.nu, inner_cycles=args.inner, omega=args.omega)
    d_fi64 = torch.zeros(nfi, dtype=torch.float64, device="cuda")

    def step64():
        d_fi64.zero_()
        return m64.solve_device(d_fi64.data_ptr(), d_rhs.data_ptr(), rel_tol=1e-10, max_cycles=400,
                                stream=sh)

    st64 = step64()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    for _ in range(args.fp64_steps):
        st64 = step64()
    f1.record(stream)
    torch.cuda.synchronize()
    t64 = f0.elapsed_time(f1) / 1e3 / args.fp64_steps
    # mixed vs FP64 solution agreement (zero-mean fields)
    a = d_fi.cpu().numpy().reshape((w.jx + 2, w.jy + 2, w.jz + 2), order="F")[1:-1, 1:-1, 1:-1]
    b = d_fi64.cpu().numpy().reshape((w.jx + 2, w.jy + 2, w.jz + 2), order="F")[1:-1, 1:-1, 1:-1]
    err_vs_fp64 = float(np.linalg.norm(a - b) / np.linalg.norm(b))
    m64.close()
    return t64, st64, err_vs_fp64


def e2e_leg(args, m, rhs, w, nfi):
    import ctypes as C
    import numpy as np
    import torch
    from ples_gb300 import mg
    # one zeroed pinned initial guess per step, prepared before the timed
    # region (each solve overwrites its fi with the solution)
    h_fis = [torch.zeros(nfi, dtype=torch.float64).pin_memory() for _ in range(args.e2e_steps + 1)]
    h_rhs = torch.from_numpy(np.ascontiguousarray(rhs.ravel(order="F"))).pin_memory()
    fi_nps = [h.numpy().reshape((w.jx + 2, w.jy + 2, w.jz + 2), order="F") for h in h_fis]
    rhs_np = h_rhs.numpy().reshape((w.jx, w.jy, w.jz), order="F")
    lib = mg.load()
    stx = mg.Stats()

    def step_e2e(fi_np):
        rc = lib.ples_mg_solve(m._h, fi_np, rhs_np, None, 1e-10, 0.0, 200, C.byref(stx))
        if rc != mg.OK:
            raise RuntimeError(f"e2e solve failed: {rc}")

    step_e2e(fi_nps[-1])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for s in range(args.e2e_steps):
        step_e2e(fi_nps[s])
    torch.cuda.synchronize()
    te = (time.perf_counter() - t0) / args.e2e_steps
    return 1.0 / te  # per replica


def batch_leg(args, local):
    """64 independent grids of uneven size (seeds 2..65) solved together by
    one batch (a captured graph of persistent step kernels per outer
    iteration), against the same 64 grids solved one after another by the
    plain FP64 solver and by the single-grid mixed solver.  Device-resident
    inputs; wall-clock time of whole calls (each returns after its solves)."""
    import numpy as np
    import torch
    from ples_gb300 import mg
    from ples_gb300 import synthetic as S
    insts = S.batch_instances()
    grids = [w.grid() for w in insts]
    rhs = [w.rhs() for w in insts]
    nfis = [(w.jx + 2) * (w.jy + 2) * (w.jz + 2) for w in insts]
    d_rhs = [torch.from_numpy(np.ascontiguousarray(r.ravel(order="F"))).cuda() for r in rhs]
    d_fi = [torch.zeros(n, dtype=torch.float64, device="cuda") for n in nfis]
    members = [mg.Multigrid(*g, device=local) for g in grids]
    b = mg.Batch(members)

    def run():
        for f in d_fi:
            f.zero_()
        torch.cuda.synchronize()
        return b.solve_device([f.data_ptr() for f in d_fi], [r.data_ptr() for r in d_rhs], rel_tol=1e-10)

    run()
    t0 = time.perf_counter()
    for _ in range(args.batch_steps):
        sts = run()
    tb = (time.perf_counter() - t0) / args.batch_steps
    info = b.info()
    ok = all(s["status"] == mg.OK for s in sts)
    relmax = max(s["rel_residual"] for s in sts)
    # end to end through ples_mg_batch_solve: pinned host arrays in and out,
    # each step from its own zeroed initial guesses (prepared before the
    # timed region; a solve overwrites them with its solutions)
    import ctypes as C
    ne = max(1, min(args.batch_steps, 3))
    h_rhs = [torch.from_numpy(np.ascontiguousarray(r.ravel(order="F"))).pin_memory() for r in rhs]
    h_fis = [[torch.zeros(n, dtype=torch.float64).pin_memory() for n in nfis] for _ in range(ne + 1)]
    lib = mg.load()
    stx = (mg.Stats * len(insts))()
    rhs_ptrs = mg._ptr_array([r.data_ptr() for r in h_rhs])

    def step_e2e(fs):
        fi_ptrs = mg._ptr_array([f.data_ptr() for f in fs])
        rc = lib.ples_mg_batch_solve(b._b, C.cast(fi_ptrs, C.c_void_p), C.cast(rhs_ptrs, C.c_void_p), 1e-10, 200,
                                     C.cast(stx, C.c_void_p))
        if rc != mg.OK:
            raise RuntimeError(f"batch e2e solve failed: {rc}")

    step_e2e(h_fis[-1])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for s in range(ne):
        step_e2e(h_fis[s])
    torch.cuda.synchronize()
    te = (time.perf_counter() - t0) / ne
    e2e_ok = all(s.status == mg.OK for s in stx)
    h2d = 8 * (sum(nfis) + sum(w.cells for w in insts))
    d2h = 8 * sum(nfis)
    del h_fis, h_rhs
    b.close()
    sh = torch.cuda.current_stream().cuda_stream

    def sequential(ms, fs, rs):
        tot = 0.0
        for mm, f, r in zip(ms, fs, rs, strict=True):
            f.zero_()
            mm.solve_device(f.data_ptr(), r.data_ptr(), rel_tol=1e-10, max_cycles=400, stream=sh)
            torch.cuda.synchronize()
            f.zero_()
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            mm.solve_device(f.data_ptr(), r.data_ptr(), rel_tol=1e-10, max_cycles=400, stream=sh)
            torch.cuda.synchronize()
            tot += time.perf_counter() - t1
        return tot

    t_mixed_seq = sequential(members, d_fi, d_rhs)
    for mm in members:
        mm.close()
    t_fp64 = 0.0
    for g, f, r in zip(grids, d_fi, d_rhs):  # one FP64 hierarchy at a time
        m64 = mg.Multigrid(*g, precision="fp64", device=local)
        t_fp64 += sequential([m64], [f], [r])
        m64.close()
    n = len(insts)
    return {"instances": n, "cells_total": int(sum(w.cells for w in insts)),
            "sizes": sorted({f"{w.jx}x{w.jy}x{w.jz}" for w in insts}),
            "value": n / tb, "unit": "solves/s", "ms_per_batch": tb * 1e3,
            "e2e": {"value": n / te, "unit": "solves/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "steps": ne, "all_converged": e2e_ok,
                    "note": "ples_mg_batch_solve on pinned host arrays (initial guesses and rhs in, "
                            "solutions out), copies inside"},
            "all_converged": ok, "max_rel_residual": relmax,
            "steps_per_outer_iteration": info["steps"],
            "sequential_fp64": {"value": n / t_fp64, "unit": "solves/s", "ms_total": t_fp64 * 1e3},
            "sequential_mixed": {"value": n / t_mixed_seq, "unit": "solves/s", "ms_total": t_mixed_seq * 1e3},
            "batch_over_sequential_fp64": t_fp64 / tb}


def serve_leg(args, local):
    """16 ensemble members on fixed grids, requests arriving as a Poisson
    process, each member's RHS the previous one plus 5% noise, warm starts,
    continuous batching in the server.  Latency = submission to completion,
    measured by the server.  Run at the configured aggregate rate and again
    at 70% of the throughput measured there (latency without a growing
    queue)."""
    import numpy as np
    from ples_gb300 import mg
    from ples_gb300 import synthetic as S
    ms = S.serve_members(16)
    handles = [mg.Multigrid(*w.grid(), device=local) for w in ms]
    srv = mg.Server(handles, hbm_budget_bytes=150e9)
    state = [w.rhs() for w in ms]
    rngs = [np.random.default_rng(2000 + i) for i in range(len(ms))]
    # warm-up: one cold solve per member
    for t in [srv.submit(i, state[i]) for i in range(len(ms))]:
        srv.wait(t)

    def run(rate, n, seed):
        at, who = S.poisson_arrivals(rate, n, seed=seed, members=len(ms))
        reqs = []
        for t, i in zip(at, who):
            state[i] = S.next_rhs(state[i], rngs[i])
            reqs.append((float(t), int(i), state[i]))
        t0 = time.perf_counter()
        tickets = []
        for t, i, r in reqs:
            d = t0 + t - time.perf_counter()
            if d > 0:
                time.sleep(d)
            tickets.append(srv.submit(i, r))
        lat, rel, ok, outer = [], 0.0, True, []
        for tk in tickets:
            _, st = srv.wait(tk)
            lat.append(st["seconds"] * 1e3)
            rel = max(rel, st["rel_residual"])
            outer.append(st["outer_iterations"])
            ok = ok and st["status"] == mg.OK
        span = time.perf_counter() - t0
        lat = np.array(lat)
        return {"offered_rate": rate, "requests": n, "solves_per_s": n / span,
                "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                "p999_ms": float(np.percentile(lat, 99.9)), "all_converged": ok, "max_rel_residual": rel,
                "outer_iterations_mean": float(np.mean(outer))}

    full = run(args.serve_rate, args.serve_requests, 7)
    # offered rates below the throughput measured at the full rate: the
    # highest one whose p99 stays within the bound is the capacity
    p99_bound_ms = 250.0
    sweep = {}
    for seed, frac in ((8, 0.7), (9, 0.5), (10, 0.9)):
        rate = frac * full["solves_per_s"]
        sweep[frac] = run(rate, max(32, int(rate * 2.0)), seed)
    light = sweep[0.7]
    ok = [v for v in sweep.values() if v["p99_ms"] <= p99_bound_ms]
    capacity = max(ok, key=lambda v: v["offered_rate"]) if ok else None
    srv.close()
    for h in handles:
        h.close()
    out = {"members": len(ms), "sizes": sorted({f"{w.jx}x{w.jy}x{w.jz}" for w in ms}),
           "cells_total": int(sum(w.cells for w in ms)), "hbm_budget_bytes": 150e9}
    out.update(full)
    out["at_70pct_throughput"] = light
    out["rate_sweep"] = [{"fraction_of_throughput": f, "offered_rate": v["offered_rate"], "p50_ms": v["p50_ms"],
                          "p99_ms": v["p99_ms"], "p999_ms": v["p999_ms"], "solves_per_s": v["solves_per_s"]}
                         for f, v in sorted(sweep.items())]
    out["capacity"] = ({"p99_bound_ms": p99_bound_ms, "offered_rate": capacity["offered_rate"],
                        "p50_ms": capacity["p50_ms"], "p99_ms": capacity["p99_ms"]}
                       if capacity else {"p99_bound_ms": p99_bound_ms, "offered_rate": None})
    out["note"] = "latency includes queueing whenever the offered rate exceeds the throughput"
    return out


def ib_leg(args, local):
    """512x256x512 channel (A 0.1, beta 3.0) with an immersed-boundary mask of
    32 seeded spheres, radius U(0.05, 0.2): mixed and plain FP64 solves to
    1e-10 from zero on device-resident inputs (CUDA events), and the HBM
    throughput of the eta-line smoother at every level (algorithmic 48 B per
    cell per sweep over its CUDA-event time)."""
    import numpy as np
    import torch
    from ples_gb300 import mg
    from ples_gb300 import synthetic as S
    w = S.WORKLOADS["channel_512x256x512"]
    x, y, z = w.grid()
    rhs = w.rhs()
    solid = S.sphere_mask(x, y, z, n=32, rmin=0.05, rmax=0.2, seed=11)
    nfi = (w.jx + 2) * (w.jy + 2) * (w.jz + 2)
    d_rhs = torch.from_numpy(np.ascontiguousarray(rhs.ravel(order="F"))).cuda()
    sh = torch.cuda.current_stream().cuda_stream
    stream = torch.cuda.current_stream()
    out = {"grid": f"{w.jx}x{w.jy}x{w.jz}", "cells": w.cells, "solid_fraction": float(solid.mean()),
           "spheres": 32}
    sols = {}
    for prec in ("mixed", "fp64"):
        m = mg.Multigrid(x, y, z, precision=prec, device=local, solid=solid)
        d_fi = torch.zeros(nfi, dtype=torch.float64, device="cuda")

        def solve():
            d_fi.zero_()
            return m.solve_device(d_fi.data_ptr(), d_rhs.data_ptr(), rel_tol=1e-10, max_cycles=400, stream=sh)

        st = solve()
        steps = args.ib_steps if prec == "mixed" else 1
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(steps):
            st = solve()
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        leg = {"solves_per_s": 1e3 / ms, "ms_per_solve": ms, "outer_iterations": st["outer_iterations"],
               "vcycles": st["vcycles"], "rel_residual": st["rel_residual"], "status": st["status"]}
        if prec == "mixed":
            levels = []
            es = 4 if prec == "mixed" else 8
            for lev in range(1, m.nlevel):
                m.time_kernel("line", lev)
                solve()
                kms, kn = m.kernel_time()
                m.time_kernel(None)
                nx, ny, nz = m.dims(lev)
                if kn:
                    per = kms / kn
                    levels.append({"level": lev, "dims": f"{nx}x{ny}x{nz}", "ms_per_sweep": per,
                                   "hbm_gbs": 12 * es * nx * ny * nz / (per / 1e3) / 1e9})
            leg["smoother_per_level"] = levels
        sols[prec] = d_fi.cpu().numpy().reshape((w.jx + 2, w.jy + 2, w.jz + 2), order="F")[1:-1, 1:-1, 1:-1]
        out[prec] = leg
        m.close()
        del d_fi
        torch.cuda.empty_cache()
    fl = ~solid
    a, b = sols["mixed"][fl], sols["fp64"][fl]
    out["err_mixed_vs_fp64"] = float(np.linalg.norm(a - b) / np.linalg.norm(b))
    out["mixed_over_fp64"] = out["mixed"]["solves_per_s"] / out["fp64"]["solves_per_s"]
    return out


def _report(args, m, w, ws, rank, dist, value, ms_per_step, outer, relres, t64, st64, err_vs_fp64,
            e2e_value, nfi, launches, kms, kn, clk, extra=None):
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    peak, peak_kind = _peaks()
    cells = w.cells
    avg_launch_s = kms / 1e3 / kn if kn else None
    achieved = LINE_BYTES_PER_CELL * cells / avg_launch_s / 1e9 if avg_launch_s else None
    kname = LINE_KERNELS.get(m.line_threads(1), "eta-line smoother")
    kernel = f"{kname} level 1, one sweep (its k-parity launches together)"
    traffic = LINE_TRAFFIC.get((args.workload, kname))
    cpu = None
    if not args.no_cpu_baseline:
        cpu = cpu_baseline(args.workload)
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic (seeded wavy-wall channel grid and divergence RHS)",
        "config": _workload_config(w),
        "solver": {"precision": "mixed: FP32 V-cycle; FP64 update/projection; outer residual FP64 differences, double-float products",
                   "parallelism": f"replicas x{ws}", "levels": m.nlevel,
                   "outer_iterations_mean": outer, "max_rel_residual": relres},
        "fp64": {"value": 1.0 / t64 if t64 else None, "unit": UNIT,
                 "ms_per_solve": t64 * 1e3 if t64 else None, "outer_iterations": st64["outer_iterations"]},
        "mixed_over_fp64": value / ws * t64 if t64 else None,
        "err_mixed_vs_fp64": err_vs_fp64,
        "e2e": {"value": e2e_value, "unit": UNIT,
                "h2d_bytes_per_step": 8 * (nfi + cells), "d2h_bytes_per_step": 8 * nfi},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak if achieved else None, "traffic": traffic,
                     "kernel": kernel,
                     "launches_timed": kn, "avg_launch_ms": avg_launch_s * 1e3 if avg_launch_s else None,
                     "peak_source": peak_kind,
                     "bytes_per_launch": LINE_BYTES_PER_CELL * cells},
        "clocks": clk,
        "cpu_baseline": cpu,
    }
    out.update(extra or {})
    print(json.dumps(out), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
