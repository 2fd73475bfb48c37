"""Benchmark of the SD-MHD residual-and-time-step path on GB300.

Workload (one "step" = one full time step of iterations.f90:19-87: five SSP-RK
stages of compresid, the CT projection, and the norms every tenth step): the
single-large-solve configuration -- Orszag-Tang on a periodic 512x512 quad mesh with
interior nodes jittered by +-0.15h (seed 1), p = 4 (N = 5 solution points per
direction), FP64, gamma = 5/3, Rusanov flux, AV on, RK_S5P3, dt from CFL 0.1.
Synthetic seeded mesh in the reference's file formats (the reference ships none).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line.  The timed steps are the LAST K steps of the configuration's
stated run (C2: 200 steps, so steps 181-200 for K = 20): the state is advanced to the
window's first step untimed, W warm-up steps run and the window's first state is put
back, then the K steps are timed.  `value` is DOF*RK-stage/s with the state resident on
the device (CUDA events on the library's stream around the K steps replayed from a CUDA
graph); `e2e` is the same metric through the C-ABI with host buffers over the same
window (each step: Q uploaded from pinned host memory, one step, Q downloaded).
`--impl reference` times the CPU oracle (a plain-C restatement of the reference; the
Fortran reference cannot be built here) with every host thread, from the same window's
first state read through the restart reader.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "chorus-mhd_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

NX = 512
N_SOL = 5
JITTER = 0.15
SEED = 1
PROBLEM = "orszag_tang"
MU = 0.0    # physical viscosity and resistivity (the configurations are inviscid with AV)
ETA0 = 0.0

# the configurations of the metric: C2 is the default (the largest that fits one GPU and
# the one the metric is quoted on); C1 and C3 can be timed the same way
WORKLOADS = {
    "C2": dict(problem="orszag_tang", nx=512, n=5, jitter=0.15, seed=1),
    "C1": dict(problem="orszag_tang", nx=64, n=4, jitter=0.0, seed=0),
    "C3": dict(problem="rotor", nx=256, n=4, jitter=0.1, seed=1),
}


# number of time steps each configuration is stated at; the timed window is the last
# K steps of that run
RUN_STEPS = {"C2": 200, "C1": 1000, "C3": 500}
WORKLOAD = "C2"


def window(steps: int, total: int | None = None):
    """(first step - 1, last step) of the timed window: the last `steps` steps of the run."""
    total = RUN_STEPS[WORKLOAD] if total is None else total
    start = max(0, total - steps)
    return start, start + steps


def config_dict(nc: int, N: int, dof: int, steps: int, world: int) -> dict:
    """The workload description both arms print (identical for the same workload)."""
    start, end = window(steps)
    return {"workload": workload_name(), "cells": nc, "N": N, "dof": dof, "stages_per_step": 5,
            "window": "steps %d-%d of the %d-step run" % (start + 1, end, RUN_STEPS[WORKLOAD]),
            "l2": "inputs larger than L2 (the state Q alone is %.0f MB)" % (72.0 * dof / 1e6),
            "parallelism": "replicas" if world > 1 else "single GPU"}


def workload_name():
    bc = "periodic" if PROBLEM != "rotor" else "free"
    visc = "_mu%g_eta%g" % (MU, ETA0) if (MU or ETA0) else ""
    return "%s_%s_%dx%d_jitter%.2f_seed%d_p%d_N%d_fp64_rk_s5p3_av%s" % (PROBLEM, bc, NX, NX, JITTER, SEED, N_SOL - 1,
                                                                       N_SOL, visc)

METRIC = "DOF*RK-stage/s"
HBM_FALLBACK = 6800.0
FP64_PEAK_GOPS_FALLBACK = 600.0  # DFMA chains on this GB300 (600 G FMA/s); measured live when a GPU is present


def b_stage(N: int) -> float:
    """Algorithmic bytes per element per RK stage (compulsory traffic with perfect
    on-chip reuse): state r/w + RK register 216N^2, face traces 1728N, geometry and
    neighbour ids 144, CT once per step (24N^2 + 64N)/5."""
    return 216 * N * N + 1728 * N + 144 + (24 * N * N + 64 * N) / 5.0


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return HBM_FALLBACK, "fallback"


def make_case(tmp):
    from chorus_mhd import meshgen
    spec = meshgen.CaseSpec(nx=NX, ny=NX, N=N_SOL, problem=PROBLEM, jitter=JITTER, seed=SEED,
                            steps=RUN_STEPS[WORKLOAD], mu=MU, eta0=ETA0)
    d = os.path.join(tmp, "case")
    meshgen.write_case(spec, d)
    return d


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            # the timed region starts once the sampler is producing (nvidia-smi takes a
            # moment to start); at most two seconds
            t_end = time.time() + 2.0
            while not self.lines and time.time() < t_end and self.proc.poll() is None:
                time.sleep(0.01)
            self.lines.clear()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() in ("active", "1"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup(args):
    from chorus_mhd import dist
    return dist.init()


def barrier(world):
    from chorus_mhd import dist
    dist.barrier(world)


def max_over_ranks(world, x: float) -> float:
    from chorus_mhd import dist
    return dist.max_over_ranks(world, x)


def fp64_peak(device: int):
    """The FP64 pipe's FMA rate, measured now on this GPU (G FMA/s), or the fallback."""
    import ctypes
    from chorus_mhd import _lib
    v, ms = ctypes.c_double(), ctypes.c_double()
    try:
        if _lib.load().chorus_gpu_fp64_fma_peak(device, ctypes.byref(v), ctypes.byref(ms)) == 0:
            return v.value / 1e9, "measured now (DFMA chains, 64 warps per SM)"
    except Exception:
        pass
    return FP64_PEAK_GOPS_FALLBACK, "fallback"


def measure_window(sol, steps: int, warmup: int, world: int, restart_path: str | None = None,
                   clocks: bool = False, local: int = 0):
    """Time the last `steps` steps of the configuration's run on a bound solve at its
    initial state: advance untimed to the window, keep its first state (and write it as
    a restart stream when asked), run `warmup` steps, put the first state back, then time
    the window with CUDA events on the library's stream (one graph replay per step)."""
    import numpy as np
    import torch
    start, end = window(steps)
    if start:
        sol.iterations(start)
    nc = sol.ncell
    skip = bool(sol.get_option("skip_active"))
    frac0 = float(sol.array("viscous_cells", nc).mean()) if skip and start else None
    snap = torch.empty(sol.nq, dtype=torch.float64, pin_memory=True).numpy()
    sol.state(out=snap)
    it0, t0 = sol.iter, sol.ctime
    if restart_path:
        sol.write_restart(restart_path)
    sol.iterations(warmup)  # warm-up (builds the CUDA graphs on first use)
    sol.upload(snap)
    sol.iter, sol.ctime = it0, t0
    stream = torch.cuda.ExternalStream(sol.stream_handle(), device=local)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    per_step, per_diag = sol.launch_counts()
    ndiag = sum(1 for i in range(start + 1, end + 1) if i % 10 == 1)
    barrier(world)
    torch.cuda.synchronize()
    clk = ClockSampler(local) if clocks else None
    if clk:
        clk.__enter__()
    try:
        e0.record(stream)
        sol.iterations(steps)
        e1.record(stream)
        torch.cuda.synchronize()
        barrier(world)
    finally:
        if clk:
            clk.__exit__()
    ms = max_over_ranks(world, e0.elapsed_time(e1))
    frac1 = float(sol.array("viscous_cells", nc).mean()) if skip else None
    Q = sol.state()
    return {"ms": ms, "launches": per_step * steps + per_diag * ndiag, "start": start, "end": end,
            "snapshot": snap, "iter0": it0, "ctime0": t0, "finite": bool(np.isfinite(Q).all()),
            "visc": {"skip_inactive_viscous": skip, "fraction_of_cells_with_viscous_flux_at_window_start": frac0,
                     "fraction_of_cells_with_viscous_flux_at_window_end": frac1},
            "clocks": clk.summary() if clk else None}


def measure_e2e(sol, snap, it0, t0, steps: int, warmup: int, world: int):
    """The window again through the C-ABI with a host-resident state: every step uploads
    Q from pinned host memory, runs one step and downloads Q (chorus_gpu_step_host)."""
    import torch
    qt = torch.empty(sol.nq, dtype=torch.float64, pin_memory=True)
    qh = qt.numpy()
    qh[:] = snap
    for _ in range(max(1, min(warmup, 3))):  # untimed: first use of the copy stream and events
        sol.step_host(qh, qh, 1)
    qh[:] = snap
    sol.iter, sol.ctime = it0, t0
    barrier(world)
    t_0 = time.perf_counter()
    for _ in range(steps):
        sol.step_host(qh, qh, 1)
    t_1 = time.perf_counter()
    e2e_s = max_over_ranks(world, t_1 - t_0)
    dof = sol.ncell * sol.N * sol.N
    link = link_rates(qt)
    return {"value": world * dof * 5 * steps / e2e_s, "unit": METRIC, "h2d_bytes_per_step": 8 * sol.nq,
            "d2h_bytes_per_step": 8 * sol.nq, "steps": steps, "ms_per_step": e2e_s / steps * 1e3,
            "link_gbs": link, "copy_ms_per_step": 8 * sol.nq / 1e6 * (1 / link["h2d"] + 1 / link["d2h"])}


def link_rates(h) -> dict:
    """Host link rates of this process (GB/s): one copy of the state each way between the
    pinned host tensor h and a device buffer, CUDA events around each, best of two."""
    import torch
    g = torch.empty(h.numel(), dtype=torch.float64, device="cuda")
    best = {"h2d": 0.0, "d2h": 0.0}
    for _ in range(2):
        for k, (dst, src) in (("h2d", (g, h)), ("d2h", (h, g))):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            dst.copy_(src, non_blocking=True)
            b.record()
            b.synchronize()
            best[k] = max(best[k], 8 * h.numel() / (a.elapsed_time(b) * 1e6))
    del g
    return best


def run_other_workloads(args, local, tmp, world):
    """The configurations other than the headline one, timed the same way (window at the
    end of each one's stated run), for the record."""
    global NX, N_SOL, JITTER, SEED, PROBLEM, WORKLOAD
    from chorus_mhd import Mesh, Solver
    saved = (NX, N_SOL, JITTER, SEED, PROBLEM, WORKLOAD)
    out = {}
    try:
        for name in ("C1", "C3"):
            if name == saved[5]:
                continue
            w = WORKLOADS[name]
            WORKLOAD, PROBLEM, JITTER, SEED, NX, N_SOL = name, w["problem"], w["jitter"], w["seed"], w["nx"], w["n"]
            d = make_case(os.path.join(tmp, name))
            mesh = Mesh(d)
            sol = Solver(mesh, device=local)
            r = measure_window(sol, args.steps, args.warmup, world, local=local)
            dof = sol.ncell * sol.N * sol.N
            e2e = measure_e2e(sol, r["snapshot"], r["iter0"], r["ctime0"], args.steps, args.warmup, world)
            out[name] = {"workload": workload_name(), "window": config_dict(sol.ncell, sol.N, dof, args.steps,
                                                                           world)["window"],
                         "value": world * dof * 5 * args.steps / (r["ms"] / 1e3), "unit": METRIC,
                         "ms_per_step": r["ms"] / args.steps, "e2e": e2e, "viscous_work": r["visc"],
                         "state_finite": r["finite"]}
            sol.close()
            mesh.close()
    finally:
        NX, N_SOL, JITTER, SEED, PROBLEM, WORKLOAD = saved
    return out


def run_gpu(args):
    import torch
    from chorus_mhd import Mesh, Solver

    world, rank, local = dist_setup(args)
    torch.cuda.set_device(local)
    tmp = tempfile.mkdtemp(prefix="chorus_bench_")
    d = make_case(tmp)
    mesh = Mesh(d)
    sol = Solver(mesh, device=local)
    N, nc = mesh.N, mesh.ncell
    dof = nc * N * N
    fp64_gops, fp64_kind = fp64_peak(local)
    restart = os.path.join(tmp, "window_start.dat") if rank == 0 and world == 1 and not args.no_cpu_baseline else None
    r = measure_window(sol, args.steps, args.warmup, world, restart_path=restart, clocks=True, local=local)
    ms = r["ms"]
    value = world * dof * 5 * args.steps / (ms / 1e3)

    # per-kernel stage profile (after the timed region; events around each kernel)
    prof = sol.profile_stage(5)
    # profile slots: E1, F1, E2, (the former face-average pass, now inside E2 and E3), E3
    names = ["e1_interp_inviscid_sensor", "f1_rusanov_faces", "e2_gradients_face_av", None,
             "e3_viscous_divergence_rk"]
    kernel_ms = {n: prof[k] for k, n in enumerate(names) if n}
    dom = max((k for k in range(5) if names[k]), key=lambda k: prof[k])
    hbm_peak, peak_kind = measured_peaks()
    stage_ms = prof[5]
    achieved = b_stage(N) * nc / (stage_ms / 1e3) / 1e9
    # the counted figures belong to the inviscid Orszag-Tang stage they were measured on
    counted = PROBLEM == "orszag_tang" and MU == 0.0 and ETA0 == 0.0
    ops = FP64_PER_ELEMENT_STAGE.get(N) if counted else None
    fp64 = {"peak_measured_gfma_per_s": fp64_gops, "peak_kind": fp64_kind}
    if ops:
        n_ops, n_flops = ops
        gops = n_ops * nc / (stage_ms / 1e3) / 1e9
        eq = FP64_FORM_OPS_PER_ELEMENT_STAGE[N] * nc / (stage_ms / 1e3) / 1e9
        fp64.update({"bound": "fp64 pipe", "achieved_gops": gops, "peak_gops": fp64_gops,
                     "frac": gops / fp64_gops, "unit": "G FP64 instructions/s (thread level)",
                     "ops_per_element_stage": n_ops, "flops_per_element_stage": n_flops,
                     "achieved_tflops": n_flops * nc / (stage_ms / 1e3) / 1e12,
                     "source": "ncu SASS counters of the four stage kernels, Orszag-Tang 262x262 N=5",
                     "integer_line_operators": {
                         "note": "Lmat/Mmat line operators run as exact integer dot products on the integer pipes; "
                                 "the FP64 pipe keeps the fluxes",
                         "fp64_form_ops_per_element_stage": FP64_FORM_OPS_PER_ELEMENT_STAGE[N],
                         "fp64_form_equivalent_gops": eq, "fp64_form_equivalent_frac": eq / fp64_gops}})
    traffic = None
    if counted and TRAFFIC_PER_ELEMENT_STAGE.get(N):
        traffic = TRAFFIC_PER_ELEMENT_STAGE[N] * nc

    # end to end through the C-ABI with host buffers, over the same window
    e2e = measure_e2e(sol, r["snapshot"], r["iter0"], r["ctime0"], args.steps, args.warmup, world)

    sol.close()
    mesh.close()
    others = None
    if not args.no_other_workloads:
        others = run_other_workloads(args, local, tmp, world)
    ens = None
    if not args.no_ensemble:
        ens = run_ensemble(args, local, tmp)
    srv = None
    if not args.no_serving:
        srv = run_serving(args, local, tmp)
    cpu = None
    if restart:
        cpu = cpu_baseline(d, dof, restart, r["start"])
        os.remove(restart)
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded %s %dx%d mesh, jitter %.2f h, %s initial data)" % (
            "periodic" if PROBLEM != "rotor" else "FREE-boundary", NX, NX, JITTER, PROBLEM),
        "config": config_dict(nc, N, dof, args.steps, world),
        "e2e": e2e,
        "gpu_launches": r["launches"],
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved / hbm_peak, "traffic": traffic,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of the four stage "
                                       "kernels at 262x262, scaled by cells (bytes per cell are size-independent)",
                     "kernel": "one RK stage (4 launches: %s)" % ", ".join(n for n in names if n),
                     "algorithmic_bytes_per_element_stage": b_stage(N), "peak_kind": peak_kind,
                     "stage_ms": stage_ms, "dominant_kernel": names[dom],
                     "kernel_ms": kernel_ms},
        "fp64_pipe": fp64,
        "cpu_baseline": cpu,
        "clocks": r["clocks"],
        "state_finite": r["finite"],
        "viscous_work": r["visc"],
        "other_workloads": others,
        "ensemble": ens,
        "serving": srv,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_ensemble(args, device, tmp):
    """The batched configuration: 256 seeded solves of mixed size (32..256 cells per side,
    log-uniform), order (N = 3..6) and problem, advanced as one batch and as the plain
    per-solve loop (each solve's own CUDA-graph step, one solve after another)."""
    import numpy as np
    import torch
    from chorus_mhd import Batch, Mesh, Solver, ensemble
    from chorus_mhd import dist
    world, rank, _ = dist.env()
    # whole solves shard across ranks (no data-path exchange)
    specs = dist.shard(ensemble.draw(count=args.ensemble_count), world, rank)
    t0 = time.perf_counter()
    dirs = ensemble.write_all(specs, os.path.join(tmp, "ensemble"))
    solvers = []
    for dd in dirs:
        s = Solver(Mesh(dd), device=device)
        s.set_option("diagnostics", 0)
        solvers.append(s)
    t_setup = time.perf_counter() - t0
    dof_local = sum(s.ncell * s.N * s.N for s in solvers)
    dof = int(dist.sum_over_ranks(world, float(dof_local)))
    K = args.ensemble_steps
    # plain loop: warm-up builds every solve's graph
    for s in solvers:
        s.iterations(1)
    torch.cuda.synchronize()
    dist.barrier(world)
    # timed both ways: wall clock, and CUDA events from the first solve's stream (start)
    # to the last solve's stream (end); the loop is serial, each solve's steps end before
    # the next solve's begin
    p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    p0.record(torch.cuda.ExternalStream(solvers[0].stream_handle(), device=device))
    t0 = time.perf_counter()
    for s in solvers:
        s.iterations(K)
    p1.record(torch.cuda.ExternalStream(solvers[-1].stream_handle(), device=device))
    torch.cuda.synchronize()
    t_plain = dist.max_over_ranks(world, time.perf_counter() - t0)
    ms_plain = dist.max_over_ranks(world, p0.elapsed_time(p1))
    b = Batch(device)
    for s in solvers:
        b.add(s)
    b.step(1)
    b.sync()
    stream = torch.cuda.ExternalStream(b.stream_handle(), device=device)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    dist.barrier(world)
    t0 = time.perf_counter()
    e0.record(stream)
    b.step(K)
    e1.record(stream)
    b.sync()
    t_batch = dist.max_over_ranks(world, time.perf_counter() - t0)
    ms_batch = dist.max_over_ranks(world, e0.elapsed_time(e1))
    info = b.info()
    finite = all(bool(np.isfinite(s.state()).all()) for s in solvers[:8])
    b.close()
    for s in solvers:
        s.close()
    Ns = {}
    for s in solvers:
        Ns[s.N] = Ns.get(s.N, 0) + 1
    v_b, v_p = dof * 5 * K / (ms_batch / 1e3), dof * 5 * K / (ms_plain / 1e3)
    return {"solves": int(dist.sum_over_ranks(world, float(len(solvers)))), "dof": dof,
            "cells": int(dist.sum_over_ranks(world, float(sum(s.ncell for s in solvers)))), "steps": K,
            "N_counts": {str(k): v for k, v in sorted(Ns.items())}, "setup_s": t_setup,
            "timing": "both legs by CUDA events (value, ms_per_step) and by the host wall clock (wall_*)",
            "batched": {"value": v_b, "unit": METRIC, "ms_per_step": ms_batch / K,
                        "wall_value": dof * 5 * K / t_batch, "wall_ms_per_step": t_batch * 1e3 / K,
                        "cell_tiles": info["cell_tiles"], "face_tiles": info["face_tiles"]},
            "plain_loop": {"value": v_p, "unit": METRIC, "ms_per_step": ms_plain / K,
                           "wall_value": dof * 5 * K / t_plain, "wall_ms_per_step": t_plain * 1e3 / K},
            "batched_over_plain": v_b / v_p,
            "batched_over_plain_wall": t_plain / t_batch,
            "spot_check_finite": finite,
            "draw": "ensemble.draw(count=%d, lo=32, hi=256, seed=2024): rotor side >= ceil(192/N)"
                    % args.ensemble_count}


def run_serving(args, device, tmp):
    """Poisson request streams (end times U(0.1, 1.0)) over a pool of small mixed solves,
    served with continuous batching under a 120 GB budget and by the plain sequential
    loop; p50/p99 time-to-solution and throughput per arrival rate.  A last stream at the
    highest rate runs under a budget of a few solves, so that admission waits for memory."""
    from chorus_mhd import Mesh, serve
    dirs = serve.serving_cases(os.path.join(tmp, "serving"))
    budget = 120 * 10 ** 9
    out = {"pool": "ensemble.draw(count=24, lo=16, hi=32, seed=11, problems=(orszag_tang, alfven))",
           "hbm_budget_bytes": budget, "requests_per_rate": args.serving_requests, "rates": {}}
    serve.serve([(dirs[0], 0.0, 0.01)], mode="batched")  # warm-up
    for rate in args.serving_rates:
        reqs = serve.poisson_requests(rate, args.serving_requests, dirs, seed=int(rate))
        rb, mb = serve.serve(reqs, mode="batched", hbm_budget_bytes=budget, device=device)
        rs, ms = serve.serve(reqs, mode="sequential", device=device)
        b, q = serve.summarize(rb, mb), serve.summarize(rs, ms)
        out["rates"][str(rate)] = {"batched": b, "sequential": q,
                                   "throughput_ratio": b["throughput_dof_stage_per_s"] / max(q["throughput_dof_stage_per_s"], 1e-30),
                                   "p99_ratio_sequential_over_batched": q["p99_latency_s"] / max(b["p99_latency_s"], 1e-30)}
    out["budget_binds_at_120GB"] = any(v["batched"]["waited_for_memory"] for v in out["rates"].values())
    # the same highest-rate stream under a budget of about four of the pool's largest solves
    from chorus_mhd import _lib
    big = 0
    for d in dirs:
        m = Mesh(d)
        big = max(big, int(_lib.load().chorus_mesh_device_bytes(m._h)))
        m.close()
    small = 4 * big
    rate = max(args.serving_rates)
    reqs = serve.poisson_requests(rate, args.serving_requests, dirs, seed=int(rate))
    rb, mb = serve.serve(reqs, mode="batched", hbm_budget_bytes=small, device=device)
    out["small_budget"] = {"hbm_budget_bytes": small, "rate": rate, "batched": serve.summarize(rb, mb)}
    return out


def run_serving_mix(args):
    """The serving configuration on its stated mix: Poisson arrivals of solves drawn from
    the batched configuration's population (cells per side log-uniform on 32..256, N in
    3..6, Orszag-Tang / rotor / Alfven, rotor sides raised to 192 points), end times
    U(0.1, 1.0), admitted under a 120 GB budget, served by continuous batching and by the
    plain sequential loop.  Each stream has the same `--serving-requests` requests (same
    cases and end times at every rate; only the arrival times scale with the rate).  A
    request averages about ten seconds of GPU work with a tail of minutes, so at every
    stated rate (10-500 per second) a stream's requests have all arrived long before the
    first large ones finish: the run is bounded by the requests, not the rates.  One more
    batched stream runs under a budget of a few of its largest solves, so that admission
    waits for memory."""
    import numpy as np
    import torch
    from chorus_mhd import Mesh, _lib, ensemble, serve
    torch.cuda.set_device(0)
    tmp = tempfile.mkdtemp(prefix="chorus_c5_")
    pool = ensemble.draw(count=256)
    rng = np.random.default_rng(5)
    picks = rng.integers(0, len(pool), args.serving_requests)
    ends = rng.uniform(0.1, 1.0, args.serving_requests)
    dirs = {}
    for i in sorted(set(int(p) for p in picks)):
        dirs[i] = ensemble.write_all([pool[i]], os.path.join(tmp, "case%03d" % i))[0]
    sizes = {}
    steps_total, work = 0, 0.0
    for i, e in zip(picks, ends):
        m = Mesh(dirs[int(i)])
        sizes[int(i)] = int(_lib.load().chorus_mesh_device_bytes(m._h))
        k = int(math.ceil(e / m.params.dt - 1e-9))
        steps_total += k
        work += 5.0 * m.ncell * m.N * m.N * k
        m.close()
    budget = 120 * 10 ** 9
    arrivals = np.cumsum(np.random.default_rng(6).exponential(1.0, args.serving_requests))
    out = {"metric": "p50/p99 time-to-solution (s) and throughput, serving stream", "impl": "chorus",
           "config": {"workload": "serving: Poisson arrivals of the 256-solve population (sides 32-256 log-uniform, "
                                  "N 3-6, Orszag-Tang/rotor/Alfven), end times U(0.1,1.0), 120 GB budget",
                      "requests_per_stream": args.serving_requests, "dof_stage_work": work, "steps": steps_total,
                      "largest_request_bytes": max(sizes.values())},
           "rates": {}}
    serve.serve([(dirs[int(picks[0])], 0.0, 0.001)], mode="batched")  # warm-up
    for rate in args.serving_rates:
        reqs = [(dirs[int(p)], float(a / rate), float(e)) for p, a, e in zip(picks, arrivals, ends)]
        rb, mb = serve.serve(reqs, mode="batched", hbm_budget_bytes=budget)
        rs, ms = serve.serve(reqs, mode="sequential")
        b, q = serve.summarize(rb, mb), serve.summarize(rs, ms)
        out["rates"][str(rate)] = {"batched": b, "sequential": q,
                                   "throughput_ratio": b["throughput_dof_stage_per_s"] / max(q["throughput_dof_stage_per_s"], 1e-30),
                                   "p99_ratio_sequential_over_batched": q["p99_latency_s"] / max(b["p99_latency_s"], 1e-30)}
        print(json.dumps({"rate": rate, **out["rates"][str(rate)]}), flush=True)
    out["budget_binds_at_120GB"] = any(v["batched"]["waited_for_memory"] for v in out["rates"].values())
    small = 3 * max(sizes.values())
    rate = max(args.serving_rates)
    reqs = [(dirs[int(p)], float(a / rate), float(e)) for p, a, e in zip(picks, arrivals, ends)]
    rb, mb = serve.serve(reqs, mode="batched", hbm_budget_bytes=small)
    out["small_budget"] = {"hbm_budget_bytes": small, "rate": rate, "batched": serve.summarize(rb, mb)}
    print(json.dumps(out), flush=True)


# per element per RK stage, from ncu on the four stage kernels (Orszag-Tang 262x262,
# N=5, after the warm-up steps): FP64 thread instructions (DFMA + DADD + DMUL) and flops
# (2*DFMA + DADD + DMUL); DRAM bytes read + written.  FP64_FORM_... is the count of the
# same stage with the line operators in FP64 as well (measured the same way before they
# moved to the integer pipes): the stage's work in FP64-instruction units.
FP64_PER_ELEMENT_STAGE: dict = {5: (5388, 7678)}
FP64_FORM_OPS_PER_ELEMENT_STAGE: dict = {5: 10638}
TRAFFIC_PER_ELEMENT_STAGE: dict = {5: 28264}


def cpu_baseline(case_dir, dof, restart, start, warm=1, timed=2):
    """The oracle on the host cores, a bounded sample of the same window: it reads the
    window's first state through its restart reader (read_data_restart.f90:35-67), runs
    a warm-up step, reads the state again and times `timed` steps from it."""
    import oracle
    threads = os.cpu_count() or 1
    o = oracle.Oracle(case_dir, threads=threads)
    if o.read_restart(restart) != 0:
        raise RuntimeError("oracle could not read " + restart)
    for _ in range(warm):
        o.step()
    o.read_restart(restart)
    t0 = time.perf_counter()
    for _ in range(timed):
        o.step()
    dt = time.perf_counter() - t0
    v = dof * 5 * timed / dt
    o.close()
    return {"value": v, "unit": METRIC, "cores": threads, "kind": "port",
            "sample": "steps %d-%d of the same %dx%d N=%d solve (after %d warm-up), started from the window's first "
                      "state through the restart reader, OpenMP over cells/faces"
                      % (start + 1, start + timed, NX, NX, N_SOL, warm), "seconds": dt}


def prepare_window_state(case_dir: str, start: int, out: str) -> str | None:
    """The state at the window's first step as a restart file, computed by the library
    on the GPU in a child process (the oracle would need minutes of CPU time per step of
    the big workloads to get there); None when no GPU can do it."""
    if start <= 0:
        return None
    cmd = [sys.executable, os.path.abspath(__file__), "--workload", WORKLOAD, "--prepare-window-state", case_dir,
           str(start), out]
    if NX != WORKLOADS[WORKLOAD]["nx"]:
        cmd += ["--nx", str(NX)]
    if N_SOL != WORKLOADS[WORKLOAD]["n"]:
        cmd += ["--order-n", str(N_SOL)]
    env = dict(os.environ)
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK", "LOCAL_WORLD_SIZE", "MASTER_ADDR", "MASTER_PORT"):
        env.pop(k, None)
    try:
        r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, env=env)
    except Exception:
        return None
    return out if r.returncode == 0 and os.path.exists(out) else None


def write_window_state(case_dir: str, start: int, out: str) -> None:
    """Child-process side of prepare_window_state."""
    from chorus_mhd import Mesh, Solver
    mesh = Mesh(case_dir)
    sol = Solver(mesh, device=0)
    sol.set_option("diagnostics", 0)
    sol.iterations(start)
    sol.write_restart(out)
    sol.close()
    mesh.close()


def run_reference(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import oracle
    tmp = tempfile.mkdtemp(prefix="chorus_ref_")
    d = make_case(tmp)
    start, end = window(args.steps)
    restart = prepare_window_state(d, start, os.path.join(tmp, "window_start.dat"))
    threads = os.cpu_count() or 1
    o = oracle.Oracle(d, threads=threads)
    nc = o.geti("NCELL")
    N = o.geti("N")
    dof = nc * N * N
    if restart and o.read_restart(restart) != 0:
        raise RuntimeError("oracle could not read " + restart)
    first = o.geti("iter") + 1
    # bounded sample: every warm-up/timed step is one full time step of the workload,
    # capped so the whole run stays within a few minutes; the warm-up steps are undone
    # by reading the window's first state again
    t_est = None
    for _ in range(args.warmup):
        t0 = time.perf_counter()
        o.step()
        t_est = time.perf_counter() - t0
    if restart:
        o.read_restart(restart)
    else:
        o.close()
        o = oracle.Oracle(d, threads=threads)
    k = args.steps
    if t_est and t_est * k > 90:
        k = max(1, int(90 / t_est))
    t0 = time.perf_counter()
    for _ in range(k):
        o.step()
    dt = time.perf_counter() - t0
    v = dof * 5 * k / dt
    src = ("the window's first state (step %d), computed by the library on the GPU in a child process and read "
           "through the oracle's restart reader" % start) if restart else "the initial state"
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": METRIC, "n_gpus": world, "steps": k,
            "warmup": args.warmup, "ms_per_step": dt / k * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (same seeded case)",
            "config": config_dict(nc, N, dof, args.steps, world),
            "cpu_baseline": {"value": v, "unit": METRIC, "cores": threads, "kind": "port",
                             "sample": "steps %d-%d (%d of the %d requested, after %d warm-up) from %s"
                                       % (first, first + k - 1, k, args.steps, args.warmup, src)},
            "e2e": {"value": v, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "plain-C restatement of the reference (the Fortran+MPI reference cannot be compiled: no "
                    "Fortran compiler or MPI on the machines); its cost per step does not depend on the state "
                    "(it evaluates every flux everywhere)"}
    print(json.dumps(line), flush=True)
    o.close()


def main():
    global NX, N_SOL, JITTER, SEED, PROBLEM, MU, ETA0, WORKLOAD
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="C2", choices=sorted(WORKLOADS) + ["C4", "C5"],
                    help="C2: Orszag-Tang 512^2 jittered N=5 (default); C1: Orszag-Tang 64^2 N=4; "
                         "C3: rotor 256^2 jittered N=4, FREE boundaries; C4: the ensemble leg alone "
                         "(--ensemble-count solves, its own JSON line); C5: the serving stream on its "
                         "stated mix (its own JSON line)")
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="chorus", choices=["chorus", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-ensemble", action="store_true")
    ap.add_argument("--no-other-workloads", action="store_true")
    ap.add_argument("--run-steps", type=int, default=None,
                    help="length of the run whose last --steps steps are timed (default: the configuration's "
                         "stated run; a short run keeps profiler captures small)")
    ap.add_argument("--prepare-window-state", nargs=3, metavar=("CASE", "STEP", "OUT"), default=None,
                    help=argparse.SUPPRESS)
    ap.add_argument("--ensemble-count", type=int, default=256)
    ap.add_argument("--ensemble-steps", type=int, default=3)
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--serving-requests", type=int, default=24)
    ap.add_argument("--serving-rates", type=float, nargs="+", default=[10.0, 20.0, 50.0, 100.0, 200.0, 500.0])
    ap.add_argument("--nx", type=int, default=None, help="cells per side (default: the workload's)")
    ap.add_argument("--order-n", type=int, default=None, help="solution points per direction")
    ap.add_argument("--mu", type=float, default=0.0, help="physical viscosity (the configurations use 0)")
    ap.add_argument("--eta0", type=float, default=0.0, help="resistivity (the configurations use 0)")
    args = ap.parse_args()
    if args.workload == "C5":
        run_serving_mix(args)
        return
    if args.workload == "C4":
        import torch
        torch.cuda.set_device(0)
        print(json.dumps({"metric": METRIC, "impl": "chorus",
                          "ensemble": run_ensemble(args, 0, tempfile.mkdtemp(prefix="chorus_c4_"))}), flush=True)
        return
    MU, ETA0 = args.mu, args.eta0
    WORKLOAD = args.workload
    if args.run_steps:
        RUN_STEPS[WORKLOAD] = max(args.run_steps, 1)
    w = WORKLOADS[args.workload]
    PROBLEM, JITTER, SEED = w["problem"], w["jitter"], w["seed"]
    NX = args.nx if args.nx else w["nx"]
    N_SOL = args.order_n if args.order_n else w["n"]
    if args.prepare_window_state:
        case, step, out = args.prepare_window_state
        write_window_state(case, int(step), out)
        return
    if args.workload != "C2":  # the ensemble, serving and other-workload legs belong to the default line
        args.no_ensemble = args.no_serving = args.no_other_workloads = True
    if args.warmup < 3 and args.impl != "reference":
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
