"""Serving form: Poisson request streams served with continuous batching.

``serve(requests, mode=...)`` runs libchorus_gpu's native request loop
(``chorus_serve_run``): requests are admitted at step boundaries while their device
memory fits the HBM budget, packed into one batch step, and retired after their last
step; ``mode="sequential"`` is the plain loop (one solve at a time, first come first
served).  ``poisson_requests`` builds a seeded stream.
"""
from __future__ import annotations

import ctypes
import math
import os

import numpy as np

from . import _lib, ensemble, meshgen
from ._lib import ChorusServeConfig, ChorusServeRequest, ChorusServeResult, check


def poisson_requests(rate: float, count: int, case_dirs: list[str], seed: int = 7, t_lo: float = 0.1,
                     t_hi: float = 1.0):
    """count requests with exponential inter-arrival times (rate per second); each picks
    one of case_dirs uniformly and an end time uniform on [t_lo, t_hi]."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, count))
    picks = rng.integers(0, len(case_dirs), count)
    ends = rng.uniform(t_lo, t_hi, count)
    return [(case_dirs[int(p)], float(a), float(e)) for p, a, e in zip(picks, t, ends)]


def serve(requests, mode: str = "batched", hbm_budget_bytes: int = 0, device: int = 0, max_active: int = 0,
          gpu_setup: bool = False):
    """Run the request loop; returns (per-request dicts, makespan seconds).

    A request is (case_dir, arrival_s, end_time) or (case_dir, arrival_s, end_time, out)
    where out may hold "Q" (a contiguous float64 array of the solve's 9*N*N*NCELL doubles,
    filled with the final state) and "restart" (a path that receives the final state as a
    restart stream).  gpu_setup builds each request's maps and geometry on the device."""
    L = _lib.load()
    n = len(requests)
    arr = (ChorusServeRequest * n)()
    keep = []
    for i, r in enumerate(requests):
        d, a, e = r[:3]
        out = r[3] if len(r) > 3 and r[3] else {}
        b = d.encode()
        keep.append(b)
        arr[i].case_dir = b
        arr[i].arrival_s = a
        arr[i].end_time = e
        q = out.get("Q")
        if q is not None:
            if q.dtype != np.float64 or not q.flags.c_contiguous or not q.flags.writeable:
                raise ValueError("Q output must be a writeable contiguous float64 array")
            keep.append(q)
            arr[i].Q_out = q.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
            arr[i].Q_out_count = q.size
        if out.get("restart"):
            rb = str(out["restart"]).encode()
            keep.append(rb)
            arr[i].restart_path = rb
    cfg = ChorusServeConfig(device=device, mode=1 if mode == "sequential" else 0,
                            hbm_budget_bytes=int(hbm_budget_bytes), max_active=int(max_active),
                            gpu_setup=1 if gpu_setup else 0)
    out = (ChorusServeResult * n)()
    mk = ctypes.c_double()
    check(L.chorus_serve_run(arr, n, ctypes.byref(cfg), out, ctypes.byref(mk)))
    res = [dict(admit_s=r.admit_s, finish_s=r.finish_s, latency_s=r.latency_s, wait_s=r.wait_s, ctime=r.ctime,
                dof=r.dof, steps=r.steps, status=r.status) for r in out]
    return res, mk.value


def summarize(res, makespan):
    ok = [r for r in res if r["status"] == 0]
    lat = np.array([r["latency_s"] for r in ok]) if ok else np.zeros(1)
    work = sum(r["dof"] * 5 * r["steps"] for r in ok)
    waits = [r.get("wait_s", 0.0) for r in ok]
    return {"requests": len(res), "completed": len(ok), "makespan_s": makespan,
            "p50_latency_s": float(np.percentile(lat, 50)), "p99_latency_s": float(np.percentile(lat, 99)),
            "mean_latency_s": float(lat.mean()), "throughput_dof_stage_per_s": work / makespan if makespan else 0.0,
            "waited_for_memory": int(sum(1 for w in waits if w > 0)),
            "total_wait_for_memory_s": float(sum(waits))}


def serving_cases(root: str, count: int = 24, seed: int = 11):
    """A pool of small mixed solves for request streams: sides 16..32 (log-uniform),
    N = 3..6, Orszag-Tang and Alfven.  The rotor is left out of streams: it needs about
    192 solution points per side, which makes each request 10-100x heavier than the rest
    and the 10-500 requests/s sweep meaningless on one GPU."""
    specs = ensemble.draw(count=count, lo=16, hi=32, seed=seed, problems=("orszag_tang", "alfven"))
    return ensemble.write_all(specs, root)
