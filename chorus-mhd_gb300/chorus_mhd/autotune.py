"""Autotuner for the launch shapes of the cell passes.

For each order N it binds a representative solve (jittered Orszag-Tang sized so one
stage is a few milliseconds), then for each cell pass (E1, E2, E3 and the CT pass)
sweeps the cells per CTA ("epb") and threads per CTA, timing the pass with CUDA events
(``chorus_gpu_profile_stage``), and keeps the fastest shape.  E2 is tuned with the
exact-zero viscous skipping off, i.e. on its full work.  Results are cached per GPU
model in a JSON file (``~/.cache/chorus_gb300/tune_<gpu>.json`` unless
``CHORUS_TUNE_FILE`` names one) and applied by ``apply`` to any bound ``Solver``; the
batched form launches each order's passes with the shapes of the first solve of that
order it holds.

    python -m chorus_mhd.autotune            # tune N = 3..6 and write the cache
"""
from __future__ import annotations

import json
import os
import tempfile

from . import meshgen

PASSES = {"e1": 0, "e2": 2, "e3": 4}  # index into profile_stage's per-kernel times
# every warp multiple: a pass's loops hand out cells x (lines, points) items, and a shape
# whose item counts fill its warps evenly avoids paying for masked lanes
EPB_CANDIDATES = [1, 2, 3, 4, 5, 6, 8, 10, 12, 16]
THREAD_CANDIDATES = list(range(32, 513, 32))
SMEM_LIMIT = 200 * 1024


def cache_path(gpu_name: str) -> str:
    env = os.environ.get("CHORUS_TUNE_FILE")
    if env:
        return env
    safe = "".join(c if c.isalnum() else "_" for c in gpu_name)
    return os.path.join(os.path.expanduser("~"), ".cache", "chorus_gb300", "tune_%s.json" % safe)


def _smem_bytes(N: int, pass_: str, epb: int) -> int:
    NS, NFP = N * N, 2 * (N + 1) * N
    per = {"e1": NS * 9 + 2 * NS + NFP * 9, "e2": NFP * 16 + NS * 17,
           "e3": NFP * 10 + NS * 13}[pass_]
    return 8 * (epb * per + (NS if pass_ == "e1" else 0))


def tune_order(N: int, device: int = 0, cells_per_side: int | None = None, reps: int = 3) -> dict:
    from .solver import Mesh, Solver
    side = cells_per_side or max(32, int(round((2.0e6 / (N * N)) ** 0.5)))
    d = tempfile.mkdtemp(prefix="chorus_tune_")
    meshgen.write_case(meshgen.CaseSpec(nx=side, ny=side, N=N, problem="orszag_tang", jitter=0.1, seed=3), d)
    s = Solver(Mesh(d), device=device)
    s.iterations(2)
    best = {}
    for pass_, k in PASSES.items():
        if pass_ == "e2":
            s.set_option("skip_inactive_viscous", 0)
        trials = []
        for epb in EPB_CANDIDATES:
            if _smem_bytes(N, pass_, epb) > SMEM_LIMIT:
                continue
            for th in THREAD_CANDIDATES:
                s.set_option("epb_" + pass_, epb)
                s.set_option("threads_" + pass_, th)
                try:
                    ms = s.profile_stage(reps)[k]
                except Exception:
                    continue
                trials.append((ms, epb, th))
        trials.sort()
        ms, epb, th = trials[0]
        best[pass_] = {"epb": epb, "threads": th, "ms": ms, "trials": len(trials)}
        s.set_option("epb_" + pass_, epb)
        s.set_option("threads_" + pass_, th)
        if pass_ == "e2":
            s.set_option("skip_inactive_viscous", 1)
    best["cells"] = side * side
    s.close()
    return best


def tune(orders=(3, 4, 5, 6), device: int = 0) -> dict:
    from .solver import device_name
    name = device_name(device)
    out = {"gpu": name, "orders": {}}
    for N in orders:
        out["orders"][str(N)] = tune_order(N, device)
    p = cache_path(name)
    os.makedirs(os.path.dirname(p), exist_ok=True)
    with open(p, "w") as f:
        json.dump(out, f, indent=1)
    return out


SHIPPED = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuned")


def shipped_path(gpu_name: str) -> str:
    safe = "".join(c if c.isalnum() else "_" for c in gpu_name)
    return os.path.join(SHIPPED, "tune_%s.json" % safe)


_TABLES: dict = {}


def load(gpu_name: str) -> dict | None:
    """The user's cache for this GPU model if present, else the table shipped with the
    package (tuned on this model and committed)."""
    if gpu_name in _TABLES:
        return _TABLES[gpu_name]
    table = None
    for p in (cache_path(gpu_name), shipped_path(gpu_name)):
        if os.path.exists(p):
            with open(p) as f:
                table = json.load(f)
            break
    _TABLES[gpu_name] = table
    return table


def apply(solver, table: dict | None) -> bool:
    """Set the tuned shapes of the solver's order (no-op if the table lacks it)."""
    if not table:
        return False
    t = table.get("orders", {}).get(str(solver.N))
    if not t:
        return False
    for pass_ in ("e1", "e2", "e3"):  # the CT passes keep their built-in shape
        if pass_ in t:
            solver.set_option("epb_" + pass_, int(t[pass_]["epb"]))
            solver.set_option("threads_" + pass_, int(t[pass_]["threads"]))
    return True


if __name__ == "__main__":
    print(json.dumps(tune(), indent=1))
