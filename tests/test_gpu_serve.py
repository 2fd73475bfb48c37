"""Serving form: continuous batching of Poisson arrivals under an HBM budget."""
import os

import numpy as np
import pytest

from chorus_mhd import Mesh, Solver, serve
from helpers import make_case

pytestmark = pytest.mark.gpu


def _alone(d, steps):
    """The same solve run alone: its own context, the single-solve CUDA-graph step."""
    s = Solver(Mesh(d))
    s.set_option("diagnostics", 0)
    s.iterations(steps)
    Q = s.state()
    t = s.ctime
    s.close()
    return Q, t


def test_each_result_same_alone_and_in_the_mix(case_root, tmp_path):
    """Overlapping requests served by the continuous-batching loop hand back their final
    state (Q_out) and a restart file; each equals the same solve run alone, bit for bit,
    and the restart file is the one the alone run writes."""
    specs = [dict(problem="orszag_tang", nx=10, ny=10, N=4, jitter=0.1, seed=1),
             dict(problem="alfven", nx=8, ny=8, N=3),
             dict(problem="orszag_tang", nx=6, ny=8, N=5, jitter=0.1, seed=2),
             dict(problem="rotor", nx=64, ny=64, N=3, jitter=0.1, seed=5)]
    dirs = [make_case(case_root, **sp) for sp in specs]
    # arrivals overlap: every request arrives while earlier ones are still on the GPU,
    # and the first case is requested twice with different end times
    plan = [(dirs[0], 0.0, 0.05), (dirs[1], 0.001, 0.08), (dirs[2], 0.002, 0.03), (dirs[3], 0.003, 0.0015),
            (dirs[0], 0.004, 0.02)]
    outs = []
    reqs = []
    for k, (d, a, e) in enumerate(plan):
        m = Mesh(d)
        o = {"Q": np.empty(9 * m.N * m.N * m.ncell), "restart": str(tmp_path / ("served_%d.dat" % k))}
        m.close()
        outs.append(o)
        reqs.append((d, a, e, o))
    res, mk = serve.serve(reqs, mode="batched")
    assert all(r["status"] == 0 for r in res), res
    # the solves shared steps of the batch: some request was admitted before another finished
    spans = sorted((r["admit_s"], r["finish_s"]) for r in res)
    assert any(b[0] < a[1] for a, b in zip(spans, spans[1:]))
    for (d, _, tend), r, o in zip(plan, res, outs):
        m = Mesh(d)
        assert r["steps"] == int(np.ceil(tend / m.params.dt - 1e-9))
        m.close()
        Q, t = _alone(d, r["steps"])
        assert r["ctime"] == t
        assert np.array_equal(o["Q"], Q)
        with open(o["restart"], "rb") as f:
            raw = f.read()
        assert np.frombuffer(raw[:4], np.int32)[0] == r["steps"]
        assert np.frombuffer(raw[4:12], np.float64)[0] == t
        s = Solver(Mesh(d), initial_state=False)
        s.upload(Q)
        s.iter, s.ctime = r["steps"], t
        ref = str(tmp_path / "alone.dat")
        s.write_restart(ref)
        s.close()
        with open(ref, "rb") as f:
            assert f.read() == raw
        assert r["latency_s"] > 0 and r["finish_s"] >= r["admit_s"]


def test_sequential_loop_returns_the_same_results(case_root):
    d = make_case(case_root, problem="alfven", nx=8, ny=8, N=3)
    m = Mesh(d)
    q = np.empty(9 * m.N * m.N * m.ncell)
    m.close()
    res, _ = serve.serve([(d, 0.0, 0.04, {"Q": q})], mode="sequential")
    assert res[0]["status"] == 0
    Q, t = _alone(d, res[0]["steps"])
    assert np.array_equal(q, Q) and res[0]["ctime"] == t


def test_wrong_output_size_fails_that_request_only(case_root):
    d = make_case(case_root, problem="alfven", nx=8, ny=8, N=3)
    bad = np.empty(10)
    res, _ = serve.serve([(d, 0.0, 0.01, {"Q": bad}), (d, 0.0, 0.01)], mode="batched")
    assert res[0]["status"] == 1  # CHORUS_EINVAL
    assert res[1]["status"] == 0


def test_budget_admission_serialises_when_memory_is_short(case_root):
    d = make_case(case_root, problem="orszag_tang", nx=12, ny=12, N=4, jitter=0.1, seed=3)
    one = Mesh(d)
    import ctypes
    from chorus_mhd import _lib
    need = _lib.load().chorus_mesh_device_bytes(one._h)
    reqs = [(d, 0.0, 0.02), (d, 0.0, 0.02), (d, 0.0, 0.02)]
    res, _ = serve.serve(reqs, mode="batched", hbm_budget_bytes=int(need * 1.5))
    assert all(r["status"] == 0 for r in res)
    # only one fits at a time: admissions happen after the previous finishes
    order = sorted(res, key=lambda r: r["admit_s"])
    for a, b in zip(order, order[1:]):
        assert b["admit_s"] >= a["finish_s"] - 1e-3
    # the later two waited for memory, and say so
    assert order[0]["wait_s"] == 0.0
    assert all(r["wait_s"] > 0 for r in order[1:])
    res2, _ = serve.serve([(d, 0.0, 0.02)], mode="batched", hbm_budget_bytes=int(need * 0.5))
    assert res2[0]["status"] == 6  # CHORUS_ENOMEM: can never fit


def test_served_state_matches_alone(case_root):
    """Bitwise check through the batch API used by the loop: two solves joining at
    different steps end like their alone runs."""
    from chorus_mhd import Batch
    d1 = make_case(case_root, problem="orszag_tang", nx=9, ny=9, N=4, jitter=0.1, seed=4)
    d2 = make_case(case_root, problem="rotor", nx=64, ny=64, N=3, jitter=0.1, seed=5)
    b = Batch()
    s1, s2 = Solver(Mesh(d1)), Solver(Mesh(d2))
    b.add(s1)
    b.step(2)
    slot2 = b.add(s2)
    b.step(3)
    b.remove(slot2)
    b.step(1)
    b.sync()
    a1, a2 = Solver(Mesh(d1)), Solver(Mesh(d2))
    a1.set_option("diagnostics", 0)
    a2.set_option("diagnostics", 0)
    a1.iterations(6)
    a2.iterations(3)
    assert np.array_equal(s1.state(), a1.state())
    assert np.array_equal(s2.state(), a2.state())


def test_sequential_mode_runs_fifo(case_root):
    d = make_case(case_root, problem="orszag_tang", nx=8, ny=8, N=3)
    reqs = [(d, 0.0, 0.02), (d, 0.0, 0.03)]
    res, mk = serve.serve(reqs, mode="sequential")
    assert all(r["status"] == 0 for r in res)
    assert res[1]["admit_s"] >= res[0]["finish_s"] - 1e-6


def test_device_setup_serves_the_same_results(case_root):
    """Requests set up on the device (gpu_setup) end in the same states as with the host
    setup: the maps and geometry are the same bit for bit."""
    specs = [dict(problem="orszag_tang", nx=10, ny=10, N=4, jitter=0.1, seed=1),
             dict(problem="rotor", nx=64, ny=64, N=3, jitter=0.1, seed=5)]
    dirs = [make_case(case_root, **sp) for sp in specs]
    out = {}
    for gpu_setup in (False, True):
        qs = []
        reqs = []
        for k, d in enumerate(dirs):
            m = Mesh(d)
            q = np.empty(9 * m.N * m.N * m.ncell)
            m.close()
            qs.append(q)
            # the rotor at this coarse grid goes non-finite after a few tens of steps (the
            # reference's scheme does): about ten steps of it
            reqs.append((d, 0.001 * k, 0.01 if k == 0 else 0.0015, {"Q": q}))
        res, _ = serve.serve(reqs, mode="batched", gpu_setup=gpu_setup)
        assert all(r["status"] == 0 for r in res)
        out[gpu_setup] = qs
    for a, b in zip(out[False], out[True]):
        assert np.array_equal(a, b)
