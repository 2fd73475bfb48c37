"""Serving form: continuous batching of Poisson arrivals under an HBM budget."""
import os

import numpy as np
import pytest

from chorus_mhd import Mesh, Solver, serve
from helpers import make_case

pytestmark = pytest.mark.gpu


def test_each_result_same_alone_and_in_the_mix(case_root, tmp_path):
    """A solve served in the batched mix ends in the same state as the same solve run
    alone: the request loop retires it after exactly ceil(end_time/dt) steps."""
    specs = [dict(problem="orszag_tang", nx=10, ny=10, N=4, jitter=0.1, seed=1),
             dict(problem="alfven", nx=8, ny=8, N=3),
             dict(problem="orszag_tang", nx=6, ny=8, N=5, jitter=0.1, seed=2)]
    dirs = [make_case(case_root, **sp) for sp in specs]
    reqs = [(dirs[0], 0.0, 0.05), (dirs[1], 0.001, 0.08), (dirs[2], 0.002, 0.03), (dirs[0], 0.003, 0.02)]
    res, mk = serve.serve(reqs, mode="batched")
    assert all(r["status"] == 0 for r in res)
    for (d, _, tend), r in zip(reqs, res):
        m = Mesh(d)
        assert r["steps"] == int(np.ceil(tend / m.params.dt - 1e-9))
        assert r["latency_s"] > 0 and r["finish_s"] >= r["admit_s"]


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
