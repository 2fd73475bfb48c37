"""Batched form: every solve of a mixed batch (different N, mesh size, problem, dt,
RK scheme) must give the same state as the same solve stepped alone."""
import numpy as np
import pytest

from chorus_mhd import Batch, Mesh, Solver
from helpers import make_case

pytestmark = pytest.mark.gpu

MIX = [
    dict(problem="orszag_tang", nx=12, ny=10, N=4, jitter=0.1, seed=1),
    dict(problem="orszag_tang", nx=7, ny=9, N=3, jitter=0.15, seed=2),
    dict(problem="alfven", nx=8, ny=8, N=5),
    dict(problem="rotor", nx=64, ny=64, N=3, jitter=0.1, seed=3),
    dict(problem="orszag_tang", nx=6, ny=6, N=6, jitter=0.1, seed=4, k_stage=5),
    dict(problem="orszag_tang", nx=5, ny=6, N=2),
    dict(problem="orszag_tang", nx=4, ny=4, N=8, jitter=0.05, seed=5),
    dict(problem="orszag_tang", nx=6, ny=5, N=4, jitter=0.1, seed=6, mu=0.01, eta0=0.02),
    dict(problem="orszag_tang", nx=1, ny=1, N=4),
    dict(problem="alfven", nx=2, ny=1, N=3),
]


def _alone(case_root, spec, nsteps):
    s = Solver(Mesh(make_case(case_root, **spec)))
    s.set_option("diagnostics", 0)
    s.iterations(nsteps)
    return s.state()


def test_batch_equals_alone(case_root):
    nsteps = 7
    b = Batch()
    solvers = []
    for spec in MIX:
        s = Solver(Mesh(make_case(case_root, **spec)))
        b.add(s)
        solvers.append(s)
    assert b.info()["solves"] == len(MIX)
    b.step(nsteps)
    b.sync()
    for spec, s in zip(MIX, solvers):
        ref = _alone(case_root, spec, nsteps)
        got = s.state()
        assert np.all(np.isfinite(got))
        err = np.abs(got - ref).max() / np.abs(ref).max()
        assert err <= 1e-14, "%s: batch vs alone %.3e" % (spec, err)


def test_batch_membership_changes_between_steps(case_root):
    """Solves join and leave between steps (the serving loop's use); a solve that
    joins late or sits next to different neighbours still matches running alone."""
    b = Batch()
    s0 = Solver(Mesh(make_case(case_root, **MIX[0])))
    s1 = Solver(Mesh(make_case(case_root, **MIX[2])))
    slot0 = b.add(s0)
    b.step(3)
    b.add(s1)
    b.step(2)
    b.remove(slot0)
    b.step(4)
    b.sync()
    assert np.abs(s0.state() - _alone(case_root, MIX[0], 5)).max() <= 1e-14 * 50
    ref1 = _alone(case_root, MIX[2], 6)
    assert np.abs(s1.state() - ref1).max() <= 1e-14 * np.abs(ref1).max()
