"""Failure detection without faulting the GPU: a non-physical state injected on the host is
reported by the kernels' error flag as CHORUS_ESTATE, and the context stays usable; the
serving loop reports a request whose case cannot be read and carries on with the others."""
import numpy as np
import pytest

from chorus_mhd import ChorusError, Mesh, Solver, serve
from helpers import make_case

pytestmark = pytest.mark.gpu
CHORUS_EIO, CHORUS_ESTATE = 4, 5


@pytest.mark.parametrize("how", ["nan_density", "nan_energy", "inf_momentum"])
def test_non_finite_state_is_reported_and_the_context_recovers(case_root, how):
    d = make_case(case_root, problem="orszag_tang", nx=8, ny=6, N=4, jitter=0.1, seed=5)
    s = Solver(Mesh(d))
    good = s.state()
    bad = good.copy()
    k = {"nan_density": 0, "nan_energy": 4, "inf_momentum": 1}[how]
    bad[9 * 37 + k] = np.nan if how.startswith("nan") else np.inf
    s.upload(bad)
    with pytest.raises(ChorusError) as e:
        s.iterations(2)
    assert e.value.code == CHORUS_ESTATE
    # a new state clears the flag; the context then steps like a fresh one
    s.upload(good)
    it0 = s.iter
    s.iterations(3)
    fresh = Solver(Mesh(d))
    fresh.iterations(3)
    assert np.array_equal(s.state(), fresh.state())
    assert s.iter == it0 + 3
    # the host-state entry reports the same way
    out = np.empty_like(good)
    with pytest.raises(ChorusError) as e:
        s.step_host(bad, out, 1)
    assert e.value.code == CHORUS_ESTATE
    s.close()
    fresh.close()


def test_serving_reports_unreadable_requests_and_serves_the_rest(case_root, tmp_path):
    d = make_case(case_root, problem="orszag_tang", nx=8, ny=8, N=3, jitter=0.1, seed=6)
    missing = str(tmp_path / "no_such_case")
    reqs = [(d, 0.0, 0.02), (missing, 0.0, 0.02), (d, 0.001, 0.02)]
    for mode in ("batched", "sequential"):
        res, _ = serve.serve(reqs, mode=mode)
        assert [r["status"] for r in res] == [0, CHORUS_EIO, 0], mode


def test_serving_a_failing_solve_does_not_fail_the_next_one_in_its_slot(case_root):
    """A request whose solve goes non-finite (an unstable time step) is reported as
    CHORUS_ESTATE; the request admitted into the batch slot it leaves completes."""
    bad = make_case(case_root, problem="orszag_tang", nx=8, ny=8, N=3, dt=0.5)  # far above the CFL limit
    good = make_case(case_root, problem="orszag_tang", nx=8, ny=8, N=3, jitter=0.1, seed=6)
    reqs = [(bad, 0.0, 100.0), (good, 0.0, 0.05), (good, 0.0, 0.03)]
    res, _ = serve.serve(reqs, mode="batched", max_active=1)  # one solve at a time: the slot is reused
    assert [r["status"] for r in res] == [CHORUS_ESTATE, 0, 0]
    alone, _ = serve.serve(reqs[1:], mode="sequential")
    assert [r["status"] for r in alone] == [0, 0]
