"""Plot output on the device (chorus_plot_*) against the oracle's restatement of
tecplotter2dsetup / tecplotter2d / tecpost_parallel, on identical states."""
import os

import numpy as np
import pytest

import oracle
from chorus_mhd import Mesh, Solver, plot_filename
from helpers import make_case
from test_oracle_plot import read_tecplot

pytestmark = pytest.mark.gpu

CASES = [
    dict(problem="orszag_tang", nx=6, ny=5, N=4, jitter=0.1, seed=3, nre=3),
    dict(problem="rotor", nx=64, ny=64, N=3, jitter=0.1, seed=6, nre=2),
    dict(problem="orszag_tang", nx=4, ny=4, N=5, jitter=0.15, seed=2, nre=1),
    dict(problem="orszag_tang", nx=5, ny=5, N=4, jitter=0.0, artiv=0, nre=2),
]


def ids(c):
    return "%s_%dx%d_N%d_nre%d%s" % (c["problem"], c["nx"], c["ny"], c["N"], c["nre"],
                                     "_noav" if c.get("artiv", 1) == 0 else "")


def same_state(case_root, case, steps=3):
    d = make_case(case_root, **case)
    o = oracle.Oracle(d)
    o.run(steps)
    s = Solver(Mesh(d), initial_state=False)
    s.upload(o.array("Q").copy())
    o.compresid()
    s.set_option("plot_sensor", 1)
    s.compresid()  # records muAV(1) and muAV(6) of this state, like the oracle's
    return d, o, s


@pytest.mark.parametrize("case", CASES, ids=ids)
def test_plot_values_match_oracle(case_root, case):
    d, o, s = same_state(case_root, case)
    nre = case["nre"]
    assert o.plot_setup(nre) == 0
    o.plot_eval()
    p = s.plot()
    assert (p.nodes, p.cells, p.warned) == (o.geti("plotnodes"), o.geti("plotcells"), False)
    v = p.values()
    # topology and coordinates: host integer maps and the same FP64 expressions
    assert np.array_equal(v["plotX"], o.array("plotX"))
    assert np.array_equal(v["connec_c2n"], o.array("connec_c2n"))
    assert np.array_equal(v["gnode_factor"], o.array("gnode_factor"))
    # node values: the reference's loop order, explicitly rounded operations
    assert np.array_equal(v["plotQ"], o.array("plotQ"))
    # muAV / etaAV go through the sensors (different summation order, log10, sin)
    a, b = v["plotAV"], o.array("plotAV")
    assert np.allclose(a, b, rtol=1e-11, atol=1e-14 * max(1.0, np.abs(b).max()))
    if case.get("artiv", 1) == 0:
        assert not a.any()
    p.close()
    s.close()


@pytest.mark.parametrize("case", CASES[:2], ids=ids)
def test_plot_file_matches_oracle(case_root, case, tmp_path):
    d, o, s = same_state(case_root, case)
    o.plot_setup(case["nre"])
    o.plot_eval()
    t = 0.4375
    ref = str(tmp_path / ("oracle_" + plot_filename(t)))
    o.plot_write(t, ref)
    p = s.plot()
    out_dir = str(tmp_path / "gpu")
    os.makedirs(out_dir)
    path = p.write(out_dir, t)
    assert os.path.basename(path) == plot_filename(t)
    a, b = read_tecplot(path), read_tecplot(ref)
    for k in a:
        if k in ("data", "minmax"):
            continue
        if k == "con":
            assert np.array_equal(a[k], b[k])
        else:
            assert a[k] == b[k], k
    # X .. Az identical; muAV, etaAV within a float ulp
    assert np.array_equal(a["data"][:11], b["data"][:11])
    assert np.allclose(a["data"][11:], b["data"][11:], rtol=2 ** -22, atol=1e-30)
    assert np.array_equal(a["minmax"][:11], b["minmax"][:11])
    assert np.allclose(a["minmax"][11:], b["minmax"][11:], rtol=1e-11, atol=1e-300)
    p.close()
    s.close()


def test_run_writes_on_the_reference_schedule(case_root, tmp_path):
    """iterations.f90:80-84: output after step iter when mod(iter, nwrite) == 1 or at
    MAXITER; plot file plus restart.<iter %08d>.dat."""
    d = make_case(case_root, problem="orszag_tang", nx=4, ny=4, N=3, jitter=0.0, nre=2)
    s = Solver(Mesh(d))
    out = str(tmp_path)
    s.run(maxiter=7, out_dir=out, nwrite=3)
    files = sorted(os.listdir(out))
    restarts = [f for f in files if f.startswith("restart.")]
    assert restarts == ["restart.%08d.dat" % i for i in (1, 4, 7)]
    plots = [f for f in files if f.endswith(".plt")]
    # names come from ctime with three decimals (several outputs may share one)
    assert 1 <= len(plots) <= 3 and plot_filename(s.ctime) in plots
    assert s.iter == 7
    s.close()


def test_plot_needs_the_sensor_of_the_last_stage(case_root):
    """etaAV comes from the variable-6 sensor of the latest residual evaluation: without the
    plot_sensor option on that evaluation the plot is refused rather than stale."""
    from chorus_mhd import ChorusError
    d = make_case(case_root, problem="orszag_tang", nx=6, ny=5, N=4, jitter=0.1, seed=3, nre=3)
    s = Solver(Mesh(d))
    s.iterations(2)
    p = s.plot()
    with pytest.raises(ChorusError):
        p.values()
    s.set_option("plot_sensor", 1)
    s.iterations(1)
    v = p.values()
    assert np.isfinite(v["plotQ"]).all()
    s.set_option("plot_sensor", 0)
    s.iterations(1)
    with pytest.raises(ChorusError):
        p.values()
    p.close()
    s.close()
