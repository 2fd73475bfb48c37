"""The single-solve workloads over their stated run lengths, against the oracle.

Orszag-Tang 64x64 N=4 for 1000 steps, the MHD rotor 256x256 N=4 (jittered, FREE
boundaries, gamma = 1.4) for 500 steps and Orszag-Tang 512x512 N=5 (jittered) for 200
steps, each through iterations_gpu from its initial data (the loop of
iterations.f90:19-87), compared at every checkpoint of the oracle's run of the same
case (tests/golden/make_long_golden.py holds the oracle's figures: per-variable norms
and sums, a count sketch of the whole state, the diagnostics every tenth step and a
strided sample of the last state).

Bar: relative L2 of Q within 1e-10 at every checkpoint (estimated from the sketch of
the difference, which covers every element; the estimate's relative spread is 1.6%),
per-variable norms and sums within 1e-10 of the state's norm, the sample within 1e-10,
residglob within 1e-9 and divBglob within 1e-9 relative plus the absolute round-off
of a derivative norm (eps times cells per side times N^2).

Where the case itself amplifies round-off past 1e-10 the bar is the reference's own
spread instead: tests/golden/<case>_sensitivity.npz holds the distance between the
committed oracle and the same oracle built with FMA contraction (the arithmetic of an
aarch64 build of the reference), and from the checkpoint where that distance passes
1e-10 the GPU must stay at least as close to the oracle as that second build does.  On
the rotor this happens from step 150 on (the two oracle builds are 1.7e-10 apart there
and grow by about 3x per 50 steps); the strict 1e-10 bar at its last step is kept as an
expected failure that reports if it ever passes."""
import importlib.util
import os

import numpy as np
import pytest

from chorus_mhd import Mesh, Solver, meshgen

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
_spec = importlib.util.spec_from_file_location("long_golden", os.path.join(HERE, "golden", "make_long_golden.py"))
LG = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(LG)

RUN_TOL = 1e-10


_RUNS: dict = {}


def sensitivity(name):
    """Per checkpoint, the distance between the two oracle builds (None if not recorded)."""
    p = os.path.join(HERE, "golden", name + "_sensitivity.npz")
    if not os.path.exists(p):
        return None
    with np.load(p) as z:
        return dict(zip(z["contracted"][:, 0].astype(int), z["contracted"][:, 1])) if "contracted" in z.files else None


def run_case(name, tmp_path):
    """GPU run of the case over its stated steps, compared at every checkpoint (cached)."""
    if name in _RUNS:
        return _RUNS[name]
    fx = LG.load(name)
    spec = fx["spec"]
    d = meshgen.write_case(meshgen.CaseSpec(**spec), str(tmp_path / name))
    mesh = Mesh(d)
    s = Solver(mesh)
    assert abs(mesh.params.dt - float(fx["dt"])) == 0.0, "the case's dt differs from the fixture's"
    Q = np.empty(s.nq)
    curve, diag = [], []
    for k, it in enumerate(fx["checkpoints"]):
        if it > s.iter:
            diag += s.iterations(int(it) - s.iter)
        s.state(out=Q)
        assert np.all(np.isfinite(Q)), "non-finite state at step %d" % it
        norms, sums = fx["norms"][k], fx["sums"][k]
        total = float(np.sqrt((norms ** 2).sum()))
        err = LG.sketch_rel_l2(LG.sketch(Q), fx["sketch"][k], norms)
        q = Q.reshape(-1, 9)
        dn = np.abs(np.sqrt((q * q).sum(0)) - norms).max() / total
        ds = np.abs(q.sum(0) - sums).max() / total
        curve.append((int(it), err, dn, ds))
        assert s.ctime == pytest.approx(float(fx["ctime"][k]), rel=1e-14, abs=0)
    idx = fx["sample_idx"]
    e_samp = float(np.linalg.norm(Q[idx] - fx["sample"]) / np.linalg.norm(fx["sample"]))
    s.close()
    mesh.close()
    _RUNS[name] = (fx, curve, diag, e_samp)
    return _RUNS[name]


@pytest.mark.parametrize("name", list(LG.LONG_CASES))
def test_long_run_matches_oracle_at_every_checkpoint(tmp_path, name):
    fx, curve, diag, e_samp = run_case(name, tmp_path)
    spec = fx["spec"]
    sens = sensitivity(name) or {}
    print("\n%s: step, est. rel L2 of Q vs oracle, max norm diff, max sum diff, two oracle builds apart" % name)
    for row in curve:
        print("  %5d  %.3e  %.3e  %.3e  %s" % (row + (("%.3e" % sens[row[0]]) if row[0] in sens else "-",)))
    print("  sample rel L2 at step %d: %.3e" % (int(fx["checkpoints"][-1]), e_samp))
    # diagnostics of every tenth step (iter, ctime, residglob, divBglob, eigvmax_g, epsilon0)
    div_atol = 1e-15 * spec["nx"] * spec["N"] ** 2
    dref = fx["diag"]
    assert len(diag) == len(dref)
    worst = 0.0
    for a, row in zip(diag, dref):
        assert a["iter"] == int(row[0])
        bar = max(1.0, min((sens.get(c, 0.0) for c in sens if c >= a["iter"]), default=0.0) / RUN_TOL)
        worst = max(worst, abs(a["residglob"] - row[2]) / row[2])
        assert abs(a["residglob"] - row[2]) <= 1e-9 * bar * row[2], "residglob at iter %d" % a["iter"]
        assert abs(a["divBglob"] - row[3]) <= 1e-9 * bar * row[3] + div_atol, "divBglob at iter %d" % a["iter"]
        assert abs(a["eigvmax_g"] - row[4]) <= 1e-10 * bar * row[4], "eigvmax at iter %d" % a["iter"]
    print("  worst residglob relative difference over %d records: %.3e" % (len(diag), worst))
    for it, err, dn, ds in curve:
        bar = max(RUN_TOL, sens.get(it, 0.0))
        assert err <= bar, "%s: relative L2 %.3e at step %d (bar %.1e)" % (name, err, it, bar)
        assert dn <= bar and ds <= bar, "%s: norms/sums at step %d" % (name, it)
    assert e_samp <= max(RUN_TOL, sens.get(int(fx["checkpoints"][-1]), 0.0))


@pytest.mark.xfail(strict=True, reason="the rotor amplifies round-off about 3x per 50 steps: two builds of the "
                                       "oracle that differ only in FMA contraction are 1e-8 apart at step 500")
def test_rotor_within_1e10_at_its_last_step(tmp_path):
    name = "rotor_256x256_N4_500steps"
    fx, curve, diag, e_samp = run_case(name, tmp_path)
    assert curve[-1][1] <= RUN_TOL
