"""The long-horizon fixtures (CPU): the oracle reproduces the first checkpoint of the
64x64 Orszag-Tang run bit for bit, and the count sketch the fixtures store measures the
relative L2 of a difference of two states."""
import importlib.util
import os

import numpy as np

import oracle
from chorus_mhd import meshgen

HERE = os.path.dirname(os.path.abspath(__file__))
_spec = importlib.util.spec_from_file_location("long_golden", os.path.join(HERE, "golden", "make_long_golden.py"))
LG = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(LG)


def test_every_long_fixture_is_present_and_consistent():
    for name, (spec, steps, every) in LG.LONG_CASES.items():
        fx = LG.load(name)
        assert fx["spec"] == spec and int(fx["steps"]) == steps
        assert list(fx["checkpoints"]) == list(range(0, steps + 1, every))
        assert fx["sketch"].shape == (len(fx["checkpoints"]), LG.SKETCH_K)
        assert len(fx["diag"]) == sum(1 for i in range(1, steps + 1) if i % 10 == 1)
        assert np.all(np.isfinite(fx["norms"])) and np.all(np.isfinite(fx["sketch"]))
        # the sketch's squared norm estimates the state's (unbiased; spread sqrt(2/K))
        est = np.linalg.norm(fx["sketch"], axis=1)
        true = np.sqrt((fx["norms"] ** 2).sum(axis=1))
        assert np.all(np.abs(est / true - 1) < 0.15)


def test_rotor_sensitivity_curves_are_recorded():
    """The rotor's round-off spread that its long-run GPU test is held to: the oracle built
    with FMA contraction and the oracle from a one-ulp perturbed start, each against the
    fixture at every checkpoint, growing with the steps."""
    name = "rotor_256x256_N4_500steps"
    with np.load(os.path.join(HERE, "golden", name + "_sensitivity.npz")) as z:
        cps = list(LG.load(name)["checkpoints"])
        for key in ("contracted", "ulp1"):
            c = z[key]
            assert list(c[:, 0].astype(int)) == cps
            assert np.all(np.isfinite(c[:, 1])) and c[-1, 1] > 100 * c[1, 1]
        # a build of the same restatement that differs only in contraction ends further from
        # the fixture than the 1e-10 bar
        assert z["contracted"][-1, 1] > 1e-10


def test_oracle_reproduces_first_checkpoint_of_orszag_tang_64():
    name = "ot_64x64_N4_1000steps"
    fx = LG.load(name)
    import tempfile
    d = meshgen.write_case(meshgen.CaseSpec(**fx["spec"]), tempfile.mkdtemp(prefix="lg_"))
    o = oracle.Oracle(d, threads=os.cpu_count() or 1)
    assert o.getd("dt") == float(fx["dt"])
    it = int(fx["checkpoints"][1])
    for _ in range(it):
        o.step()
    Q = o.array("Q")
    s = LG.summary(Q)
    assert np.array_equal(s["sketch"], fx["sketch"][1])
    assert np.array_equal(s["norms"], fx["norms"][1])
    assert o.getd("ctime") == float(fx["ctime"][1])
    o.close()


def test_sketch_estimates_relative_l2_of_a_difference():
    rng = np.random.default_rng(1)
    a = rng.standard_normal(300_000)
    na = np.sqrt((a.reshape(-1, 9 if a.size % 9 == 0 else 1) ** 2).sum(0))
    for scale, spread in ((1e-11, "dense"), (1e-7, "sparse")):
        e = np.zeros_like(a)
        if spread == "dense":
            e[:] = scale * rng.standard_normal(a.size)
        else:
            e[rng.integers(0, a.size, 50)] = scale
        est = LG.sketch_rel_l2(LG.sketch(a + e), LG.sketch(a), na)
        true = np.linalg.norm(e) / np.linalg.norm(a)
        assert abs(est / true - 1) < 0.2, (spread, est, true)
    # linear: the sketch of a sum is the sum of the sketches (to rounding)
    b = rng.standard_normal(a.size)
    assert np.allclose(LG.sketch(a + b), LG.sketch(a) + LG.sketch(b), rtol=0, atol=1e-9)
