"""Committed golden fixtures (tests/golden/*.npz, made by tests/golden/make_golden.py
from the oracle): the oracle must keep reproducing them (CPU), the product setup must
reproduce their map digests (CPU), and the CUDA path must match them (GPU)."""
import hashlib
import json
import os

import numpy as np
import pytest

import oracle
from chorus_mhd import Mesh, Solver, meshgen

HERE = os.path.dirname(os.path.abspath(__file__))


def _short_cases():
    """The fixtures make_golden.py writes (the long-horizon ones have their own tests)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(HERE, "golden", "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return list(mod.CASES)


FIXTURES = sorted(os.path.join(HERE, "golden", n + ".npz") for n in _short_cases())
MAPS = ["IF2C", "IC2F", "IF2V", "IBFINTER", "IBFREE", "CYC2FPAIR"]


def _load(path):
    z = np.load(path)
    return {k: z[k] for k in z.files}


def _case(path, root):
    g = _load(path)
    spec = json.loads(str(g["spec"]))
    d = meshgen.write_case(meshgen.CaseSpec(**spec), os.path.join(root, os.path.basename(path)[:-4]))
    return g, d


def _check_state(Q, g, prefix, rtol):
    q = np.asarray(Q).reshape(-1, 9)
    assert np.all(np.isfinite(q))
    norms = np.sqrt((q * q).sum(axis=0))
    assert np.allclose(norms, g[prefix + "norms"], rtol=rtol, atol=rtol), prefix + " per-variable norms"
    if prefix + "full" in g:
        ref = g[prefix + "full"]
        err = np.linalg.norm(Q - ref) / np.linalg.norm(ref)
        assert err <= rtol, "%s full state rel L2 %.3e" % (prefix, err)
    else:
        idx = g[prefix + "sample_idx"]
        ref = g[prefix + "sample"]
        err = np.linalg.norm(np.asarray(Q)[idx] - ref) / np.linalg.norm(ref)
        assert err <= rtol, "%s sampled state rel L2 %.3e" % (prefix, err)


def test_fixtures_present():
    assert len(FIXTURES) >= 7 and all(os.path.exists(p) for p in FIXTURES)


@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: os.path.basename(p)[:-4])
def test_oracle_reproduces_golden(path, case_root):
    g, d = _case(path, case_root)
    o = oracle.Oracle(d)
    maps = json.loads(str(g["maps"]))
    for m in MAPS:
        assert hashlib.sha256(np.ascontiguousarray(o.array(m)).tobytes()).hexdigest() == maps[m], m
    _check_state(o.array("Q"), g, "q0_", 1e-13)
    diags = []
    for _ in range(int(g["steps"])):
        r = o.step()
        if r is not None:
            diags.append((o.geti("iter"),) + r)
    _check_state(o.array("Q"), g, "q1_", 1e-12)
    assert np.allclose(np.array(diags), g["diag"], rtol=1e-10, atol=1e-14)


@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: os.path.basename(p)[:-4])
def test_product_setup_reproduces_golden_maps(path, case_root):
    g, d = _case(path, case_root)
    m = Mesh(d)
    maps = json.loads(str(g["maps"]))
    for name in MAPS:
        assert hashlib.sha256(np.ascontiguousarray(m.iarray(name)).tobytes()).hexdigest() == maps[name], name
    assert m.params.dt == float(g["dt"])


@pytest.mark.gpu
@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: os.path.basename(p)[:-4])
def test_gpu_matches_golden(path, case_root):
    g, d = _case(path, case_root)
    s = Solver(Mesh(d))
    _check_state(s.state(), g, "q0_", 1e-12)
    diags = s.iterations(int(g["steps"]))
    _check_state(s.state(), g, "q1_", 1e-10)
    ref = g["diag"]
    assert len(diags) == len(ref)
    for a, r in zip(diags, ref):
        assert a["iter"] == int(r[0])
        assert abs(a["residglob"] - r[1]) <= 1e-9 * r[1]
        assert abs(a["divBglob"] - r[2]) <= 1e-9 * r[2] + 1e-13
    assert s.ctime == pytest.approx(float(g["ctime"]), rel=1e-14)
