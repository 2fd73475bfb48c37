"""The product's host setup (libchorus_gpu.so, C++) against the oracle's restatement
of the reference setup chain: integer maps bit-exact, geometry bit-exact (both follow
the reference's evaluation order with FP contraction off).  CPU only: no kernels run."""
import numpy as np
import pytest

import oracle
from chorus_mhd import ChorusError, Mesh, meshgen
from helpers import make_case

IMAPS = ["IF2C", "IC2F", "IF2V", "IVCELL", "IBFINTER", "IBFREE", "IBFCYC", "IBFCYCLOC", "CYC2FPAIR",
         "iface2fp", "jface2fp"]
DMAPS = ["XV", "YV", "Xs", "Xf", "Lmat", "Mmat", "S1", "S2", "Jac", "XXsolu"]

MESHES = [
    dict(problem="orszag_tang", nx=8, ny=8, N=4, jitter=0.15, seed=1),
    dict(problem="orszag_tang", nx=2, ny=2, N=2),
    dict(problem="orszag_tang", nx=7, ny=3, N=6, jitter=0.1, seed=2),
    dict(problem="rotor", nx=12, ny=9, N=3, jitter=0.1, seed=3),
    dict(problem="alfven", nx=6, ny=5, N=5),
    dict(problem="orszag_tang", nx=33, ny=31, N=8, jitter=0.15, seed=4),
]


@pytest.mark.parametrize("spec", MESHES, ids=lambda s: "%s-%dx%d-N%d" % (s["problem"], s["nx"], s["ny"], s["N"]))
def test_maps_and_geometry_bit_exact(case_root, spec):
    d = make_case(case_root, **spec)
    o = oracle.Oracle(d)
    m = Mesh(d)
    for nm in IMAPS:
        a, b = o.array(nm), m.iarray(nm)
        assert a.shape == b.shape and np.array_equal(a, b), nm
    for nm in DMAPS:
        a, b = o.array(nm), m.darray(nm)
        assert a.shape == b.shape and np.array_equal(a, b), nm
    assert m.params.dt == o.getd("dt")
    assert m.params.gam == o.getd("gam")
    assert m.dims.NINTER == o.geti("NINTER") and m.dims.NPAIR == o.geti("NPAIR")


def _corrupt(d, fname, fn):
    p = d + "/" + fname
    lines = open(p).read().splitlines()
    open(p, "w").write("\n".join(fn(lines)) + "\n")


def test_rejects_clockwise_cells(tmp_path):
    d = meshgen.write_case(meshgen.CaseSpec(nx=3, ny=3, N=3), str(tmp_path / "cw"))

    def flip(lines):
        out = []
        for ln in lines:
            f = ln.split()
            out.append(" ".join([f[0], f[4], f[3], f[2], f[1], f[5], f[6]]))
        return out

    _corrupt(d, "mesh.CEL", flip)
    with pytest.raises(ChorusError) as e:
        Mesh(d)
    assert e.value.code == 3


def test_rejects_missing_boundary_face(tmp_path):
    d = meshgen.write_case(meshgen.CaseSpec(nx=3, ny=3, N=3), str(tmp_path / "nb"))
    _corrupt(d, "mesh.BND", lambda L: L[:-1])
    with pytest.raises(ChorusError) as e:
        Mesh(d)
    assert "missing" in str(e.value) or "partner" in str(e.value)


def test_rejects_unsupported_boundary_type(tmp_path):
    d = meshgen.write_case(meshgen.CaseSpec(nx=3, ny=3, N=3, problem="rotor"), str(tmp_path / "wall"))
    _corrupt(d, "mesh.BND", lambda L: [ln.replace("FREE", "WALL") for ln in L])
    with pytest.raises(ChorusError) as e:
        Mesh(d)
    assert "WALL" in str(e.value)


def test_rejects_bad_order(tmp_path):
    d = meshgen.write_case(meshgen.CaseSpec(nx=3, ny=3, N=3), str(tmp_path / "bad_n"))
    _corrupt(d, "QUAD.INP", lambda L: L[:9] + ["12"] + L[10:])
    with pytest.raises(ChorusError) as e:
        Mesh(d)
    assert e.value.code == 1


def test_rejects_missing_files(tmp_path):
    with pytest.raises(ChorusError) as e:
        Mesh(str(tmp_path / "nothing"))
    assert e.value.code == 4
