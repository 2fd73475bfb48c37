"""The setup chain on the device (chorus_mesh_load_gpu) against the host path and the
oracle: every integer map and every geometry array bit for bit, and the same errors for
broken meshes (a mesh the kernels find invalid is rebuilt on the host, which names the
reference's error)."""
import time

import numpy as np
import pytest

import oracle
from chorus_mhd import ChorusError, Mesh, meshgen
from helpers import make_case

pytestmark = pytest.mark.gpu

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
    dict(problem="rotor", nx=160, ny=150, N=4, jitter=0.1, seed=5),
    dict(problem="orszag_tang", nx=1, ny=1, N=4),
    dict(problem="alfven", nx=2, ny=1, N=3),
    dict(problem="rotor", nx=1, ny=1, N=2),
]


def _same(a: Mesh, b: Mesh):
    for nm in IMAPS:
        x, y = a.iarray(nm), b.iarray(nm)
        assert x.shape == y.shape and np.array_equal(x, y), nm
    for nm in DMAPS:
        x, y = a.darray(nm), b.darray(nm)
        assert x.shape == y.shape and np.array_equal(x, y), nm
    for f in ("N", "NCELL", "NFACE", "NINTER", "NFREE", "NPAIR"):
        assert getattr(a.dims, f) == getattr(b.dims, f), f


@pytest.mark.parametrize("spec", MESHES, ids=lambda s: "%s-%dx%d-N%d" % (s["problem"], s["nx"], s["ny"], s["N"]))
def test_device_setup_equals_host_setup(case_root, spec):
    d = make_case(case_root, **spec)
    host, dev = Mesh(d), Mesh(d, device=0)
    _same(host, dev)
    if spec["nx"] * spec["ny"] <= 4096:
        o = oracle.Oracle(d)
        for nm in IMAPS:
            assert np.array_equal(o.array(nm), dev.iarray(nm)), nm
        for nm in ("S1", "S2", "Jac", "XXsolu"):
            assert np.array_equal(o.array(nm), dev.darray(nm)), nm
        o.close()
    host.close()
    dev.close()


def test_device_setup_at_full_size_is_bit_identical_and_faster(case_root):
    d = make_case(case_root, problem="orszag_tang", nx=512, ny=512, N=5, jitter=0.15, seed=1)
    Mesh(d, device=0).close()  # first use: module load, allocator
    t0 = time.perf_counter()
    dev = Mesh(d, device=0)
    t1 = time.perf_counter()
    host = Mesh(d)
    t2 = time.perf_counter()
    _same(host, dev)
    print("\n512x512 N=5 setup: device %.3f s, host %.3f s" % (t1 - t0, t2 - t1))
    assert t1 - t0 < t2 - t1


def _corrupt(d, fname, fn):
    p = d + "/" + fname
    lines = open(p).read().splitlines()
    open(p, "w").write("\n".join(fn(lines)) + "\n")


def _errors(d):
    out = []
    for dev in (None, 0):
        with pytest.raises(ChorusError) as e:
            Mesh(d, device=dev)
        out.append((e.value.code, str(e.value)))
    return out


def test_device_setup_reports_the_host_errors(tmp_path):
    # a clockwise cell
    d = meshgen.write_case(meshgen.CaseSpec(nx=4, ny=3, N=3), str(tmp_path / "cw"))

    def flip_one(lines):
        f = lines[5].split()
        lines[5] = " ".join([f[0], f[4], f[3], f[2], f[1], f[5], f[6]])
        return lines

    _corrupt(d, "mesh.CEL", flip_one)
    (hc, hm), (dc, dm) = _errors(d)
    assert hc == dc == 3 and hm == dm
    # a boundary record missing
    d = meshgen.write_case(meshgen.CaseSpec(nx=3, ny=3, N=3), str(tmp_path / "nb"))
    _corrupt(d, "mesh.BND", lambda L: L[:4] + L[5:])
    (hc, hm), (dc, dm) = _errors(d)
    assert hc == dc == 3 and hm == dm and "missing" in hm
    # a boundary type with no flux routine
    d = meshgen.write_case(meshgen.CaseSpec(nx=3, ny=3, N=3, problem="rotor"), str(tmp_path / "wall"))
    _corrupt(d, "mesh.BND", lambda L: L[:2] + [L[2].replace("FREE", "WALL")] + L[3:])
    (hc, hm), (dc, dm) = _errors(d)
    assert hc == dc == 3 and hm == dm and "WALL" in hm
    # a boundary record naming an interior edge
    d = meshgen.write_case(meshgen.CaseSpec(nx=3, ny=3, N=3, problem="rotor"), str(tmp_path / "inner"))
    cel = open(d + "/mesh.CEL").read().split("\n")[0].split()  # cell 1: vertices 1 2 6 5 (4x4 vertex grid)

    def inner(lines):
        f = lines[0].split()
        f[1], f[2] = cel[2], cel[3]  # the edge 2-6, shared by cells 1 and 2
        lines[0] = " ".join(f)
        return lines

    _corrupt(d, "mesh.BND", inner)
    (hc, hm), (dc, dm) = _errors(d)
    assert hc == dc == 3 and hm == dm and "interior" in hm
