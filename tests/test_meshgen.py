"""Synthetic case writer: reference file formats and seeded reproducibility."""
import os

import numpy as np

from chorus_mhd import meshgen


def test_d20_12_format():
    assert meshgen.fortran_d20_12(1.0) == "  0.100000000000D+01"
    assert meshgen.fortran_d20_12(-0.0625) == " -0.625000000000D-01"
    assert meshgen.fortran_d20_12(6.283185307179586) == "  0.628318530718D+01"
    assert meshgen.fortran_d20_12(0.0) == "  0.000000000000D+00"
    for v in [1e-7, 123.456, -9.99999999999e5]:
        s = meshgen.fortran_d20_12(v)
        assert len(s) == 20
        assert abs(float(s.replace("D", "E")) - v) <= 1e-11 * abs(v)


def test_vertex_file_columns(tmp_path):
    d = meshgen.write_case(meshgen.CaseSpec(nx=3, ny=2, N=3, jitter=0.1, seed=5), str(tmp_path / "c"))
    lines = open(os.path.join(d, "mesh.VRT")).read().splitlines()
    assert len(lines) == 4 * 3
    for i, ln in enumerate(lines, 1):
        assert int(ln[:9]) == i and ln[9:15] == " " * 6
        float(ln[15:35].replace("D", "E"))
        float(ln[36:56].replace("D", "E"))
    cel = open(os.path.join(d, "mesh.CEL")).read().splitlines()
    assert len(cel) == 6 and len(cel[0].split()) == 7
    bnd = open(os.path.join(d, "mesh.BND")).read().splitlines()
    assert len(bnd) == 2 * (3 + 2) and all(ln.split()[-1] == "CYCL" for ln in bnd)
    q = meshgen.read_quad_inp(d)
    assert q["N"] == 3 and q["k_stage"] == 3 and q["vismode"] == 1 and q["artiv"] == 1


def test_seeded_jitter_is_reproducible_and_bounded():
    s = meshgen.CaseSpec(nx=16, ny=16, N=3, jitter=0.15, seed=7)
    X1, Y1, *_ = meshgen.mesh_vertices(s)
    X2, Y2, *_ = meshgen.mesh_vertices(s)
    assert np.array_equal(X1, X2) and np.array_equal(Y1, Y2)
    X0, Y0, *_ = meshgen.mesh_vertices(meshgen.CaseSpec(nx=16, ny=16, N=3))
    h = 2 * np.pi / 16
    assert np.abs(X1 - X0).max() <= 0.15 * h + 1e-12
    bx = (np.isclose(X0, 0) | np.isclose(X0, 2 * np.pi) | np.isclose(Y0, 0) | np.isclose(Y0, 2 * np.pi))
    assert np.array_equal(X1[bx], X0[bx]) and np.array_equal(Y1[bx], Y0[bx])


def test_cfl_dt_positive_and_scales_with_h():
    a = meshgen.CaseSpec(nx=16, ny=16, N=4)
    b = meshgen.CaseSpec(nx=32, ny=32, N=4)
    da = meshgen.cfl_dt(a, *meshgen.mesh_vertices(a)[:3])
    db = meshgen.cfl_dt(b, *meshgen.mesh_vertices(b)[:3])
    assert da > 0 and abs(da / db - 2.0) < 0.05
