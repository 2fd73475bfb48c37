"""Restart stream of the device-resident state (write_data.f90:5-83,
read_data_restart.f90:35-67) against the oracle's writer and reader: the file the
library writes is byte-identical to the oracle's for the same state, each side reads
the other's file back exactly, and a run resumed from a restart file equals the
uninterrupted run bit for bit."""
import os

import numpy as np
import pytest

import oracle
from chorus_mhd import Mesh, Solver
from helpers import make_case

pytestmark = pytest.mark.gpu

CASES = [dict(problem="orszag_tang", nx=10, ny=9, N=4, jitter=0.1, seed=7),
         dict(problem="rotor", nx=64, ny=64, N=3, jitter=0.1, seed=8),
         dict(problem="orszag_tang", nx=6, ny=6, N=5, jitter=0.1, seed=9, k_stage=5)]


def _bytes(path):
    with open(path, "rb") as f:
        return f.read()


@pytest.mark.parametrize("spec", CASES, ids=["ot_10x9_N4", "rotor_64x64_N3", "ot_6x6_N5_fivestage"])
def test_restart_file_byte_identical_to_oracle_writer(case_root, tmp_path, spec):
    d = make_case(case_root, **spec)
    s = Solver(Mesh(d))
    s.iterations(7)
    gpu_file = str(tmp_path / "gpu.dat")
    s.write_restart(gpu_file)
    # the oracle writes the same state with its own writer
    o = oracle.Oracle(d)
    o.array("Q")[:] = s.state()
    o.seti("iter", s.iter)
    o.setd("ctime", s.ctime)
    orc_file = str(tmp_path / "orc.dat")
    assert o.write_restart(orc_file) == 0
    a, b = _bytes(gpu_file), _bytes(orc_file)
    nq = 9 * s.N * s.N
    assert len(a) == 12 + s.ncell * (4 + 8 * nq)
    assert a == b
    # header: int32 iter, float64 ctime; then per cell int32 global id + Q(9,N,N)
    assert np.frombuffer(a[:4], np.int32)[0] == 7
    assert np.frombuffer(a[4:12], np.float64)[0] == s.ctime
    s.close()
    o.close()


def test_each_side_reads_the_others_restart(case_root, tmp_path):
    d = make_case(case_root, **CASES[0])
    # oracle run -> oracle file -> GPU reader
    o = oracle.Oracle(d)
    for _ in range(4):
        o.step()
    f1 = str(tmp_path / "orc.dat")
    o.write_restart(f1)
    s = Solver(Mesh(d))
    s.read_restart(f1)
    assert (s.iter, s.ctime) == (o.geti("iter"), o.getd("ctime"))
    assert np.array_equal(s.state(), o.array("Q"))
    # GPU run -> GPU file -> oracle reader
    s.iterations(3)
    f2 = str(tmp_path / "gpu.dat")
    s.write_restart(f2)
    o2 = oracle.Oracle(d)
    assert o2.read_restart(f2) == 0
    assert o2.geti("iter") == s.iter == 7
    assert o2.getd("ctime") == s.ctime
    assert np.array_equal(o2.array("Q"), s.state())
    s.close()
    o.close()
    o2.close()


@pytest.mark.parametrize("spec", CASES[:2], ids=["ot_10x9_N4", "rotor_64x64_N3"])
def test_resumed_run_equals_uninterrupted_run(case_root, tmp_path, spec):
    """k steps, restart file, a fresh context reads it and runs j more steps: the same
    state, iteration, time and diagnostics as k + j steps without interruption."""
    d = make_case(case_root, **spec)
    k, j = 6, 9
    full = Solver(Mesh(d))
    diag_full = full.iterations(k + j)
    part = Solver(Mesh(d))
    part.iterations(k)
    f = str(tmp_path / ("restart.%08d.dat" % k))
    part.write_restart(f)
    part.close()
    resumed = Solver(Mesh(d), initial_state=False)
    resumed.read_restart(f)
    assert resumed.iter == k
    diag_res = resumed.iterations(j)
    assert resumed.iter == full.iter and resumed.ctime == full.ctime
    assert np.array_equal(resumed.state(), full.state())
    # the norms of the resumed steps (iter 11) are the uninterrupted run's
    later = [r for r in diag_full if r["iter"] > k]
    assert len(later) == len(diag_res) >= 1
    for a, b in zip(later, diag_res):
        assert a == b
    full.close()
    resumed.close()


def test_restart_reader_keeps_cells_the_file_does_not_name(case_root, tmp_path):
    """READ_ALL_DATA_BINARY reads NCELLGLOB records in the order they come and assigns
    only the cells they name (read_data_restart.f90:50-56): records in any order give
    the same state, a cell named twice takes its last record, and a cell the stream does
    not name keeps the state it had."""
    d = make_case(case_root, **CASES[0])
    s = Solver(Mesh(d))
    s.iterations(2)
    Q = s.state().copy()
    nq = 9 * s.N * s.N
    perm = np.random.default_rng(3).permutation(s.ncell)
    missing, twice = int(perm[0]), int(perm[1])
    recs = [(e, Q[e * nq:(e + 1) * nq]) for e in perm[1:]] + [(twice, Q[twice * nq:(twice + 1) * nq] + 1.0)]
    f = str(tmp_path / "shuffled.dat")
    with open(f, "wb") as fh:
        fh.write(np.int32(2).tobytes())
        fh.write(np.float64(s.ctime).tobytes())
        for e, q in recs:
            fh.write(np.int32(e + 1).tobytes())
            fh.write(np.ascontiguousarray(q).tobytes())
    t = Solver(Mesh(d))  # holds the initial state
    Q0 = t.state().copy()
    t.read_restart(f)
    want = Q.copy()
    want[missing * nq:(missing + 1) * nq] = Q0[missing * nq:(missing + 1) * nq]
    want[twice * nq:(twice + 1) * nq] += 1.0
    assert np.array_equal(t.state(), want)
    # the oracle's reader agrees
    o = oracle.Oracle(d)
    assert o.read_restart(f) == 0
    o0 = oracle.Oracle(d)
    wo = Q.copy()
    wo[missing * nq:(missing + 1) * nq] = o0.array("Q")[missing * nq:(missing + 1) * nq]
    wo[twice * nq:(twice + 1) * nq] += 1.0
    assert np.array_equal(o.array("Q"), wo)
    s.close()
    t.close()
    o.close()
    o0.close()
