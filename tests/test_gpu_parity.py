"""CUDA path vs the oracle on the same inputs (through the C-ABI).

Tolerances: FP64 throughout; the kernels regroup the reference's algebra (fused
multiply-adds, one reciprocal per point, precomputed metric weights), so single-stage
arrays agree to ~1e-13 relative and whole runs to the stated 1e-10 relative L2.
"""
import numpy as np
import pytest

import oracle
from chorus_mhd import Mesh, Solver, reference_layout_sizes
from helpers import alfven_wave_bz, alfven_wave_case, diffusion_wave_case, entropy_wave_case, entropy_wave_state, quadrature_l2, assert_close, make_case, rel_l2, shuffled_case

pytestmark = pytest.mark.gpu

STAGE_TOL = 1e-12   # one compresid, normwise relative
RUN_TOL = 1e-10     # whole run, relative L2 of Q (the stated bar)

CASES = [
    dict(problem="orszag_tang", nx=6, ny=6, N=4, jitter=0.0),
    dict(problem="orszag_tang", nx=5, ny=7, N=3, jitter=0.15, seed=2),
    dict(problem="orszag_tang", nx=4, ny=4, N=5, jitter=0.15, seed=3),
    dict(problem="orszag_tang", nx=4, ny=3, N=6, jitter=0.1, seed=4),
    dict(problem="orszag_tang", nx=3, ny=3, N=2, jitter=0.0),
    dict(problem="orszag_tang", nx=3, ny=4, N=7, jitter=0.1, seed=5),
    dict(problem="orszag_tang", nx=3, ny=3, N=8, jitter=0.0),
    dict(problem="rotor", nx=64, ny=64, N=3, jitter=0.1, seed=6),
    dict(problem="alfven", nx=6, ny=5, N=4, jitter=0.0),
    dict(problem="orszag_tang", nx=6, ny=6, N=4, jitter=0.1, mu=0.01, eta0=0.02, seed=7),
    dict(problem="orszag_tang", nx=5, ny=5, N=4, jitter=0.0, artiv=0),
]


def ids(c):
    return "%s-%dx%d-N%d-j%s%s" % (c["problem"], c["nx"], c["ny"], c["N"], c.get("jitter", 0),
                                 "-visc" if c.get("mu") else "" + ("-noav" if c.get("artiv") == 0 else ""))


@pytest.mark.parametrize("case", CASES, ids=ids)
def test_initial_state_matches_oracle(case_root, case):
    d = make_case(case_root, **case)
    o = oracle.Oracle(d)
    s = Solver(Mesh(d))
    assert_close(s.state(), o.array("Q"), 1e-13, "initial Q")


@pytest.mark.parametrize("case", CASES, ids=ids)
def test_one_stage_arrays_match_oracle(case_root, case):
    """compresid on identical input: every intermediate array of compflux."""
    d = make_case(case_root, **case)
    o = oracle.Oracle(d)
    o.run(2)  # move away from the symmetric initial data
    Q = o.array("Q").copy()
    s = Solver(Mesh(d), initial_state=False)
    s.set_option("skip_inactive_viscous", 0)  # fill every gradient array for comparison
    s.upload(Q)
    o.compresid()
    s.compresid()
    sz = reference_layout_sizes(s.N, s.ncell)
    for name in ["F1", "G2", "Qvfi", "Qvfj", "Azfi", "Azfj", "nablaAs", "resid"]:
        assert_close(s.array(name, sz[name]), o.array(name), STAGE_TOL, name)
    for name in ["nablaQs", "nablaQvfi", "nablaQvfj"]:
        a = s.array(name, sz[name]).reshape(-1, 9)[:, :8]
        b = o.array(name).reshape(-1, 9)[:, :8]
        assert_close(a, b, STAGE_TOL, name)
    if case.get("artiv", 1):
        for name in ["muAVfi", "muAVfj"]:
            a = s.array(name, sz[name]).reshape(-1, 9)[:, 0]
            b = o.array(name).reshape(-1, 9)[:, 0]
            assert np.allclose(a, b, rtol=1e-11, atol=1e-14 * max(1.0, np.abs(b).max())), name
        # the sensor only matters through muAV: below -6 the viscosity is zero, so a
        # smoothing that reproduces a constant density exactly (-inf) and one that
        # leaves 1e-30 of round-off (-30) are the same answer
        se = s.array("SM_IND1", s.ncell)
        so = o.array("SM_IND").reshape(-1, 9)[:, 0]
        assert np.array_equal(se >= -6.0, so >= -6.0)
        live = so >= -12.0
        assert np.allclose(se[live], so[live], rtol=0, atol=1e-8)
    ev, eps = s.eigvmax()
    assert abs(ev - o.getd("eigvmax")) <= 1e-13 * o.getd("eigvmax")


@pytest.mark.parametrize("case", CASES[:4] + CASES[6:9], ids=ids)
def test_comp_inviscid_flux_drop_in_matches_oracle(case_root, case):
    """comp_inviscid_flux_gpu alone (compflux.f90:33-49): the interior and face
    inviscid fluxes F1/G2, the face-averaged traces Qvfi/Qvfj, the upwinded A_z traces
    Azfi/Azfj and the stage's maximum wave speed, on the oracle's state after two steps."""
    d = make_case(case_root, **case)
    o = oracle.Oracle(d)
    o.run(2)
    s = Solver(Mesh(d), initial_state=False)
    s.upload(o.array("Q").copy())
    # the reference's routine only raises the module's eigvmax, which compflux zeroes
    # before it (compflux.f90:1-31); the drop-in reports the maximum of its own faces
    o.setd("eigvmax", 0.0)
    o.comp_inviscid_flux()
    s.comp_inviscid_flux()
    sz = reference_layout_sizes(s.N, s.ncell)
    for name in ["F1", "G2", "Qvfi", "Qvfj", "Azfi", "Azfj"]:
        assert_close(s.array(name, sz[name]), o.array(name), STAGE_TOL, name)
    ev, _ = s.eigvmax()
    assert abs(ev - o.getd("eigvmax")) <= 1e-13 * o.getd("eigvmax")


@pytest.mark.parametrize("case", CASES, ids=ids)
def test_run_matches_oracle(case_root, case):
    """iterations: RK steps + CT projection + diagnostics vs the oracle."""
    d = make_case(case_root, **case)
    nsteps = 12
    o = oracle.Oracle(d)
    s = Solver(Mesh(d))
    diag_o = []
    for _ in range(nsteps):
        r = o.step()
        if r is not None:
            diag_o.append(r)
    diag_s = s.iterations(nsteps)
    assert_close(s.state(), o.array("Q"), RUN_TOL, "Q after %d steps" % nsteps)
    assert s.iter == o.geti("iter")
    assert abs(s.ctime - o.getd("ctime")) <= 1e-15 * max(1.0, o.getd("ctime"))
    assert len(diag_s) == len(diag_o) == 2
    for a, (rg, db) in zip(diag_s, diag_o):
        assert abs(a["residglob"] - rg) <= 1e-9 * rg
        assert abs(a["divBglob"] - db) <= 1e-9 * db + 1e-13


SMALLEST = [dict(problem="orszag_tang", nx=1, ny=1, N=4), dict(problem="orszag_tang", nx=1, ny=3, N=3),
            dict(problem="orszag_tang", nx=3, ny=1, N=5), dict(problem="rotor", nx=1, ny=1, N=2),
            dict(problem="alfven", nx=2, ny=1, N=3)]


@pytest.mark.parametrize("case", SMALLEST, ids=lambda c: "%s-%dx%d-N%d" % (c["problem"], c["nx"], c["ny"], c["N"]))
def test_smallest_meshes_match_oracle(case_root, case):
    """Meshes one cell wide, where a periodic face's partner is a face of the same cell
    (and a 1x1 FREE mesh with every face on the boundary): one residual evaluation and
    a short run against the oracle."""
    d = make_case(case_root, **case)
    o = oracle.Oracle(d)
    s = Solver(Mesh(d))
    assert_close(s.state(), o.array("Q"), 1e-13, "initial Q")
    o1 = oracle.Oracle(d)
    o1.run(2)
    t = Solver(Mesh(d), initial_state=False)
    t.set_option("skip_inactive_viscous", 0)
    t.upload(o1.array("Q").copy())
    o1.compresid()
    t.compresid()
    sz = reference_layout_sizes(t.N, t.ncell)
    for name in ["F1", "G2", "Qvfi", "Qvfj", "Azfi", "Azfj"]:
        assert_close(t.array(name, sz[name]), o1.array(name), STAGE_TOL, name)
    # a uniform state (the 1x1 rotor cell has no point inside the disk) has a residual of
    # pure round-off on both sides: then the bound is absolute, on the scale of the fluxes
    r_gpu, r_orc = t.array("resid", sz["resid"]), o1.array("resid")
    scale = max(np.linalg.norm(r_orc), np.linalg.norm(o1.array("F1")))
    assert np.linalg.norm(r_gpu - r_orc) <= STAGE_TOL * scale, "resid"
    for _ in range(6):
        o.step()
    s.iterations(6)
    assert_close(s.state(), o.array("Q"), RUN_TOL, "Q after 6 steps")
    s.close()
    t.close()


def test_fivestage_rk_matches_oracle(case_root):
    d = make_case(case_root, problem="orszag_tang", nx=5, ny=5, N=4, jitter=0.1, k_stage=5, seed=9)
    o = oracle.Oracle(d)
    s = Solver(Mesh(d))
    for _ in range(6):
        o.step()
    s.iterations(6)
    assert_close(s.state(), o.array("Q"), RUN_TOL, "FiveStageRk")


def test_drop_in_sequence_matches_oracle(case_root):
    """RK_S5P3 + correct_B_via_curl_Az called one by one, like iterations.f90:22-33."""
    d = make_case(case_root, problem="orszag_tang", nx=6, ny=5, N=4, jitter=0.1, seed=11)
    o = oracle.Oracle(d)
    s = Solver(Mesh(d))
    for _ in range(3):
        o.rk_s5p3()
        o.correct_B_via_curl_Az()
        s.RK_S5P3()
        s.correct_B_via_curl_Az()
    assert_close(s.state(), o.array("Q"), RUN_TOL, "drop-in sequence")
    assert s.ctime == pytest.approx(o.getd("ctime"), rel=1e-15)


def gpu_entropy_wave_error(case_root, nx, N, cfl, T=0.4, jitter=0.0):
    d, steps = entropy_wave_case(case_root, nx, N, cfl, T, jitter)
    m = Mesh(d)
    s = Solver(m, initial_state=False)
    X = m.darray("XXsolu").reshape(-1, 2)
    s.upload(np.ascontiguousarray(entropy_wave_state(X).ravel()))
    s.iterations(steps)
    err = s.state().reshape(-1, 9)[:, 0] - entropy_wave_state(X, T)[:, 0]
    e = quadrature_l2(err, m.darray("Jac"), m.darray("Xs"))
    s.close()
    return e


@pytest.mark.parametrize("N,cfl,sizes,rate", [(3, 0.2, (8, 16, 32, 64), 2.9), (5, 0.02, (8, 16, 32, 64), 4.8)])
def test_entropy_wave_converges_at_design_order(case_root, N, cfl, sizes, rate):
    """Through the C-ABI, the exact advected entropy wave is approached as h^N; on the
    meshes the oracle finishes quickly the errors equal the oracle's to 1e-8 relative."""
    import math
    errs = [gpu_entropy_wave_error(case_root, nx, N, cfl) for nx in sizes]
    rates = [math.log2(errs[i] / errs[i + 1]) for i in range(len(errs) - 1)]
    assert rates[-1] >= rate, (errs, rates)
    d, steps = entropy_wave_case(case_root, sizes[1], N, cfl, 0.4)
    o = oracle.Oracle(d, threads=0)
    X = o.array("XXsolu").reshape(-1, 2)
    o.array("Q")[:] = entropy_wave_state(X).ravel()
    for _ in range(steps):
        o.step()
    e_o = quadrature_l2(o.array("Q").reshape(-1, 9)[:, 0] - entropy_wave_state(X, 0.4)[:, 0], o.array("Jac"), o.array("Xs"))
    assert abs(errs[1] - e_o) <= 1e-8 * e_o
    o.close()


@pytest.mark.parametrize("kind", ["viscous", "resistive"])
def test_diffusion_waves_decay_at_the_exact_rate(case_root, kind):
    """The viscous shear and resistive magnetic waves through the C-ABI (N = 4, 8^2..32^2):
    the error against A sin(x) exp(-0.05 t) falls as h^4 and equals the oracle's on 16^2."""
    import math
    errs = []
    for nx in (8, 16, 32):
        d, steps, state, var = diffusion_wave_case(case_root, nx, 4, kind, 0.05, 0.5)
        m = Mesh(d)
        s = Solver(m, initial_state=False)
        X = m.darray("XXsolu").reshape(-1, 2)
        s.upload(np.ascontiguousarray(state(X).ravel()))
        s.iterations(steps)
        err = s.state().reshape(-1, 9)[:, var] - state(X, 0.5)[:, var]
        errs.append(quadrature_l2(err, m.darray("Jac"), m.darray("Xs")) / 1e-3)
        s.close()
    rates = [math.log2(errs[i] / errs[i + 1]) for i in range(len(errs) - 1)]
    assert rates[-1] >= 3.5, (errs, rates)
    d, steps, state, var = diffusion_wave_case(case_root, 16, 4, kind, 0.05, 0.5)
    o = oracle.Oracle(d, threads=0)
    X = o.array("XXsolu").reshape(-1, 2)
    o.array("Q")[:] = state(X).ravel()
    for _ in range(steps):
        o.step()
    e_o = quadrature_l2(o.array("Q").reshape(-1, 9)[:, var] - state(X, 0.5)[:, var], o.array("Jac"), o.array("Xs")) / 1e-3
    assert abs(errs[1] - e_o) <= 1e-8 * e_o
    o.close()


def test_alfven_wave_converges_at_design_order(case_root):
    """The circularly polarised Alfven wave through the C-ABI (N = 4, 8^2..64^2): B_z after
    t = 0.25 approaches the exact wave as h^4, and on 16^2 equals the oracle's error to 1e-8."""
    import math
    errs = []
    for nx in (8, 16, 32, 64):
        d, steps = alfven_wave_case(case_root, nx, 4, 0.05, 0.25)
        m = Mesh(d)
        s = Solver(m)
        X = m.darray("XXsolu").reshape(-1, 2)
        s.iterations(steps)
        errs.append(quadrature_l2(s.state().reshape(-1, 9)[:, 7] - alfven_wave_bz(X, 0.25), m.darray("Jac"),
                                  m.darray("Xs")))
        s.close()
    rates = [math.log2(errs[i] / errs[i + 1]) for i in range(len(errs) - 1)]
    assert rates[-1] >= 3.7, (errs, rates)  # RK3 time error enters at the finest mesh
    d, steps = alfven_wave_case(case_root, 16, 4, 0.05, 0.25)
    o = oracle.Oracle(d, threads=0)
    X = o.array("XXsolu").reshape(-1, 2)
    for _ in range(steps):
        o.step()
    e_o = quadrature_l2(o.array("Q").reshape(-1, 9)[:, 7] - alfven_wave_bz(X, 0.25), o.array("Jac"), o.array("Xs"))
    assert abs(errs[1] - e_o) <= 1e-8 * e_o
    o.close()


@pytest.mark.parametrize("spec", [dict(problem="orszag_tang", nx=6, ny=5, N=4, jitter=0.1, seed=17),
                                  dict(problem="rotor", nx=64, ny=64, N=3, jitter=0.1, seed=6)],
                         ids=["orszag_tang", "rotor_free"])
def test_ct_projection_arrays_match_oracle(case_root, spec):
    """After correct_B_via_curl_Az, alone and at the end of graph-replayed steps, the
    arrays the projection defines match the oracle: the state (B), the face-averaged A_z
    traces of Qvfi(9)/Qvfj(9) and nablaQs(9,:) (kept apart on the device and merged where
    they are read), also through nablaQsp(9,9) and after further drop-in calls."""
    d = make_case(case_root, **spec)
    o = oracle.Oracle(d)
    o.run(2)
    Q = o.array("Q").copy()
    s = Solver(Mesh(d), initial_state=False)
    s.upload(Q)
    o.correct_B_via_curl_Az()
    s.correct_B_via_curl_Az()
    sz = reference_layout_sizes(s.N, s.ncell)

    def var9(name):
        a = s.array(name, sz[name]).reshape(-1, 9)[:, 8]
        b = o.array(name).reshape(-1, 9)[:, 8]
        return a, b

    assert_close(s.state(), o.array("Q"), STAGE_TOL, "Q after the projection")
    for name in ("Qvfi", "Qvfj", "nablaQs"):
        a, b = var9(name)
        assert_close(a, b, STAGE_TOL, name + "(9)")
    # nablaQsp(9,9) recomputes variable 9 from the (pending) traces
    s.nablaQsp(9, 9)
    o.nablaQsp(9, 9)
    a, b = var9("nablaQs")
    assert_close(a, b, STAGE_TOL, "nablaQs(9) after nablaQsp(9,9)")
    # a residual evaluation rewrites every Qvf variable; nablaQs(9) keeps the projection's
    s.compresid()
    o.compresid()
    for name in ("Qvfi", "Qvfj", "nablaQs"):
        a, b = var9(name)
        assert_close(a, b, STAGE_TOL, name + "(9) after compresid")
    # graph-replayed steps end with the projection
    s2 = Solver(Mesh(d), initial_state=False)
    s2.upload(Q)
    o2 = oracle.Oracle(d)
    o2.array("Q")[:] = Q
    for _ in range(3):
        o2.step()
    s2.iterations(3)
    for name in ("Qvfi", "Qvfj", "nablaQs"):
        a = s2.array(name, sz[name]).reshape(-1, 9)[:, 8]
        b = o2.array(name).reshape(-1, 9)[:, 8]
        assert_close(a, b, RUN_TOL, name + "(9) after steps")
    for x in (s, s2):
        x.close()


@pytest.mark.parametrize("case", [c for c in CASES if c.get("artiv", 1) and not c.get("mu")], ids=ids)
def test_skipping_inactive_viscous_work_changes_nothing(case_root, case):
    """With mu = eta0 = 0 the skipped work is an exact zero: the residual with skipping
    equals the residual computed on every cell."""
    d = make_case(case_root, **case)
    o = oracle.Oracle(d)
    o.run(2)
    Q = o.array("Q").copy()
    sz = reference_layout_sizes(case["N"], case["nx"] * case["ny"])
    res = []
    for opt in (0, 1):
        s = Solver(Mesh(d), initial_state=False)
        s.set_option("skip_inactive_viscous", opt)
        assert s.get_option("skip_active") == opt
        s.upload(Q)
        s.compresid()
        res.append(s.array("resid", sz["resid"]))
    assert np.array_equal(res[0], res[1])


def test_step_host_graph_cache(case_root):
    """The captured host-state steps (one graph per pinned buffer pair and step kind) give
    the resident run's bits while the buffers alternate, a pageable buffer (the uncaptured
    path) comes between them, the chunk count changes and the time step changes."""
    torch = pytest.importorskip("torch")
    d = make_case(case_root, problem="orszag_tang", nx=256, ny=240, N=4, jitter=0.1, seed=21)
    a = Solver(Mesh(d))
    b = Solver(Mesh(d))
    q = a.state()
    dt0 = a.mesh.params.dt
    pins = [torch.empty(q.size, dtype=torch.float64, pin_memory=True).numpy() for _ in range(2)]
    page = np.empty_like(q)
    bufs = [pins[0], pins[1], page, pins[0], pins[1], pins[0], pins[1], pins[0], pins[1], pins[0], pins[1], pins[0]]
    for k, buf in enumerate(bufs):
        if k == 5:
            for s in (a, b):
                s.set_params(dt=0.5 * dt0)
        if k == 8:
            b.set_option("host_chunks", 3)
        buf[:] = q
        b.step_host(buf, buf, 1)
        a.iterations(1)
        q = a.state()
        assert np.array_equal(buf, q), "step %d" % (k + 1)
    assert b.iter == a.iter and b.ctime == a.ctime
    assert [r["residglob"] for r in b.diagnostics] == [r["residglob"] for r in a.diagnostics]
    a.close()
    b.close()


def test_step_host_on_scattered_cell_numbering(case_root):
    """Cells numbered in a random order: nearly every cell has a face neighbour in the last
    chunk, so the chunk plan downloads whole chunks, each once its last neighbour is through;
    the host-state step still gives the resident steps' bits."""
    torch = pytest.importorskip("torch")
    d = shuffled_case(case_root, 3, problem="orszag_tang", nx=256, ny=240, N=4, jitter=0.1, seed=21)
    a = Solver(Mesh(d))
    q0 = a.state()
    a.iterations(2)
    ref = a.state()
    pin = torch.empty(q0.size, dtype=torch.float64, pin_memory=True).numpy()
    pin[:] = q0
    b = Solver(Mesh(d))
    b.step_host(pin, pin, 2)
    assert np.array_equal(pin, ref)
    a.close()
    b.close()


def test_host_chunks_option_range(case_root):
    d = make_case(case_root, problem="orszag_tang", nx=8, ny=8, N=3)
    s = Solver(Mesh(d))
    assert s.get_option("host_chunks") == 16
    for bad in (0, 33):
        with pytest.raises(Exception, match="host_chunks"):
            s.set_option("host_chunks", bad)
    assert s.get_option("host_chunks") == 16
    s.close()


@pytest.mark.parametrize("problem,nx,ny,nsteps,chunks", [
    ("orszag_tang", 72, 64, 1, 16), ("orszag_tang", 72, 64, 3, 16), ("orszag_tang", 256, 240, 1, 16),
    ("orszag_tang", 256, 240, 12, 16), ("orszag_tang", 256, 240, 2, 5), ("orszag_tang", 256, 240, 2, 32),
    ("rotor", 256, 240, 2, 16), ("rotor", 256, 240, 1, 7)])
def test_step_host_equals_resident_steps(case_root, problem, nx, ny, nsteps, chunks):
    """chorus_gpu_step_host gives the same bits as upload + iterations_gpu + download, for
    pageable and pinned host buffers: small states (plain copies around the step graph)
    and states of 64 MB and more (chunked copies overlapping the first stage's E1/F1 and
    the last stage's E3 and CT passes), periodic and FREE boundaries, several chunk counts."""
    d = make_case(case_root, problem=problem, nx=nx, ny=ny, N=4, jitter=0.1, seed=21)
    a = Solver(Mesh(d))
    Q0 = a.state()
    ref_diag = a.iterations(nsteps)
    ref = a.state()
    b = Solver(Mesh(d))
    b.set_option("host_chunks", chunks)
    assert b.get_option("host_chunks") == chunks
    out = np.empty_like(Q0)
    diag = b.step_host(Q0.copy(), out, nsteps)
    assert np.array_equal(out, ref)
    assert [r["residglob"] for r in diag] == [r["residglob"] for r in ref_diag]
    assert b.iter == a.iter and b.ctime == a.ctime
    # the same buffer in and out, pinned
    torch = pytest.importorskip("torch")
    pin = torch.empty(Q0.size, dtype=torch.float64, pin_memory=True).numpy()
    pin[:] = Q0
    c = Solver(Mesh(d))
    c.set_option("host_chunks", chunks)
    c.step_host(pin, pin, nsteps)
    assert np.array_equal(pin, ref)
    for s in (a, b, c):
        s.close()
