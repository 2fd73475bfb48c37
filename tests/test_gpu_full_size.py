"""The Orszag-Tang workload at its full size (512 x 512 cells, jittered mesh, N = 5,
6.55 M solution points) through the C-ABI: parity with the threaded oracle over the
first steps, then properties that hold at any size -- discrete conservation of the
weighted totals, bitwise repeatability, a resident run equal to the host-resident one,
positive density and pressure."""
import os

import numpy as np
import pytest

import oracle
from chorus_mhd import Mesh, Solver
from helpers import assert_close, make_case

pytestmark = pytest.mark.gpu

FULL = dict(problem="orszag_tang", nx=512, ny=512, N=5, jitter=0.15, seed=1)
RUN_TOL = 1e-10
GAM = 5.0 / 3.0


@pytest.fixture(scope="module")
def full_case(case_root):
    return make_case(case_root, **FULL)


@pytest.fixture(scope="module")
def mesh(full_case):
    m = Mesh(full_case)
    yield m
    m.close()


def quadrature_weights(xs):
    """Interpolatory weights on [0, 1] for the solution points xs: exact for the degree
    N-1 polynomials that the residual's flux derivative is, so that the weighted sum of
    the residual over a cell is its boundary flux."""
    n = len(xs)
    V = np.vander(np.asarray(xs, np.float64), n, increasing=True).T
    return np.linalg.solve(V, 1.0 / np.arange(1, n + 1))


def weighted_totals(Q, mesh):
    """sum over cells and points of Jac * w_i * w_j * Q_v, per variable v."""
    w = quadrature_weights(mesh.darray("Xs"))
    W = np.outer(w, w).ravel()
    J = mesh.darray("Jac")
    wJ = J * np.tile(W, J.size // W.size)
    Qv = np.asarray(Q).reshape(-1, 9)
    return (Qv * wJ[:, None]).sum(0), (np.abs(Qv) * wJ[:, None]).sum(0)


def test_full_size_first_steps_match_threaded_oracle(full_case, mesh):
    """Two RK steps, the CT projection and the first norms at full size."""
    o = oracle.Oracle(full_case, threads=os.cpu_count() or 1)
    diag_o = [r for r in (o.step(), o.step()) if r is not None]
    s = Solver(mesh)
    diag_s = s.iterations(2)
    assert_close(s.state(), o.array("Q"), RUN_TOL, "Q after 2 steps at 512x512")
    assert len(diag_s) == len(diag_o) >= 1
    # div B is a norm of derivatives that cancel down to the truncation error (2.7e-8
    # here), so its round-off is absolute: about eps times the scale of the derivative
    # operator, cells per side times N^2
    div_atol = 1e-15 * FULL["nx"] * FULL["N"] ** 2
    for a, (rg, db) in zip(diag_s, diag_o):
        assert abs(a["residglob"] - rg) <= 1e-9 * rg
        assert abs(a["divBglob"] - db) <= 1e-9 * db + div_atol
    s.close()
    o.close()


def test_full_size_conserves_weighted_totals(mesh):
    """The face fluxes are single-valued, so over the periodic domain the quadrature
    totals of rho, rho*u, rho*v, rho*w, E, Bx, By, Bz change only by round-off; A_z is
    advected in non-conservative form and is left out."""
    s = Solver(mesh)
    t0, scale = weighted_totals(s.state(), mesh)
    s.iterations(40)
    Q = s.state()
    t1, _ = weighted_totals(Q, mesh)
    assert np.all(np.isfinite(Q))
    ref = max(scale[0], scale[4])  # the mass and energy totals set the round-off level
    for v in range(8):
        assert abs(t1[v] - t0[v]) <= 1e-12 * ref, "variable %d: %.3e -> %.3e" % (v, t0[v], t1[v])
    s.close()


def test_full_size_positive_density_and_pressure(mesh):
    s = Solver(mesh)
    s.iterations(40)
    Q = s.state().reshape(-1, 9)
    rho = Q[:, 0]
    kin = 0.5 * (Q[:, 1] ** 2 + Q[:, 2] ** 2 + Q[:, 3] ** 2) / rho
    mag = 0.5 * (Q[:, 5] ** 2 + Q[:, 6] ** 2 + Q[:, 7] ** 2)
    p = (GAM - 1.0) * (Q[:, 4] - kin - mag)
    assert rho.min() > 0.0 and p.min() > 0.0
    s.close()


def test_full_size_runs_are_bitwise_repeatable(mesh):
    """No order-dependent reduction touches the state: two runs agree bit for bit."""
    out = []
    for _ in range(2):
        s = Solver(mesh)
        diag = s.iterations(12)
        out.append((s.state(), [(d["residglob"], d["divBglob"], d["eigvmax_g"]) for d in diag]))
        s.close()
    assert np.array_equal(out[0][0], out[1][0])
    assert out[0][1] == out[1][1]


def test_full_size_host_step_equals_resident_steps(mesh):
    """chorus_gpu_step_host at full size: 472 MB of state, copied in chunks that overlap the
    stage kernels, gives the resident result bit for bit."""
    a = Solver(mesh)
    q0 = a.state()
    ref_diag = a.iterations(3)
    qa = a.state()
    a.close()
    b = Solver(mesh, initial_state=False)
    qout = np.empty_like(q0)
    diag = b.step_host(q0, qout, 3)
    b.close()
    assert np.array_equal(qa, qout)
    assert [r["residglob"] for r in diag] == [r["residglob"] for r in ref_diag]


def test_full_size_free_stream_is_preserved(mesh):
    """A uniform state on the jittered 512x512 mesh has a zero residual to round-off: the
    residual scales as |flux| * N^2 / h, so its round-off grows with the cells per side
    (1e-9 here, 1e-12 on the oracle's 5x4 cells)."""
    s = Solver(mesh, initial_state=False)
    q0 = np.array([1.3, 0.4, -0.2, 0.1, 5.0, 0.7, -0.3, 0.2, 0.0])
    s.upload(np.ascontiguousarray(np.tile(q0, s.nq // 9)))
    s.compresid()
    from chorus_mhd import reference_layout_sizes
    r = s.array("resid", reference_layout_sizes(s.N, s.ncell)["resid"])
    scale = np.abs(q0).max() ** 2 * s.N ** 2 * FULL["nx"]
    assert np.abs(r).max() < 1e-13 * scale
    s.close()
