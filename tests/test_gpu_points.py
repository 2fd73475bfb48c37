"""Device point functions (getrusanovflux / getIfluxvectors / getVfluxvectors) vs
the oracle's restatement, on random physical states."""
import ctypes

import numpy as np
import pytest

import oracle
from chorus_mhd import _lib

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))


def random_states(rng, n):
    rho = rng.uniform(0.5, 3.0, n)
    u = rng.uniform(-1, 1, (n, 3))
    B = rng.uniform(-1, 1, (n, 3))
    p = rng.uniform(0.2, 2.0, n)
    gam = 5.0 / 3
    Q = np.zeros((n, 9))
    Q[:, 0] = rho
    Q[:, 1:4] = rho[:, None] * u
    Q[:, 4] = p / (gam - 1) + 0.5 * rho * (u ** 2).sum(1) + 0.5 * (B ** 2).sum(1)
    Q[:, 5:8] = B
    Q[:, 8] = rng.uniform(-1, 1, n)
    return Q


def test_rusanov_points():
    rng = np.random.default_rng(0)
    n = 500
    gam = 5.0 / 3
    Ql, Qr = random_states(rng, n), random_states(rng, n)
    nf = rng.uniform(-2, 2, (n, 2))
    sl = rng.choice([-1, 1], n).astype(np.int32)
    sr = rng.choice([-1, 1], n).astype(np.int32)
    Fl, Fr, Az, ev = np.zeros((n, 8)), np.zeros((n, 8)), np.zeros(n), np.zeros(n)
    L = _lib.load()
    _lib.check(L.getrusanovflux_gpu(n, gam, _dp(Ql), _dp(Qr), _dp(Fl), _dp(Fr), _dp(Az), _dp(nf), _ip(sl), _ip(sr),
                                    _dp(ev)))
    for i in range(n):
        a, b, z, e = oracle.getrusanovflux(gam, Ql[i], Qr[i], nf[i], sl[i], sr[i])
        sc = np.abs(a).max() + 1.0
        assert np.abs(Fl[i] - a).max() <= TOL * sc
        assert np.abs(Fr[i] - b).max() <= TOL * sc
        assert Az[i] == z
        assert abs(ev[i] - e) <= TOL * e


def test_iflux_points():
    rng = np.random.default_rng(1)
    n = 300
    gam = 1.4
    Q = random_states(rng, n)[:, :8].copy()
    F, G = np.zeros((n, 8)), np.zeros((n, 8))
    L = _lib.load()
    _lib.check(L.getifluxvectors_gpu(n, gam, _dp(Q), _dp(F), _dp(G)))
    for i in range(n):
        a, b = oracle.getifluxvectors(gam, Q[i])
        assert np.abs(F[i] - a).max() <= TOL * (np.abs(a).max() + 1)
        assert np.abs(G[i] - b).max() <= TOL * (np.abs(b).max() + 1)


@pytest.mark.parametrize("mu,eta0", [(0.01, 0.0), (0.0, 0.03), (0.02, 0.05)])
def test_vflux_points(mu, eta0):
    rng = np.random.default_rng(2)
    n = 300
    gam = 5.0 / 3
    Q = random_states(rng, n)
    G = rng.uniform(-1, 1, (n, 18))
    Fv, Gv = np.zeros((n, 9)), np.zeros((n, 9))
    L = _lib.load()
    _lib.check(L.getvfluxvectors_gpu(n, gam, mu, eta0, _dp(Q), _dp(G), _dp(Fv), _dp(Gv)))
    for i in range(n):
        a, b = oracle.getvfluxvectors(gam, mu, eta0, Q[i], G[i])
        assert np.abs(Fv[i] - a).max() <= TOL * (np.abs(a).max() + 1e-300) + 1e-300
        assert np.abs(Gv[i] - b).max() <= TOL * (np.abs(b).max() + 1e-300) + 1e-300


def test_vflux_av_points_use_the_solve_face_viscosity(case_root):
    """getVfluxvectors_AV(Qv,nablaQ,Fv,Gv,fam,ifp,jfp,ic) on a bound solve: mu_art from
    the face viscosities its last compresid left, against the oracle's own muAVfi/j."""
    from chorus_mhd import Mesh, Solver
    from helpers import make_case
    d = make_case(case_root, problem="rotor", nx=64, ny=64, N=3, jitter=0.1, seed=6)
    o = oracle.Oracle(d)
    o.run(2)
    s = Solver(Mesh(d), initial_state=False)
    s.upload(o.array("Q").copy())
    o.compresid()
    s.compresid()
    N, NC, gam = s.N, s.ncell, o.getd("gam")
    Xf = o.array("Xf")
    mfi = o.array("muAVfi").reshape(NC, 2, 9)[:, :, 0]
    mfj = o.array("muAVfj").reshape(NC, 2, 9)[:, :, 0]
    hot = np.flatnonzero((mfi > 0).any(1) | (mfj > 0).any(1))
    assert hot.size > 0, "the case must have AV somewhere"
    rng = np.random.default_rng(11)
    n = 600
    fam = rng.integers(1, 3, n).astype(np.int32)
    ifp = np.where(fam == 1, rng.integers(1, N + 2, n), rng.integers(1, N + 1, n)).astype(np.int32)
    jfp = np.where(fam == 1, rng.integers(1, N + 1, n), rng.integers(1, N + 2, n)).astype(np.int32)
    ic = np.where(rng.random(n) < 0.7, rng.choice(hot, n) + 1, rng.integers(1, NC + 1, n)).astype(np.int32)
    Q = random_states(rng, n)
    G = rng.normal(size=(n, 18))
    Fv, Gv = np.zeros((n, 9)), np.zeros((n, 9))
    L = _lib.load()
    _lib.check(L.getvfluxvectors_av_gpu(s._ctx, n, _dp(Q), _dp(G), _dp(Fv), _dp(Gv), _ip(fam), _ip(ifp), _ip(jfp),
                                        _ip(ic)))
    worst = 0.0
    for i in range(n):
        c = ic[i] - 1
        if fam[i] == 1:
            x = Xf[ifp[i] - 1]
            mu_art = mfi[c, 0] * (1.0 - x) + mfi[c, 1] * x
        else:
            x = Xf[jfp[i] - 1]
            mu_art = mfj[c, 0] * (1.0 - x) + mfj[c, 1] * x
        a, b = oracle.getvfluxvectors(gam, mu_art, 0.0, Q[i], G[i])
        scale = max(1e-300, np.abs(a).max(), np.abs(b).max())
        worst = max(worst, np.abs(Fv[i] - a).max() / scale, np.abs(Gv[i] - b).max() / scale)
    assert worst <= 1e-11, worst
    # indices outside the solve are refused before any device work
    bad = ic.copy()
    bad[3] = NC + 1
    assert L.getvfluxvectors_av_gpu(s._ctx, n, _dp(Q), _dp(G), _dp(Fv), _dp(Gv), _ip(fam), _ip(ifp), _ip(jfp),
                                    _ip(bad)) == 1
    s.close()


def test_single_point_forms_with_the_reference_argument_lists():
    """getrusanovflux_c / getifluxvectors_c / getvfluxvectors_c: one point, arguments by
    reference as a Fortran CALL passes them, gam/mu/eta0 as module state; eigvmax is
    raised only by a larger wave speed (getrusanov.f90:105-107)."""
    L = _lib.load()
    rng = np.random.default_rng(5)
    gam, mu, eta0 = 1.4, 0.02, 0.01
    _lib.check(L.chorus_point_set_params(gam, mu, eta0))
    try:
        Q = random_states(rng, 4)
        nf = rng.normal(size=(4, 2))
        eigvmax = np.array([0.0])
        seen = []
        for i in range(3):
            Fl, Fr, Az, ev = np.zeros(8), np.zeros(8), np.zeros(1), np.zeros(1)
            sl, sr = np.array([1], np.int32), np.array([-1 if i % 2 else 1], np.int32)
            _lib.check(L.getrusanovflux_c(_dp(Q[i]), _dp(Q[i + 1]), _dp(Fl), _dp(Fr), _dp(Az), _dp(nf[i]), _ip(sl),
                                          _ip(sr), _dp(ev), _dp(eigvmax)))
            a, b, z, e = oracle.getrusanovflux(gam, Q[i], Q[i + 1], nf[i], sl[0], sr[0])
            assert np.allclose(Fl, a, rtol=TOL, atol=TOL) and np.allclose(Fr, b, rtol=TOL, atol=TOL)
            assert Az[0] == z and abs(ev[0] - e) <= TOL * e
            seen.append(ev[0])
            assert eigvmax[0] == max(seen)
        F, G = np.zeros(8), np.zeros(8)
        _lib.check(L.getifluxvectors_c(_dp(np.ascontiguousarray(Q[0, :8])), _dp(F), _dp(G)))
        a, b = oracle.getifluxvectors(gam, Q[0, :8])
        assert np.allclose(F, a, rtol=TOL, atol=TOL) and np.allclose(G, b, rtol=TOL, atol=TOL)
        g = rng.normal(size=18)
        Fv, Gv = np.zeros(9), np.zeros(9)
        _lib.check(L.getvfluxvectors_c(_dp(Q[1]), _dp(g), _dp(Fv), _dp(Gv)))
        a, b = oracle.getvfluxvectors(gam, mu, eta0, Q[1], g)
        assert np.allclose(Fv, a, rtol=1e-11, atol=1e-13) and np.allclose(Gv, b, rtol=1e-11, atol=1e-13)
    finally:
        _lib.check(L.chorus_point_set_params(5.0 / 3, 0.0, 0.0))
