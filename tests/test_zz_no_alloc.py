"""getrusanovflux_noalloc_gpu: the Rusanov point evaluator for callers that cannot
allocate device memory (their device memory is all held by their own pool, or they have
work in flight that a cudaFree would stall).  It must give what getrusanovflux_gpu gives,
call after call, while staging through the library's fixed device array.

This file is collected last on purpose, so a run that stops at the first failure has
already run every other test; it also passes alone in a fresh process."""
import ctypes

import numpy as np
import pytest

from chorus_mhd import _lib

TOL = 1e-12  # the point-function tolerance used by tests/test_gpu_points.py
MAX_POINTS = 32768


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))


def _states(rng, n, gam):
    rho = rng.uniform(0.5, 3.0, n)
    u = rng.uniform(-1, 1, (n, 3))
    B = rng.uniform(-1, 1, (n, 3))
    p = rng.uniform(0.2, 2.0, n)
    Q = np.zeros((n, 9))
    Q[:, 0] = rho
    Q[:, 1:4] = rho[:, None] * u
    Q[:, 4] = p / (gam - 1) + 0.5 * rho * (u ** 2).sum(1) + 0.5 * (B ** 2).sum(1)
    Q[:, 5:8] = B
    Q[:, 8] = rng.uniform(-1, 1, n)
    return Q


def _call(fn, n, gam, Ql, Qr, nf, sl, sr):
    Fl, Fr, Az, ev = np.zeros((n, 8)), np.zeros((n, 8)), np.zeros(n), np.zeros(n)
    _lib.check(fn(n, gam, _dp(Ql), _dp(Qr), _dp(Fl), _dp(Fr), _dp(Az), _dp(nf), _ip(sl), _ip(sr), _dp(ev)))
    return Fl, Fr, Az, ev


@pytest.mark.gpu
def test_no_alloc_rusanov_matches_allocating_entry_point_twice():
    L = _lib.load()
    gam = 5.0 / 3
    for call, n in enumerate([3000, 1700]):  # two calls in a row, the second smaller
        rng = np.random.default_rng(100 + call)
        Ql, Qr = _states(rng, n, gam), _states(rng, n, gam)
        nf = rng.uniform(-2, 2, (n, 2))
        sl = rng.choice([-1, 1], n).astype(np.int32)
        sr = rng.choice([-1, 1], n).astype(np.int32)
        ref = _call(L.getrusanovflux_gpu, n, gam, Ql, Qr, nf, sl, sr)
        got = _call(L.getrusanovflux_noalloc_gpu, n, gam, Ql, Qr, nf, sl, sr)
        for a, b, name in zip(got, ref, ["Fnl", "Fnr", "Az", "eigv"]):
            scale = np.abs(b).max() + 1.0
            assert np.all(np.isfinite(a)), name
            assert np.abs(a - b).max() <= TOL * scale, "call %d: %s differs" % (call + 1, name)


@pytest.mark.gpu
def test_no_alloc_rejects_more_points_than_its_capacity():
    L = _lib.load()
    n = MAX_POINTS + 1
    z9, z8, z2, z1 = np.zeros((n, 9)), np.zeros((n, 8)), np.zeros((n, 2)), np.zeros(n)
    s = np.ones(n, np.int32)
    rc = L.getrusanovflux_noalloc_gpu(n, 1.4, _dp(z9), _dp(z9), _dp(z8), _dp(z8), _dp(z1), _dp(z2), _ip(s),
                                      _ip(s), _dp(z1))
    assert rc == 1
    assert b"capacity" in L.chorus_gpu_last_error()
