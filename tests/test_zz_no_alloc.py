"""getrusanovflux_noalloc_gpu: the Rusanov point evaluator for callers that cannot
allocate device memory (their device memory is all held by their own pool, or they have
work in flight that a cudaFree would stall).  It must give what getrusanovflux_gpu gives,
call after call, while staging through the library's fixed device array.

This file is collected last on purpose, so a run that stops at the first failure has
already run every other test; it also passes alone in a fresh process."""
import ctypes

import numpy as np
import pytest

import oracle
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


def _inputs(seed, n, gam):
    rng = np.random.default_rng(seed)
    Ql, Qr = _states(rng, n, gam), _states(rng, n, gam)
    nf = rng.uniform(-2, 2, (n, 2))
    sl = rng.choice([-1, 1], n).astype(np.int32)
    sr = rng.choice([-1, 1], n).astype(np.int32)
    return Ql, Qr, nf, sl, sr


@pytest.mark.gpu
def test_no_alloc_full_capacity_matches_oracle_and_allocates_nothing():
    """n equal to the capacity (the last slot of every region of the array is written)
    against the oracle's getrusanovflux point by point and against getrusanovflux_gpu; a
    second call leaves the device's free memory unchanged."""
    import torch
    L = _lib.load()
    gam = 1.4
    assert L.getrusanovflux_noalloc_gpu(0, gam, None, None, None, None, None, None, None, None, None) == 0  # set-up
    n = MAX_POINTS
    args = _inputs(7, n, gam)
    got = _call(L.getrusanovflux_noalloc_gpu, n, gam, *args)
    ref = _call(L.getrusanovflux_gpu, n, gam, *args)
    Ql, Qr, nf, sl, sr = args
    orc = [np.zeros((n, 8)), np.zeros((n, 8)), np.zeros(n), np.zeros(n)]
    for i in range(n):
        Fl, Fr, az, ev = oracle.getrusanovflux(gam, Ql[i], Qr[i], nf[i], sl[i], sr[i])
        orc[0][i], orc[1][i], orc[2][i], orc[3][i] = Fl, Fr, az, ev
    for a, b, c, name in zip(got, ref, orc, ["Fnl", "Fnr", "Az", "eigv"]):
        scale = np.abs(c).max() + 1.0
        assert np.all(np.isfinite(a)), name
        assert np.abs(a - c).max() <= TOL * scale, "%s differs from the oracle" % name
        assert np.abs(a - b).max() <= TOL * scale, "%s differs from getrusanovflux_gpu" % name
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info(0)
    again = _call(L.getrusanovflux_noalloc_gpu, n, gam, *_inputs(8, n, gam))
    free1, _ = torch.cuda.mem_get_info(0)
    assert free1 == free0, "a call changed the device's free memory by %d bytes" % (free0 - free1)
    assert all(np.all(np.isfinite(a)) for a in again)


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
