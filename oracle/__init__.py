"""CPU oracle for the CHORUS-MHD residual-and-time-step path (test infrastructure).

A plain-C restatement of the reference Fortran (``chorus_oracle.c``), compiled with
``gcc -O2 -ffp-contract=off`` (no fast-math), wrapped here with ctypes.  Only the
tests, ``__graft_entry__.smoke()`` (as the checker) and ``bench.py``'s CPU-baseline
leg may use it; the product library never does.

Parity status: pinned by analytic known answers only (the reference ships no golden
data and no Fortran compiler is available); UNPINNED against the reference binary.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liborc.so")
SRC = os.path.join(HERE, "chorus_oracle.c")


def build(force: bool = False) -> str:
    """Compile the oracle into oracle/_build/liborc.so (OpenMP-enabled)."""
    os.makedirs(BUILD, exist_ok=True)
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= os.path.getmtime(SRC)
            and os.path.getmtime(LIB) >= os.path.getmtime(os.path.join(HERE, "chorus_oracle.h"))):
        return LIB
    cmd = ["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared",
           "-std=c99", "-Wall", "-Wno-unused-variable", "-Wno-unused-but-set-variable",
           "-o", LIB + ".tmp", SRC, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        vp, cp, ip, dp = ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double)
        L.orc_load.restype = vp
        L.orc_load.argtypes = [cp, cp, ip]
        L.orc_free.argtypes = [vp]
        L.orc_geti.restype = ip
        L.orc_geti.argtypes = [vp, cp]
        L.orc_getd.restype = ctypes.c_double
        L.orc_getd.argtypes = [vp, cp]
        L.orc_setd.argtypes = [vp, cp, ctypes.c_double]
        L.orc_seti.argtypes = [vp, cp, ip]
        L.orc_darray.restype = dp
        L.orc_darray.argtypes = [vp, cp, ctypes.POINTER(ctypes.c_int64)]
        L.orc_iarray.restype = ctypes.POINTER(ctypes.c_int32)
        L.orc_iarray.argtypes = [vp, cp, ctypes.POINTER(ctypes.c_int64)]
        for f in ("orc_compresid", "orc_compflux", "orc_comp_inviscid_flux", "orc_correct_B_via_curl_Az",
                  "orc_rk_s5p3", "orc_fivestagerk"):
            getattr(L, f).argtypes = [vp]
        L.orc_nablaQsp.argtypes = [vp, ip, ip]
        L.orc_step.restype = ip
        L.orc_step.argtypes = [vp, dp, dp]
        L.orc_run.argtypes = [vp, ip]
        L.orc_write_restart.argtypes = [vp, cp]
        L.orc_read_restart.argtypes = [vp, cp]
        L.orc_set_threads.argtypes = [ip]
        L.orc_set_threads.restype = ip
        L.orc_getrusanovflux.argtypes = [ctypes.c_double, dp, dp, dp, dp, dp, dp, ip, ip, dp, dp]
        L.orc_getifluxvectors.argtypes = [ctypes.c_double, dp, dp, dp]
        L.orc_getvfluxvectors.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_double, dp, dp, dp, dp]
        L.orc_plot_setup.argtypes = [vp, ip]
        L.orc_plot_eval.argtypes = [vp]
        L.orc_plot_filename.argtypes = [ctypes.c_double, cp, ip]
        L.orc_plot_write.argtypes = [vp, ctypes.c_double, cp]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class Oracle:
    """One reference-state instance (the setup2d module globals) loaded from a case dir."""

    def __init__(self, case_dir: str, threads: int = 1):
        L = lib()
        L.orc_set_threads(threads)
        err = ctypes.create_string_buffer(512)
        self._h = L.orc_load(case_dir.encode(), err, 512)
        if not self._h:
            raise RuntimeError("oracle load failed: " + err.value.decode())
        self.L = L

    def close(self):
        if getattr(self, "_h", None):
            self.L.orc_free(self._h)
            self._h = None

    __del__ = close

    def geti(self, name):
        return self.L.orc_geti(self._h, name.encode())

    def getd(self, name):
        return self.L.orc_getd(self._h, name.encode())

    def setd(self, name, v):
        if self.L.orc_setd(self._h, name.encode(), float(v)) != 0:
            raise KeyError(name)

    def seti(self, name, v):
        if self.L.orc_seti(self._h, name.encode(), int(v)) != 0:
            raise KeyError(name)

    def array(self, name) -> np.ndarray:
        """Live view (no copy) of a named array in the reference (Fortran) layout, flat."""
        n = ctypes.c_int64()
        p = self.L.orc_darray(self._h, name.encode(), ctypes.byref(n))
        if p:
            return np.ctypeslib.as_array(p, shape=(n.value,)) if n.value else np.zeros(0)
        p = self.L.orc_iarray(self._h, name.encode(), ctypes.byref(n))
        if p:
            return np.ctypeslib.as_array(p, shape=(n.value,)) if n.value else np.zeros(0, np.int32)
        raise KeyError(name)

    def compresid(self):
        self.L.orc_compresid(self._h)

    def plot_setup(self, nre: int) -> int:
        """tecplotter2dsetup; returns 1 where the reference would print its warnings."""
        return self.L.orc_plot_setup(self._h, int(nre))

    def plot_eval(self):
        if self.L.orc_plot_eval(self._h) != 0:
            raise RuntimeError("plot_setup first")

    def plot_write(self, ctime: float, path: str):
        if self.L.orc_plot_write(self._h, float(ctime), path.encode()) != 0:
            raise RuntimeError("cannot write " + path)

    def compflux(self):
        self.L.orc_compflux(self._h)

    def comp_inviscid_flux(self):
        self.L.orc_comp_inviscid_flux(self._h)

    def nablaQsp(self, v_sta, v_end):
        self.L.orc_nablaQsp(self._h, v_sta, v_end)

    def correct_B_via_curl_Az(self):
        self.L.orc_correct_B_via_curl_Az(self._h)

    def rk_s5p3(self):
        self.L.orc_rk_s5p3(self._h)

    def fivestagerk(self):
        self.L.orc_fivestagerk(self._h)

    def step(self):
        r = ctypes.c_double(np.nan)
        d = ctypes.c_double(np.nan)
        did = self.L.orc_step(self._h, ctypes.byref(r), ctypes.byref(d))
        return (r.value, d.value) if did else None

    def run(self, n):
        self.L.orc_run(self._h, int(n))

    def write_restart(self, path):
        return self.L.orc_write_restart(self._h, path.encode())

    def read_restart(self, path):
        return self.L.orc_read_restart(self._h, path.encode())


def getrusanovflux(gam, Qfl, Qfr, normf, sign_l, sign_r):
    L = lib()
    Qfl = np.ascontiguousarray(Qfl, np.float64)
    Qfr = np.ascontiguousarray(Qfr, np.float64)
    normf = np.ascontiguousarray(normf, np.float64)
    Fnl = np.zeros(8)
    Fnr = np.zeros(8)
    Az = ctypes.c_double()
    ev = ctypes.c_double()
    em = ctypes.c_double(0.0)
    L.orc_getrusanovflux(gam, _dp(Qfl), _dp(Qfr), _dp(Fnl), _dp(Fnr), ctypes.byref(Az), _dp(normf),
                         int(sign_l), int(sign_r), ctypes.byref(ev), ctypes.byref(em))
    return Fnl, Fnr, Az.value, ev.value


def getifluxvectors(gam, Qi):
    L = lib()
    Qi = np.ascontiguousarray(Qi[:8], np.float64)
    F = np.zeros(8)
    G = np.zeros(8)
    L.orc_getifluxvectors(gam, _dp(Qi), _dp(F), _dp(G))
    return F, G


def getvfluxvectors(gam, mu, eta0, Qv, nablaQ):
    """nablaQ: (9,2) in Fortran order, i.e. flat [k + 9*d]."""
    L = lib()
    Qv = np.ascontiguousarray(Qv, np.float64)
    nq = np.ascontiguousarray(nablaQ, np.float64).reshape(-1)
    Fv = np.zeros(9)
    Gv = np.zeros(9)
    L.orc_getvfluxvectors(gam, mu, eta0, _dp(Qv), _dp(nq), _dp(Fv), _dp(Gv))
    return Fv, Gv


def plot_filename(ctime: float) -> str:
    """The reference's plot file name for solution time ctime (tecplotter.f90:179-180)."""
    b = ctypes.create_string_buffer(64)
    lib().orc_plot_filename(float(ctime), b, 64)
    return b.value.decode()
