"""Host-side mirror of the reference's hot-path interface.

``Mesh`` wraps the library's setup chain (QUAD.INP + .CEL/.VRT/.BND -> the reference's
maps and geometry).  ``Solver`` binds a mesh to one GPU and exposes the reference
routines by their names -- ``compresid``, ``comp_inviscid_flux``, ``nablaQsp``,
``correct_B_via_curl_Az``, ``RK_S5P3``, ``FiveStageRk``, ``iterations`` -- operating on
the device-resident state.  Arrays come back in the reference's Fortran layout,
flattened (first index fastest).
"""
from __future__ import annotations

import ctypes
import os
import weakref

import numpy as np

from . import _lib
from ._lib import ChorusDiag, ChorusDims, ChorusParams, check


def _dp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))


class Mesh:
    """The reference's setup chain for one case directory (readinput ... calcjacob).

    With `device` given, the maps and the geometry are built on that GPU
    (chorus_mesh_load_gpu; the same arrays bit for bit)."""

    def __init__(self, case_dir: str, device: int | None = None):
        self.L = _lib.load()
        h = ctypes.c_void_p()
        if device is None:
            check(self.L.chorus_mesh_load(case_dir.encode(), ctypes.byref(h)))
        else:
            check(self.L.chorus_mesh_load_gpu(case_dir.encode(), int(device), ctypes.byref(h)))
        self._h = h
        self.case_dir = case_dir
        self.dims = ChorusDims()
        self.params = ChorusParams()
        mi, pb = ctypes.c_int32(), ctypes.c_int32()
        check(self.L.chorus_mesh_info(self._h, ctypes.byref(self.dims), ctypes.byref(self.params),
                                      ctypes.byref(mi), ctypes.byref(pb)))
        self.maxiter, self.problem = mi.value, pb.value
        nre, nw = ctypes.c_int32(), ctypes.c_int32()
        check(self.L.chorus_mesh_output_info(self._h, ctypes.byref(nre), ctypes.byref(nw)))
        self.nre, self.nwrite = nre.value, nw.value

    @property
    def N(self):
        return self.dims.N

    @property
    def ncell(self):
        return self.dims.NCELL

    def iarray(self, name) -> np.ndarray:
        n = ctypes.c_int64()
        p = self.L.chorus_mesh_iarray(self._h, name.encode(), ctypes.byref(n))
        if not p:
            raise KeyError(name)
        return np.ctypeslib.as_array(p, shape=(n.value,)).copy() if n.value else np.zeros(0, np.int32)

    def darray(self, name) -> np.ndarray:
        n = ctypes.c_int64()
        p = self.L.chorus_mesh_darray(self._h, name.encode(), ctypes.byref(n))
        if not p:
            raise KeyError(name)
        return np.ctypeslib.as_array(p, shape=(n.value,)).copy() if n.value else np.zeros(0)

    def close(self):
        if getattr(self, "_h", None):
            self.L.chorus_mesh_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Plot:
    """Plot output of one solve (tecplotter2dsetup / tecplotter2d / tecpost_parallel):
    the plot-node topology is built once; values() evaluates the nodes on the device,
    write() also writes the reference's Tecplot binary file.  With AV on, the solve's
    latest step (or compresid) must have run with the plot_sensor option set, which
    records the sensor behind etaAV (Solver.run does this for its output steps)."""

    def __init__(self, solver: "Solver", nre: int = 0):
        self.L = solver.L
        self.solver = solver
        h = ctypes.c_void_p()
        check(self.L.chorus_plot_create_mesh(solver._ctx, solver.mesh._h, int(nre), ctypes.byref(h)))
        self._h = h
        if not hasattr(solver, "_plots"):
            solver._plots = weakref.WeakSet()
        solver._plots.add(self)
        n, c, w = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int32()
        check(self.L.chorus_plot_info(self._h, ctypes.byref(n), ctypes.byref(c), ctypes.byref(w)))
        self.nodes, self.cells, self.warned = n.value, c.value, bool(w.value)

    def values(self) -> dict:
        X = np.empty(2 * self.nodes)
        Q = np.empty(9 * self.nodes)
        AV = np.empty(2 * self.nodes)
        con = np.empty(4 * self.cells, np.int32)
        fac = np.empty(self.nodes, np.int32)
        check(self.L.chorus_plot_values(self._h, _dp(X), _dp(Q), _dp(AV), _ip(con), _ip(fac)))
        return dict(plotX=X, plotQ=Q, plotAV=AV, connec_c2n=con, gnode_factor=fac)

    def write(self, directory: str, ctime: float | None = None) -> str:
        out = ctypes.create_string_buffer(4096)
        t = self.solver.ctime if ctime is None else float(ctime)
        check(self.L.chorus_plot_write(self._h, t, directory.encode(), out, 4096))
        return out.value.decode()

    def close(self):
        if getattr(self, "_h", None):
            self.L.chorus_plot_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def plot_filename(ctime: float) -> str:
    buf = ctypes.create_string_buffer(64)
    check(_lib.load().chorus_plot_filename(float(ctime), buf, 64))
    return buf.value.decode()


def device_name(device: int = 0) -> str:
    buf = ctypes.create_string_buffer(256)
    check(_lib.load().chorus_gpu_device_name(int(device), buf, 256))
    return buf.value.decode()


class Solver:
    """One solve resident on one GPU; method names follow the reference routines.

    tuned=True applies the autotuned launch shapes of this GPU model, if a table exists
    (chorus_mhd.autotune)."""

    def __init__(self, mesh: Mesh, device: int = 0, initial_state: bool = True, tuned: bool = True):
        self.L = _lib.load()
        self.mesh = mesh
        ctx = ctypes.c_void_p()
        check(self.L.chorus_gpu_bind_mesh(mesh._h, device, ctypes.byref(ctx)))
        self._ctx = ctx
        self.N, self.ncell = mesh.N, mesh.ncell
        self.tuned = False
        if tuned:
            from . import autotune
            self.tuned = autotune.apply(self, autotune.load(device_name(device)))
        self.nq = 9 * self.N * self.N * self.ncell
        self.iter = 0
        self.ctime = 0.0
        self.diagnostics: list[dict] = []
        if initial_state:
            self.set_initial_state()

    # ---- state
    def set_initial_state(self) -> np.ndarray:
        Q = np.empty(self.nq)
        check(self.L.chorus_initial_state(self.mesh._h, self._ctx, _dp(Q)))
        self.iter, self.ctime = 0, 0.0
        return Q

    def upload(self, Q: np.ndarray):
        Q = np.ascontiguousarray(Q, np.float64).reshape(-1)
        assert Q.size == self.nq
        check(self.L.chorus_gpu_upload_state(self._ctx, _dp(Q)))

    def state(self, out: np.ndarray | None = None) -> np.ndarray:
        """Download Q (the reference's Q(9,N,N,NCELL), flat); into `out` if given
        (e.g. a pinned buffer, so the copy runs at full link speed)."""
        Q = np.empty(self.nq) if out is None else out
        assert Q.dtype == np.float64 and Q.flags.c_contiguous and Q.size == self.nq
        check(self.L.chorus_gpu_download_state(self._ctx, _dp(Q)))
        return Q

    def array(self, name: str, count: int) -> np.ndarray:
        out = np.empty(count)
        check(self.L.chorus_gpu_download_array(self._ctx, name.encode(), _dp(out), count))
        return out

    def eigvmax(self):
        a, b = ctypes.c_double(), ctypes.c_double()
        check(self.L.chorus_gpu_get_eigvmax(self._ctx, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def set_params(self, **kw):
        p = ChorusParams.from_buffer_copy(self.mesh.params)
        for k, v in kw.items():
            setattr(p, k, v)
        check(self.L.chorus_gpu_set_params(self._ctx, ctypes.byref(p)))

    # ---- reference routines
    def compresid(self):
        check(self.L.compresid_gpu(self._ctx))

    def comp_inviscid_flux(self):
        check(self.L.comp_inviscid_flux_gpu(self._ctx))

    def nablaQsp(self, v_sta: int, v_end: int):
        a, b = ctypes.c_int32(v_sta), ctypes.c_int32(v_end)
        check(self.L.nablaqsp_gpu(self._ctx, ctypes.byref(a), ctypes.byref(b)))

    def correct_B_via_curl_Az(self):
        check(self.L.correct_b_via_curl_az_gpu(self._ctx))

    def RK_S5P3(self):
        t = ctypes.c_double(self.ctime)
        check(self.L.rk_s5p3_gpu(self._ctx, ctypes.byref(t)))
        self.ctime = t.value

    def FiveStageRk(self):
        t = ctypes.c_double(self.ctime)
        check(self.L.fivestagerk_gpu(self._ctx, ctypes.byref(t)))
        self.ctime = t.value

    def iterations(self, nsteps: int) -> list[dict]:
        """nsteps of iterations.f90:19-87 (RK step, CT projection, norms every 10)."""
        it = ctypes.c_int32(self.iter)
        t = ctypes.c_double(self.ctime)
        cap = nsteps // 10 + 2
        recs = (ChorusDiag * cap)()
        nd = ctypes.c_int32(0)
        check(self.L.iterations_gpu(self._ctx, int(nsteps), ctypes.byref(it), ctypes.byref(t), recs, cap,
                                    ctypes.byref(nd)))
        self.iter, self.ctime = it.value, t.value
        out = [dict(iter=r.iter, ctime=r.ctime, residglob=r.residglob, divBglob=r.divBglob,
                    eigvmax_g=r.eigvmax_g, epsilon0=r.epsilon0) for r in recs[: min(nd.value, cap)]]
        self.diagnostics.extend(out)
        return out

    def step_host(self, Qin: np.ndarray | None, Qout: np.ndarray | None, nsteps: int = 1) -> list[dict]:
        """nsteps of iterations on a host-resident state: Q is uploaded from Qin before the
        first step and downloaded into Qout after the last (chorus_gpu_step_host; the copies
        overlap the kernels chunk by chunk, fully so for pinned arrays)."""
        for a in (Qin, Qout):
            if a is not None and (a.dtype != np.float64 or a.size != self.nq or not a.flags.c_contiguous):
                raise ValueError("Q arrays must be contiguous float64 of %d elements" % self.nq)
        it = ctypes.c_int32(self.iter)
        t = ctypes.c_double(self.ctime)
        cap = nsteps // 10 + 2
        recs = (ChorusDiag * cap)()
        nd = ctypes.c_int32(0)
        check(self.L.chorus_gpu_step_host(self._ctx, _dp(Qin) if Qin is not None else None,
                                          _dp(Qout) if Qout is not None else None, int(nsteps), ctypes.byref(it),
                                          ctypes.byref(t), recs, cap, ctypes.byref(nd)))
        self.iter, self.ctime = it.value, t.value
        out = [dict(iter=r.iter, ctime=r.ctime, residglob=r.residglob, divBglob=r.divBglob,
                    eigvmax_g=r.eigvmax_g, epsilon0=r.epsilon0) for r in recs[: min(nd.value, cap)]]
        self.diagnostics.extend(out)
        return out

    def run(self, maxiter: int | None = None, out_dir: str | None = None, nwrite: int | None = None,
            nre: int = 0) -> list[dict]:
        """The iteration loop of iterations.f90:19-87 up to MAXITER, with its output
        schedule (:80-84): after step iter, when mod(iter, nwrite) == 1 or iter >=
        MAXITER, the Tecplot file and the restart file restart.<iter %08d>.dat
        (write_data.f90:44) go to out_dir (no output when out_dir is None)."""
        maxiter = self.mesh.maxiter if maxiter is None else int(maxiter)
        nwrite = self.mesh.nwrite if nwrite is None else int(nwrite)
        plot = Plot(self, nre) if out_dir else None
        recs = []
        try:
            while self.iter < maxiter:
                nxt = maxiter
                if out_dir and nwrite > 1:
                    # next iter with mod(iter, nwrite) == 1
                    k = self.iter + 1
                    r = (1 - k) % nwrite
                    nxt = min(maxiter, k + r)
                if out_dir:
                    # the step before an output records the sensor that the plot's etaAV needs
                    if nxt - self.iter > 1:
                        recs += self.iterations(nxt - self.iter - 1)
                    self.set_option("plot_sensor", 1)
                    recs += self.iterations(1)
                    self.set_option("plot_sensor", 0)
                else:
                    recs += self.iterations(nxt - self.iter)
                if out_dir and ((nwrite > 1 and self.iter % nwrite == 1) or self.iter >= maxiter):
                    plot.write(out_dir)
                    self.write_restart(os.path.join(out_dir, "restart.%08d.dat" % self.iter))
        finally:
            if plot:
                plot.close()
        return recs

    def plot(self, nre: int = 0) -> "Plot":
        """Plot output object for this solve (NRE from the case file when nre <= 0)."""
        return Plot(self, nre)

    # ---- runtime helpers
    def set_option(self, name: str, value: int):
        check(self.L.chorus_gpu_set_option(self._ctx, name.encode(), int(value)))

    def get_option(self, name: str) -> int:
        return int(self.L.chorus_gpu_get_option(self._ctx, name.encode()))

    def stream_handle(self) -> int:
        """cudaStream_t of this solve (for events / ordering)."""
        return int(self.L.chorus_gpu_stream(self._ctx) or 0)

    def profile_stage(self, reps: int = 5) -> list:
        """Mean durations (ms) of E1, F1, E2, F2, E3 and of a whole stage."""
        ms = np.zeros(6)
        check(self.L.chorus_gpu_profile_stage(self._ctx, int(reps), _dp(ms)))
        return ms.tolist()

    def launch_counts(self):
        a, b = ctypes.c_int32(), ctypes.c_int32()
        check(self.L.chorus_gpu_launch_counts(self._ctx, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def device_bytes(self) -> int:
        return int(self.L.chorus_gpu_device_bytes(self._ctx))

    def write_restart(self, path: str):
        check(self.L.chorus_write_restart(self._ctx, path.encode(), self.iter, self.ctime))

    def read_restart(self, path: str):
        it, t = ctypes.c_int32(), ctypes.c_double()
        check(self.L.chorus_read_restart(self._ctx, path.encode(), ctypes.byref(it), ctypes.byref(t)))
        self.iter, self.ctime = it.value, t.value

    def close(self):
        for p in list(getattr(self, "_plots", ())):  # plots refer to the context
            p.close()
        if getattr(self, "_ctx", None):
            self.L.chorus_gpu_free(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def reference_layout_sizes(N: int, ncell: int) -> dict:
    """Element counts of the reference's work arrays (for download_array)."""
    ns, nf = N * N * ncell, (N + 1) * N * ncell
    return {"Q": 9 * ns, "resid": 9 * ns, "F1": 8 * nf, "G2": 8 * nf, "Qvfi": 9 * nf, "Qvfj": 9 * nf,
            "Azfi": nf, "Azfj": nf, "nablaQs": 18 * ns, "nablaQvfi": 18 * nf, "nablaQvfj": 18 * nf,
            "nablaAs": 2 * ns, "muAVfi": 18 * ncell, "muAVfj": 18 * ncell, "SM_IND1": ncell}
