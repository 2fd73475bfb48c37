"""Batched form: many independent solves advanced together on one GPU.

``Batch`` holds bound ``Solver`` objects (any N, mesh size, problem, dt) and advances
all of them with one persistent launch per pass (libchorus_gpu ``chorus_batch_*``).
Each solve keeps its own resident state; results are the same as stepping it alone.
"""
from __future__ import annotations

import ctypes

from . import _lib
from ._lib import check


class Batch:
    def __init__(self, device: int = 0):
        self.L = _lib.load()
        h = ctypes.c_void_p()
        check(self.L.chorus_batch_create(int(device), ctypes.byref(h)))
        self._h = h
        self.solvers: dict[int, object] = {}

    def add(self, solver) -> int:
        slot = ctypes.c_int32()
        check(self.L.chorus_batch_add(self._h, solver._ctx, ctypes.byref(slot)))
        self.solvers[slot.value] = solver
        return slot.value

    def remove(self, slot: int):
        check(self.L.chorus_batch_remove(self._h, int(slot)))
        self.solvers.pop(slot, None)

    def step(self, nsteps: int = 1):
        """Enqueue nsteps time steps of every solve (asynchronous)."""
        check(self.L.chorus_batch_step(self._h, int(nsteps)))
        for s in self.solvers.values():
            s.iter += nsteps
            s.ctime += nsteps * s.mesh.params.dt

    def sync(self):
        bad = ctypes.c_int32(-1)
        check(self.L.chorus_batch_sync(self._h, ctypes.byref(bad)))

    def stream_handle(self) -> int:
        p = ctypes.c_void_p()
        check(self.L.chorus_batch_stream(self._h, ctypes.byref(p)))
        return int(p.value or 0)

    def info(self) -> dict:
        n, ct, ft, d = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int64()
        check(self.L.chorus_batch_info(self._h, ctypes.byref(n), ctypes.byref(ct), ctypes.byref(ft), ctypes.byref(d)))
        return {"solves": n.value, "cell_tiles": ct.value, "face_tiles": ft.value, "dofs": d.value}

    def close(self):
        if getattr(self, "_h", None):
            self.L.chorus_batch_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
