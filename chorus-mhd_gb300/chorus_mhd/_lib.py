"""ctypes binding of libchorus_gpu.so (the C-ABI declared in include/chorus_gpu.h).

The shared library is built in-tree by ``chorus-mhd_gb300/build.py``.  There is no
CPU fallback: if the library is missing or cannot be loaded, every entry point raises.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libchorus_gpu.so")

c_int, c_double, c_char_p, c_void_p = ctypes.c_int32, ctypes.c_double, ctypes.c_char_p, ctypes.c_void_p
P = ctypes.POINTER
dp, ip = P(c_double), P(c_int)


class ChorusDims(ctypes.Structure):
    _fields_ = [("N", c_int), ("NCELL", c_int), ("NFACE", c_int), ("NINTER", c_int), ("NFREE", c_int),
                ("NPAIR", c_int)]


class ChorusParams(ctypes.Structure):
    _fields_ = [("gam", c_double), ("mu", c_double), ("eta0", c_double), ("DXCYCL", c_double),
                ("DYCYCL", c_double), ("dt", c_double), ("B0x", c_double), ("B0y", c_double),
                ("NCELLGLOB", c_int), ("vismode", c_int), ("ARTIV", c_int), ("k_stage", c_int)]


class ChorusServeRequest(ctypes.Structure):
    _fields_ = [("case_dir", c_char_p), ("arrival_s", c_double), ("end_time", c_double),
                ("Q_out", ctypes.POINTER(c_double)), ("Q_out_count", ctypes.c_int64), ("restart_path", c_char_p)]


class ChorusServeConfig(ctypes.Structure):
    _fields_ = [("device", c_int), ("mode", c_int), ("hbm_budget_bytes", ctypes.c_int64), ("max_active", c_int),
                ("gpu_setup", c_int)]


class ChorusServeResult(ctypes.Structure):
    _fields_ = [("admit_s", c_double), ("finish_s", c_double), ("latency_s", c_double), ("wait_s", c_double),
                ("ctime", c_double), ("dof", ctypes.c_int64), ("steps", c_int), ("status", c_int)]


class ChorusDiag(ctypes.Structure):
    _fields_ = [("iter", c_int), ("pad", c_int), ("ctime", c_double), ("residglob", c_double),
                ("divBglob", c_double), ("eigvmax_g", c_double), ("epsilon0", c_double)]


# name -> (restype, argtypes); every function of include/chorus_gpu.h
SIGNATURES = {
    "chorus_gpu_last_error": (c_char_p, []),
    "chorus_gpu_version": (c_char_p, []),
    "chorus_gpu_device_name": (c_int, [c_int, c_char_p, c_int]),
    "chorus_gpu_bind": (c_int, [P(ChorusDims), ip, ip, ip, ip, ip, ip, dp, dp, dp, dp, dp, dp, dp,
                                P(ChorusParams), c_int, P(c_void_p)]),
    "chorus_gpu_free": (c_int, [c_void_p]),
    "chorus_gpu_set_params": (c_int, [c_void_p, P(ChorusParams)]),
    "chorus_gpu_upload_state": (c_int, [c_void_p, dp]),
    "chorus_gpu_download_state": (c_int, [c_void_p, dp]),
    "chorus_gpu_download_array": (c_int, [c_void_p, c_char_p, dp, ctypes.c_int64]),
    "chorus_gpu_get_eigvmax": (c_int, [c_void_p, dp, dp]),
    "compresid_gpu": (c_int, [c_void_p]),
    "comp_inviscid_flux_gpu": (c_int, [c_void_p]),
    "nablaqsp_gpu": (c_int, [c_void_p, ip, ip]),
    "correct_b_via_curl_az_gpu": (c_int, [c_void_p]),
    "rk_s5p3_gpu": (c_int, [c_void_p, dp]),
    "fivestagerk_gpu": (c_int, [c_void_p, dp]),
    "iterations_gpu": (c_int, [c_void_p, c_int, ip, dp, P(ChorusDiag), c_int, ip]),
    "chorus_gpu_step_host": (c_int, [c_void_p, dp, dp, c_int, ip, dp, P(ChorusDiag), c_int, ip]),
    "getrusanovflux_gpu": (c_int, [c_int, c_double, dp, dp, dp, dp, dp, dp, ip, ip, dp]),
    "getrusanovflux_noalloc_gpu": (c_int, [c_int, c_double, dp, dp, dp, dp, dp, dp, ip, ip, dp]),
    "getifluxvectors_gpu": (c_int, [c_int, c_double, dp, dp, dp]),
    "getvfluxvectors_gpu": (c_int, [c_int, c_double, c_double, c_double, dp, dp, dp, dp]),
    "getvfluxvectors_av_gpu": (c_int, [c_void_p, c_int, dp, dp, dp, dp, ip, ip, ip, ip]),
    "chorus_point_set_params": (c_int, [c_double, c_double, c_double]),
    "getrusanovflux_c": (c_int, [dp, dp, dp, dp, dp, dp, ip, ip, dp, dp]),
    "getifluxvectors_c": (c_int, [dp, dp, dp]),
    "getvfluxvectors_c": (c_int, [dp, dp, dp, dp]),
    "getvfluxvectors_av_c": (c_int, [c_void_p, dp, dp, dp, dp, ip, ip, ip, ip]),
    "chorus_gpu_stream": (c_void_p, [c_void_p]),
    "chorus_gpu_set_option": (c_int, [c_void_p, c_char_p, ctypes.c_int64]),
    "chorus_gpu_get_option": (ctypes.c_int64, [c_void_p, c_char_p]),
    "chorus_gpu_profile_stage": (c_int, [c_void_p, c_int, dp]),
    "chorus_gpu_launch_counts": (c_int, [c_void_p, ip, ip]),
    "chorus_gpu_device_bytes": (ctypes.c_int64, [c_void_p]),
    "chorus_gpu_fp64_fma_peak": (c_int, [c_int, dp, dp]),
    "chorus_batch_create": (c_int, [c_int, P(c_void_p)]),
    "chorus_batch_free": (c_int, [c_void_p]),
    "chorus_batch_add": (c_int, [c_void_p, c_void_p, ip]),
    "chorus_batch_remove": (c_int, [c_void_p, c_int]),
    "chorus_batch_step": (c_int, [c_void_p, c_int]),
    "chorus_batch_sync": (c_int, [c_void_p, ip]),
    "chorus_batch_stream": (c_int, [c_void_p, P(c_void_p)]),
    "chorus_batch_info": (c_int, [c_void_p, ip, ip, ip, P(ctypes.c_int64)]),
    "chorus_serve_run": (c_int, [P(ChorusServeRequest), c_int, P(ChorusServeConfig), P(ChorusServeResult), dp]),
    "chorus_mesh_device_bytes": (ctypes.c_int64, [c_void_p]),
    "chorus_mesh_host_chunks": (c_int, [c_void_p, c_int, ip, ip, ip, ip, ip, ip]),
    "chorus_mesh_load": (c_int, [c_char_p, P(c_void_p)]),
    "chorus_mesh_load_gpu": (c_int, [c_char_p, c_int, P(c_void_p)]),
    "chorus_mesh_free": (c_int, [c_void_p]),
    "chorus_mesh_output_info": (c_int, [c_void_p, ip, ip]),
    "chorus_plot_create": (c_int, [c_void_p, ip, ip, dp, dp, c_int, c_int, dp, c_int, P(c_void_p)]),
    "chorus_plot_create_mesh": (c_int, [c_void_p, c_void_p, c_int, P(c_void_p)]),
    "chorus_plot_free": (c_int, [c_void_p]),
    "chorus_plot_info": (c_int, [c_void_p, P(ctypes.c_int64), P(ctypes.c_int64), ip]),
    "chorus_plot_values": (c_int, [c_void_p, dp, dp, dp, ip, ip]),
    "chorus_plot_filename": (c_int, [c_double, c_char_p, c_int]),
    "chorus_plot_write": (c_int, [c_void_p, c_double, c_char_p, c_char_p, c_int]),
    "chorus_mesh_info": (c_int, [c_void_p, P(ChorusDims), P(ChorusParams), ip, ip]),
    "chorus_mesh_iarray": (ip, [c_void_p, c_char_p, P(ctypes.c_int64)]),
    "chorus_mesh_darray": (dp, [c_void_p, c_char_p, P(ctypes.c_int64)]),
    "chorus_gpu_bind_mesh": (c_int, [c_void_p, c_int, P(c_void_p)]),
    "chorus_initial_state": (c_int, [c_void_p, c_void_p, dp]),
    "chorus_write_restart": (c_int, [c_void_p, c_char_p, c_int, c_double]),
    "chorus_read_restart": (c_int, [c_void_p, c_char_p, ip, dp]),
}

_lib = None


class ChorusError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("chorus error %d: %s" % (code, msg))
        self.code = code


def load(path: str | None = None):
    """Load the in-tree library (raises if it has not been built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError("libchorus_gpu.so is not built (%s); run chorus-mhd_gb300/build.py" % p)
    L = ctypes.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = L
    return L


def check(rc: int):
    if rc != 0:
        raise ChorusError(rc, load().chorus_gpu_last_error().decode())
    return rc
