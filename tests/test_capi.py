"""The C-ABI library loads and exports every entry point that include/chorus_gpu.h
declares (no kernels are launched here)."""
import os
import re
import subprocess

from chorus_mhd import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for h in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if h.endswith(".h"):
            src = open(os.path.join(ROOT, "include", h)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names += re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b([a-z_][a-z0-9_]*)\s*\(", src, flags=re.M)
    return sorted(set(n for n in names if n not in ("if", "for", "while")))


def test_header_declares_the_drop_ins():
    names = declared_functions()
    for n in ["compresid_gpu", "rk_s5p3_gpu", "fivestagerk_gpu", "correct_b_via_curl_az_gpu", "nablaqsp_gpu",
              "comp_inviscid_flux_gpu", "iterations_gpu", "getrusanovflux_gpu", "chorus_gpu_bind"]:
        assert n in names


def test_library_exports_every_declared_symbol():
    L = _lib.load()
    names = declared_functions()
    assert len(names) > 20
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(ln.split()[-1] for ln in out.splitlines() if ln.strip())
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    for n in names:
        getattr(L, n)
    assert set(names) <= set(_lib.SIGNATURES)


def test_version_and_error_strings():
    L = _lib.load()
    assert b"sm_103a" in L.chorus_gpu_version()
    assert isinstance(L.chorus_gpu_last_error(), bytes)
