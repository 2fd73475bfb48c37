"""Build libchorus_gpu.so for sm_103a (in-tree, no cmake).

Every CUDA translation unit is compiled by nvcc with
``-gencode arch=compute_103a,code=sm_103a -lineinfo -O3``; host code is compiled with
``-ffp-contract=off`` so the host-side geometry (metrics, normals, Lagrange operators)
follows the reference's evaluation order bit for bit on both x86-64 and aarch64.
Translation units compile in parallel; outputs go to ``_build/`` and the shared
library to ``chorus_mhd/_lib/``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "chorus_mhd", "_lib")
LIB = os.path.join(LIBDIR, "libchorus_gpu.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-lineinfo", "-O3", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
                     "-Xcompiler", "-ffp-contract=off", "-I" + CSRC, "-I" + INCLUDE]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I" + CSRC, "-I" + INCLUDE]


def _nvcc():
    for p in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if p and os.path.exists(p):
            return p
    raise RuntimeError("nvcc not found")


def _cuda_home(nvcc):
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def sources():
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    cpp = sorted(f for f in os.listdir(CSRC) if f.endswith(".cpp"))
    return cu, cpp


def _newer(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, jobs: int | None = None) -> str:
    nvcc = _nvcc()
    cuda = _cuda_home(nvcc)
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(INCLUDE, "chorus_gpu.h"))
    cu, cpp = sources()
    cmds, objs = [], []
    for f in cu:
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, f + ".o")
        objs.append(obj)
        if force or _newer(obj, [src] + headers):
            cmds.append([nvcc] + NVCC_FLAGS + ["-c", src, "-o", obj])
    for f in cpp:
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, f + ".o")
        objs.append(obj)
        if force or _newer(obj, [src] + headers):
            cmds.append(["g++"] + CXX_FLAGS + ["-I" + os.path.join(cuda, "include"), "-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
        if verbose and (r.stdout or r.stderr):
            sys.stderr.write(r.stdout + r.stderr)
        return r

    if cmds:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(len(cmds), os.cpu_count() or 4)) as ex:
            list(ex.map(run, cmds))
    if force or cmds or _newer(LIB, objs):
        run([nvcc] + ARCH + ["-shared", "-o", LIB + ".tmp"] + objs + ["-lcudart"])
        os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
