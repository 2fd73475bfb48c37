"""Host code under AddressSanitizer + UndefinedBehaviorSanitizer (CPU): the oracle through
setup, steps, plot output and restart, and the product's host setup chain, on small meshes of
every boundary kind.  compute-sanitizer is not available for the device code; its bounds are
checked by reading the index arithmetic and by the element-wise parity tests."""
import os
import shutil
import subprocess

import pytest

from helpers import make_case

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SAN = ["-fsanitize=address,undefined", "-fno-sanitize-recover=all", "-fno-omit-frame-pointer", "-g", "-O1"]
CASES = [dict(problem="orszag_tang", nx=3, ny=3, N=2), dict(problem="orszag_tang", nx=4, ny=3, N=5, jitter=0.15, seed=2),
         dict(problem="rotor", nx=4, ny=4, N=3, jitter=0.1, seed=3), dict(problem="alfven", nx=3, ny=4, N=4)]


def _cuda_include():
    for p in (os.environ.get("CUDA_HOME", ""), "/usr/local/cuda"):
        if p and os.path.exists(os.path.join(p, "include", "cuda_runtime.h")):
            return os.path.join(p, "include")
    return None


@pytest.fixture(scope="module")
def drivers(tmp_path_factory):
    if not shutil.which("gcc") or not shutil.which("g++"):
        pytest.skip("no host compiler")
    out = tmp_path_factory.mktemp("san")
    orc = str(out / "oracle_driver")
    r = subprocess.run(["gcc"] + SAN + ["-ffp-contract=off", "-I", os.path.join(ROOT, "oracle"),
                                        os.path.join(HERE, "sanitize", "oracle_driver.c"),
                                        os.path.join(ROOT, "oracle", "chorus_oracle.c"), "-lm", "-o", orc],
                       capture_output=True, text=True)
    if r.returncode != 0 and "asan" in (r.stderr + r.stdout).lower():
        pytest.skip("AddressSanitizer runtime unavailable")
    assert r.returncode == 0, r.stderr
    mesh = None
    inc = _cuda_include()
    if inc:
        mesh = str(out / "mesh_driver")
        csrc = os.path.join(ROOT, "chorus-mhd_gb300", "csrc")
        r = subprocess.run(["g++"] + SAN + ["-std=c++17", "-ffp-contract=off", "-I", csrc, "-I",
                                            os.path.join(ROOT, "include"), "-I", inc,
                                            os.path.join(HERE, "sanitize", "mesh_driver.cpp"),
                                            os.path.join(csrc, "mesh.cpp"), "-o", mesh], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
    return orc, mesh, str(out)


@pytest.mark.parametrize("case", CASES, ids=lambda c: "%s_%dx%d_N%d" % (c["problem"], c["nx"], c["ny"], c["N"]))
def test_oracle_clean_under_sanitizers(drivers, case_root, case):
    orc, _, scratch = drivers
    d = make_case(case_root, **case)
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=0", UBSAN_OPTIONS="print_stacktrace=1")
    r = subprocess.run([orc, d, scratch, "4"], capture_output=True, text=True, env=env, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("ok"), r.stdout


@pytest.mark.parametrize("case", CASES, ids=lambda c: "%s_%dx%d_N%d" % (c["problem"], c["nx"], c["ny"], c["N"]))
def test_host_setup_clean_under_sanitizers(drivers, case_root, case):
    _, mesh, _ = drivers
    if mesh is None:
        pytest.skip("CUDA headers not found")
    d = make_case(case_root, **case)
    r = subprocess.run([mesh, d], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("ok"), r.stdout
