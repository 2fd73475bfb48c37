"""The integer form of the line operators (chorus-mhd_gb300/csrc/fixdot.cuh), compiled for
the host with UndefinedBehaviorSanitizer (signed overflow of the accumulators, shifts out of
range), against exact rational sums of the same double coefficients and inputs.  CPU only."""
import math
import os
import shutil
import struct
import subprocess
from fractions import Fraction

import numpy as np
import pytest

import oracle
from helpers import make_case

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    if not shutil.which("g++"):
        pytest.skip("no host compiler")
    out = str(tmp_path_factory.mktemp("fixdot") / "fixdot_driver")
    cmd = ["g++", "-std=c++17", "-O1", "-fsanitize=undefined", "-fno-sanitize-recover=all",
           "-I", os.path.join(ROOT, "chorus-mhd_gb300", "csrc"), os.path.join(HERE, "fixdot", "fixdot_driver.cpp"),
           "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0 and "ubsan" in (r.stderr + r.stdout).lower():
        cmd = [c for c in cmd if not c.startswith("-fsanitize") and not c.startswith("-fno-sanitize")]
        r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def apply(driver, tmp_path, C, X):
    C = np.ascontiguousarray(C, np.float64)
    X = np.ascontiguousarray(X, np.float64)
    NO, NI = C.shape
    src, dst = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    with open(src, "wb") as f:
        f.write(struct.pack("<3i", NO, NI, X.shape[0]))
        f.write(C.tobytes())
        f.write(X.tobytes())
    r = subprocess.run([driver, src, dst], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    return np.fromfile(dst, np.float64).reshape(X.shape[0], NO)


def operators():
    """Lmat (flux points from solution points) and Mmat (derivative at the solution points
    from the flux points) as row-major matrices, N = 2..8, from the oracle's setup."""
    import tempfile
    root = tempfile.mkdtemp()
    ops = []
    for N in range(2, 9):
        o = oracle.Oracle(make_case(root, problem="orszag_tang", nx=2, ny=2, N=N, steps=1))
        L = o.array("Lmat").reshape(N, N + 1).T.copy()  # [flux point, solution point]
        M = o.array("Mmat").reshape(N, N + 1).copy()    # [solution point, flux point]
        ops.append(("L%d" % N, L))
        ops.append(("M%d" % N, M))
        o.close()
    return ops


OPS = operators()


def exact(C, x):
    return sum(Fraction(float(c)) * Fraction(float(v)) for c, v in zip(C, x))


def ulp(v):
    return math.ulp(abs(float(v))) if v != 0 else 0.0


def lines(rng, NI, n):
    """Rows of typical and awkward inputs: uniform, smooth profiles, mixed magnitudes,
    near-constant lines (cancellation in a derivative), zeros, signed zeros, subnormals."""
    t = np.linspace(0, 1, NI)
    out = [rng.uniform(-1, 1, NI) for _ in range(n)]
    out += [rng.uniform(-3, 3) + rng.uniform(-1, 1) * t + rng.uniform(-0.5, 0.5) * np.sin(5 * t) for _ in range(n)]
    out += [rng.choice([-1, 1], NI) * 10.0 ** rng.uniform(-20, 20, NI) for _ in range(n)]
    out += [1e5 + 1e-9 * rng.standard_normal(NI) for _ in range(n)]
    z = rng.uniform(-1, 1, NI)
    z[rng.random(NI) < 0.5] = 0.0
    out += [z, np.zeros(NI), -np.zeros(NI), np.full(NI, 5e-324), rng.uniform(-1, 1, NI) * 1e-300,
            2.0 ** rng.integers(-30, 30, NI), rng.uniform(-1, 1, NI) * 1e200]
    return np.array(out)


@pytest.mark.parametrize("name,C", OPS, ids=[o[0] for o in OPS])
def test_error_bound_against_exact_sums(driver, tmp_path, name, C):
    rng = np.random.default_rng(sum(map(ord, name)))
    NO, NI = C.shape
    X = lines(rng, NI, 40)
    Y = apply(driver, tmp_path, C, X)
    cmax = np.abs(C).max()
    worst = 0.0
    for x, y in zip(X, Y):
        xmax = np.abs(x).max()
        for k in range(NO):
            e = exact(C[k], x)
            err = abs(Fraction(float(y[k])) - e)
            tol = 0.5 * ulp(e) + 2.0 ** -55 * xmax * (np.abs(C[k]).sum() + NI * cmax)
            if xmax < 2.0 ** -960:  # results below the normal range flush to zero
                tol = max(tol, 2.0 ** -1022)
            assert float(err) <= tol, (name, x, k, float(y[k]), float(e))
            if xmax >= 2.0 ** -960:
                worst = max(worst, float(err) / (xmax * np.abs(C[k]).sum()))
    assert worst <= 2.0 ** -52  # one rounding of the result, relative to the terms


@pytest.mark.parametrize("name,C", [o for o in OPS if o[0] in ("L5", "M5", "L8", "M8")], ids=["L5", "M5", "L8", "M8"])
def test_as_accurate_as_an_fp64_chain(driver, tmp_path, name, C):
    """On smooth lines the integer form is at least as close to the exact sums as the FP64
    multiply-add chain it replaces; interpolated values (no cancellation) are mostly
    rounded correctly."""
    rng = np.random.default_rng(7)
    NO, NI = C.shape
    t = np.linspace(0, 1, NI)
    X = np.array([rng.uniform(0.5, 3) + rng.uniform(-1, 1) * np.sin(3 * t + rng.uniform(0, 6)) for _ in range(300)])
    Y = apply(driver, tmp_path, C, X)
    err_fix = err_fp = 0.0
    correct = 0
    for x, y in zip(X, Y):
        for k in range(NO):
            e = exact(C[k], x)
            acc = 0.0
            for c, v in zip(C[k], x):
                acc = acc + float(c) * float(v)
            err_fix += float(abs(Fraction(float(y[k])) - e))
            err_fp += float(abs(Fraction(acc) - e))
            correct += float(y[k]) == float(e)
    assert err_fix <= err_fp
    if name.startswith("L"):
        assert correct >= 0.9 * X.shape[0] * NO


def apply_mirror(driver, tmp_path, C, X, sigma):
    """The mirror form (what the stage kernels run): results, and the effective operator
    as exact rationals c / 2^S."""
    C = np.ascontiguousarray(C, np.float64)
    X = np.ascontiguousarray(X, np.float64)
    NO, NI = C.shape
    src, dst, opf = str(tmp_path / "in.bin"), str(tmp_path / "out.bin"), str(tmp_path / "op.bin")
    with open(src, "wb") as f:
        f.write(struct.pack("<3i", NO, NI, X.shape[0]))
        f.write(C.tobytes())
        f.write(X.tobytes())
    r = subprocess.run([driver, src, dst, str(sigma), opf], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    raw = open(opf, "rb").read()
    S = struct.unpack("<i", raw[:4])[0]
    ce = np.frombuffer(raw[4:], np.int64).reshape(NO, NI)
    return np.fromfile(dst, np.float64).reshape(X.shape[0], NO), S, ce


MIRROR = [(name, C, 1 if name.startswith("L") else -1) for name, C in OPS]


@pytest.mark.parametrize("name,C,sigma", MIRROR, ids=[o[0] for o in MIRROR])
def test_mirror_form(driver, tmp_path, name, C, sigma):
    """The mirror form pairs outputs k and NO-1-k on half the multiply-adds: its effective
    operator is exactly (anti)symmetric, lies within 1.5 units of 2^-S plus half the given
    operator's own mirror asymmetry (the rounding of its construction) of every coefficient,
    and its results keep the error bound of the plain form against exact sums of it."""
    rng = np.random.default_rng(sum(map(ord, name)) + 1)
    NO, NI = C.shape
    X = lines(rng, NI, 40)
    Y, S, ce = apply_mirror(driver, tmp_path, C, X, sigma)
    assert np.array_equal(ce[::-1, ::-1], sigma * ce)
    unit = Fraction(1, 2 ** S)
    asym = np.abs(C - sigma * C[::-1, ::-1]) / 2
    assert asym.max() <= 4e-15 * np.abs(C).max()
    Ce = [[Fraction(int(ce[k, j])) * unit for j in range(NI)] for k in range(NO)]
    for k in range(NO):
        for j in range(NI):
            assert abs(Ce[k][j] - Fraction(float(C[k, j]))) <= Fraction(3, 2) * unit + Fraction(float(asym[k, j]))
    cabs = [sum(abs(float(c)) for c in row) for row in Ce]
    cmax = max(max(abs(float(c)) for c in row) for row in Ce)
    for x, y in zip(X, Y):
        xmax = np.abs(x).max()
        for k in range(NO):
            e = sum(c * Fraction(float(v)) for c, v in zip(Ce[k], x))
            err = abs(Fraction(float(y[k])) - e)
            tol = 0.5 * ulp(e) + 2.0 ** -55 * xmax * (cabs[k] + NI * cmax)
            if xmax < 2.0 ** -960:
                tol = max(tol, 2.0 ** -1022)
            assert float(err) <= tol, (name, x, k, float(y[k]), float(e))


def test_special_lines(driver, tmp_path):
    C = dict(OPS)["L5"]
    X = np.array([[np.nan, 1, 2, 3, 4], [np.inf, 0, 0, 0, 0], [1e290, 1, 1, 1, 1], [0.0] * 5, [-0.0] * 5,
                  [1.0, 1.0, 1.0, 1.0, 1.0]])
    Y = apply(driver, tmp_path, C, X)
    assert np.isnan(Y[:3]).all()  # outside the integer form: the kernels keep FP64 for these
    assert (Y[3:5] == 0).all() and not np.signbit(Y[3:5]).any()
    # a constant line interpolates to the constant (rows of Lmat sum to 1 within rounding)
    assert np.allclose(Y[5], 1.0, rtol=0, atol=4e-16)

