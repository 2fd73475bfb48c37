"""Shared test helpers: synthetic cases and norm-wise comparisons."""
import os

import numpy as np

from chorus_mhd import meshgen

_CACHE = {}


def make_case(root, **kw):
    """Write (once per session) a case for CaseSpec(**kw) under root; return its dir."""
    key = tuple(sorted(kw.items()))
    if key not in _CACHE:
        name = "_".join("%s%s" % (k, v) for k, v in sorted(kw.items())).replace(".", "p")
        d = os.path.join(root, name)
        meshgen.write_case(meshgen.CaseSpec(**kw), d)
        _CACHE[key] = d
    return _CACHE[key]


def shuffled_case(root, order_seed, **kw):
    """The case of CaseSpec(**kw) with its cells listed in a seeded random order (the mesh
    reader numbers cells by their line in the .CEL file), i.e. the same mesh with scattered
    cell numbers; written once per session."""
    import shutil
    key = ("shuffled", order_seed) + tuple(sorted(kw.items()))
    if key not in _CACHE:
        src = make_case(root, **kw)
        d = src + "_shuffled%d" % order_seed
        if os.path.exists(d):
            shutil.rmtree(d)
        shutil.copytree(src, d)
        cel = os.path.join(d, "mesh.CEL")
        lines = open(cel).read().splitlines()
        order = np.random.default_rng(order_seed).permutation(len(lines))
        with open(cel, "w") as f:
            for i, j in enumerate(order, 1):
                f.write("%8d%s\n" % (i, lines[j][8:]))
        _CACHE[key] = d
    return _CACHE[key]


def rel_l2(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def assert_close(a, b, rtol, name=""):
    e = rel_l2(a, b)
    assert np.all(np.isfinite(a)), "%s: non-finite values" % name
    assert e <= rtol, "%s: relative L2 error %.3e > %.1e" % (name, e, rtol)
    return e


def var_slice(arr, nvar, keep):
    """Select variables `keep` (0-based) from a flat array whose fastest index has nvar entries."""
    a = np.asarray(arr).reshape(-1, nvar)
    return a[:, keep]


ENTROPY_GAM = 5.0 / 3.0


def entropy_wave_case(root, nx, N, cfl, T, jitter=0.0):
    """A periodic [0, 2pi]^2 case (no AV) with dt = T / steps for the entropy wave below:
    returns (case dir, steps)."""
    import math
    h = 2 * math.pi / nx
    lam = math.sqrt(2) + math.sqrt(ENTROPY_GAM / 0.8)  # |u| + the largest sound speed
    steps = max(1, int(math.ceil(T / (cfl * h / (N * lam)))))
    d = make_case(root, problem="orszag_tang", nx=nx, ny=nx, N=N, jitter=jitter, seed=5, artiv=0, dt=T / steps)
    return d, steps


def entropy_wave_state(X, t=0.0):
    """rho = 1 + 0.2 sin(x + y - 2t), u = v = 1, p = 1, B = A_z = 0: an exact solution of
    ideal MHD that the scheme advects unchanged in shape.  X is (points, 2)."""
    rho = 1 + 0.2 * np.sin(X[:, 0] + X[:, 1] - 2 * t)
    Q = np.zeros((X.shape[0], 9))
    Q[:, 0] = rho
    Q[:, 1] = rho
    Q[:, 2] = rho
    Q[:, 4] = 1.0 / (ENTROPY_GAM - 1) + rho
    return Q


def quadrature_l2(values, Jac, Xs):
    """sqrt(sum J w_i w_j v^2 / sum J w_i w_j) with the interpolatory weights of the
    solution points."""
    N = len(Xs)
    w = np.linalg.solve(np.vander(np.asarray(Xs, np.float64), N, increasing=True).T, 1.0 / np.arange(1, N + 1))
    wJ = np.asarray(Jac) * np.tile(np.outer(w, w).ravel(), np.asarray(Jac).size // (N * N))
    return float(np.sqrt((np.asarray(values) ** 2 * wJ).sum() / wJ.sum()))


def alfven_wave_case(root, nx, N, cfl, T, jitter=0.0):
    """The circularly polarised Alfven wave case (no AV): returns (case dir, steps).  The
    wave of amplitude 0.1 on rho = 1, p = 0.1, B_par = 1 moves at the Alfven speed 1 along
    -(cos 30, sin 30) without change of shape (an exact solution of ideal MHD)."""
    import math
    lam = 1.0 + math.sqrt(5.0 / 3 * 0.1 + 1.01) + 0.2
    h = (1.0 / math.cos(math.radians(30.0))) / nx
    steps = max(1, int(math.ceil(T / (cfl * h / (N * lam)))))
    d = make_case(root, problem="alfven", nx=nx, ny=nx, N=N, jitter=jitter, seed=5, artiv=0, dt=T / steps)
    return d, steps


def alfven_wave_bz(X, t):
    """B_z of the exact wave at time t."""
    import math
    xp = X[:, 0] * math.sqrt(3.0) / 2 + X[:, 1] * 0.5
    return 0.1 * np.cos(2 * math.pi * (xp + t))


def diffusion_wave_case(root, nx, N, kind, coef, T, A=1e-3, cfl=0.05):
    """A small shear wave v = A sin(x) (kind "viscous", mu = coef) or magnetic wave
    B_z = A sin(x) (kind "resistive", eta0 = coef) on rho = 1, p = 1 at rest: both decay as
    exp(-coef t) (the heating and magnetic pressure they cause enter at A^2).  Returns
    (case dir, steps, Q0 builder, variable index)."""
    import math
    h = 2 * math.pi / nx
    lam = math.sqrt(ENTROPY_GAM) + A
    dt0 = min(cfl * h / (N * lam), 0.05 * (h / N) ** 2 / coef)
    steps = int(math.ceil(T / dt0))
    kw = dict(mu=coef) if kind == "viscous" else dict(eta0=coef)
    d = make_case(root, problem="orszag_tang", nx=nx, ny=nx, N=N, artiv=0, dt=T / steps, **kw)
    var = 2 if kind == "viscous" else 7

    def state(X, t=0.0):
        Q = np.zeros((X.shape[0], 9))
        Q[:, 0] = 1.0
        Q[:, var] = A * np.sin(X[:, 0]) * math.exp(-coef * t)
        Q[:, 4] = 1.0 / (ENTROPY_GAM - 1) + 0.5 * Q[:, var] ** 2
        return Q

    return d, steps, state, var
