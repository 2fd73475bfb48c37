"""Synthetic cases in the reference's input formats.

The reference ships no input deck and no mesh, so every run here starts from a seeded
synthetic case written in exactly the formats the reference reads:

* ``QUAD.INP``  -- positional lines, readinput.f90:6-36 (29 lines), followed by an
  extension block (gamma, problem id, B0x, B0y) that the reference never reads;
* ``*.CEL``     -- ``IC IV1 IV2 IV3 IV4 ICTYPE ICKEY`` per line (readGRIDinfo.f90:33);
* ``*.VRT``     -- ``FORMAT(I9,6X,3(D20.12,1X))`` (readGRIDinfo.f90:79-80), so vertex
  coordinates carry 12 significant digits and every reader sees the rounded values;
* ``*.BND``     -- ``IB IV1 IV2 IREGION IPATCH TYPE`` (readGRIDinfo.f90:237-238).

Meshes are structured nx x ny quads written as an unstructured list, counter-clockwise
(CHECK_MESH does not reorient, connectivity.f90:264-272).  Interior nodes may be
jittered uniformly by +-jitter*h (seeded); boundary nodes stay on the boundary so that
periodic partner faces match within tolCYC (connect_bdry.f90:293).
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

import numpy as np

PROBLEMS = {"orszag_tang": 0, "rotor": 1, "alfven": 2}


def fortran_d20_12(v: float) -> str:
    """Format like Fortran's D20.12 edit descriptor: ' 0.ddddddddddddD+ee'."""
    if v == 0.0 or not math.isfinite(v):
        return " 0.000000000000D+00".rjust(20)
    s = "%.11E" % abs(v)           # d.dddddddddddE+xx, correctly rounded to 12 digits
    mant, ex = s.split("E")
    digits = mant.replace(".", "")
    e = int(ex) + 1
    sign = "-" if v < 0 else " "
    body = "%s0.%sD%s%02d" % (sign, digits, "+" if e >= 0 else "-", abs(e))
    return body.rjust(20)


@dataclass
class CaseSpec:
    """One solve: mesh, order, physics and time stepping."""
    nx: int = 8
    ny: int = 8
    N: int = 4                      # solution points per direction (= order p + 1)
    problem: str = "orszag_tang"
    jitter: float = 0.0             # interior-node jitter as a fraction of h
    seed: int = 0
    steps: int = 10
    dt: float | None = None         # None: from CFL at t=0
    cfl: float = 0.1
    k_stage: int = 3                # 3: RK_S5P3, 5: FiveStageRk (both 5 stages)
    vismode: int = 1                # must be 1 (compflux.f90:72-75)
    mu: float = 0.0
    eta0: float = 0.0
    artiv: int = 1
    nwrite: int = 1000000
    nre: int = 1                    # plot sub-intervals per cell edge (readinput.f90:32)
    gamma: float | None = None      # None: the problem's default
    extra: dict = field(default_factory=dict)

    def domain(self):
        if self.problem == "orszag_tang":
            return 0.0, 2 * math.pi, 0.0, 2 * math.pi, "CYCL"
        if self.problem == "rotor":
            return 0.0, 1.0, 0.0, 1.0, "FREE"
        if self.problem == "alfven":
            a = math.radians(30.0)
            return 0.0, 1.0 / math.cos(a), 0.0, 1.0 / math.sin(a), "CYCL"
        raise ValueError("unknown problem %r" % self.problem)

    def gam(self) -> float:
        if self.gamma is not None:
            return float(self.gamma)
        return 1.4 if self.problem == "rotor" else 5.0 / 3

    def background_field(self):
        if self.problem == "alfven":
            a = math.radians(30.0)
            return math.cos(a), math.sin(a)
        return 0.0, 0.0

    @property
    def ncell(self) -> int:
        return self.nx * self.ny


def mesh_vertices(spec: CaseSpec):
    """Vertex coordinates (global id = j*(nx+1)+i+1), cells (ccw) and boundary edges."""
    x0, x1, y0, y1, btype = spec.domain()
    nx, ny = spec.nx, spec.ny
    hx, hy = (x1 - x0) / nx, (y1 - y0) / ny
    ii, jj = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), indexing="xy")
    X = x0 + ii * hx
    Y = y0 + jj * hy
    X[:, -1] = x1
    Y[-1, :] = y1
    if spec.jitter > 0:
        rng = np.random.default_rng(spec.seed)
        dx = rng.uniform(-spec.jitter, spec.jitter, size=X.shape) * hx
        dy = rng.uniform(-spec.jitter, spec.jitter, size=Y.shape) * hy
        inner = np.zeros(X.shape, bool)
        inner[1:-1, 1:-1] = True
        X = np.where(inner, X + dx, X)
        Y = np.where(inner, Y + dy, Y)
    vid = lambda i, j: j * (nx + 1) + i + 1  # noqa: E731
    cells = np.empty((nx * ny, 4), np.int64)
    c = 0
    for j in range(ny):
        for i in range(nx):
            cells[c] = (vid(i, j), vid(i + 1, j), vid(i + 1, j + 1), vid(i, j + 1))
            c += 1
    bnd = []
    for i in range(nx):
        bnd.append((vid(i, 0), vid(i + 1, 0), 1))
    for j in range(ny):
        bnd.append((vid(nx, j), vid(nx, j + 1), 2))
    for i in range(nx):
        bnd.append((vid(i + 1, ny), vid(i, ny), 3))
    for j in range(ny):
        bnd.append((vid(0, j + 1), vid(0, j), 4))
    return X.reshape(-1), Y.reshape(-1), cells, bnd, btype


def _ic_primitive(problem, x, y, gam):
    """rho, u, v, w, p, Bx, By, Bz of the analytic initial data (for the CFL estimate)."""
    if problem == "orszag_tang":
        rho = np.full_like(x, gam * gam)
        u, v, w = -np.sin(y), np.sin(x), 0 * x
        p = np.full_like(x, gam)
        bx, by, bz = -np.sin(y), np.sin(2 * x), 0 * x
    elif problem == "rotor":
        r0, r1, u0 = 0.1, 0.115, 2.0
        dx, dy = x - 0.5, y - 0.5
        r = np.sqrt(dx * dx + dy * dy)
        f = np.clip((r1 - r) / (r1 - r0), 0.0, 1.0)
        rho = np.where(r < r0, 10.0, 1.0 + 9.0 * f)
        sc = np.where(r < r0, 1.0 / r0, f / np.maximum(r, 1e-300))
        u, v, w = -u0 * dy * sc, u0 * dx * sc, 0 * x
        p = np.ones_like(x)
        bx, by, bz = np.full_like(x, 5.0 / math.sqrt(4 * math.pi)), 0 * x, 0 * x
    else:
        ca, sa, amp = math.sqrt(3) / 2, 0.5, 0.1
        xp = x * ca + y * sa
        vp, vz = amp * np.sin(2 * math.pi * xp), amp * np.cos(2 * math.pi * xp)
        rho, p = np.ones_like(x), np.full_like(x, 0.1)
        u, v, w = -vp * sa, vp * ca, vz
        bx, by, bz = ca - vp * sa, sa + vp * ca, vz
    return rho, u, v, w, p, bx, by, bz


def cfl_dt(spec: CaseSpec, X, Y, cells) -> float:
    """dt = CFL * h_min / (N * lambda_max(t=0)); the reference uses a fixed dt from
    QUAD.INP (readinput.f90:24), so this value is computed once and written there."""
    gam = spec.gam()
    c = cells - 1
    xc = X[c].mean(axis=1)
    yc = Y[c].mean(axis=1)
    # sample the initial data on a fine uniform grid plus the cell centres
    x0, x1, y0, y1, _ = spec.domain()
    gx, gy = np.meshgrid(np.linspace(x0, x1, 257), np.linspace(y0, y1, 257))
    xs = np.concatenate([xc, gx.ravel()])
    ys = np.concatenate([yc, gy.ravel()])
    rho, u, v, w, p, bx, by, bz = _ic_primitive(spec.problem, xs, ys, gam)
    b2 = bx * bx + by * by + bz * bz
    cf = np.sqrt((gam * p + b2) / rho)
    lam = float(np.max(np.sqrt(u * u + v * v) + cf))
    e = [np.hypot(X[c[:, (k + 1) % 4]] - X[c[:, k]], Y[c[:, (k + 1) % 4]] - Y[c[:, k]]) for k in range(4)]
    hmin = float(np.min(np.minimum(np.minimum(e[0], e[1]), np.minimum(e[2], e[3]))))
    return spec.cfl * hmin / (spec.N * lam)


def write_case(spec: CaseSpec, out_dir: str, name: str = "mesh") -> str:
    """Write QUAD.INP + mesh files for `spec` into out_dir; returns out_dir."""
    os.makedirs(out_dir, exist_ok=True)
    X, Y, cells, bnd, btype = mesh_vertices(spec)
    with open(os.path.join(out_dir, name + ".CEL"), "w") as f:
        for ic, c in enumerate(cells, 1):
            f.write("%8d %8d %8d %8d %8d %4d %4d\n" % (ic, c[0], c[1], c[2], c[3], 1, 1))
    with open(os.path.join(out_dir, name + ".VRT"), "w") as f:
        for iv, (x, y) in enumerate(zip(X, Y), 1):
            f.write("%9d      %s %s %s \n" % (iv, fortran_d20_12(float(x)), fortran_d20_12(float(y)),
                                             fortran_d20_12(0.0)))
    with open(os.path.join(out_dir, name + ".BND"), "w") as f:
        for ib, (a, b, side) in enumerate(bnd, 1):
            f.write("%8d %8d %8d %4d %4d %s\n" % (ib, a, b, 1, side, btype))
    x0, x1, y0, y1, _ = spec.domain()
    # the periodic lengths as the mesh file spells them (12 significant digits)
    dxc = float(fortran_d20_12(x1 - x0).replace("D", "E"))
    dyc = float(fortran_d20_12(y1 - y0).replace("D", "E"))
    dt = spec.dt if spec.dt is not None else cfl_dt(spec, X, Y, cells)
    b0x, b0y = spec.background_field()
    lines = [
        "CHORUS-MHD input (readinput.f90 layout)",
        "mesh files",
        name + ".CEL",
        name + ".VRT",
        name + ".VRT8",
        name + ".BND",
        "metis.part",
        "restart.dat",
        "SD order / physics",
        "%d" % spec.N,
        "0",
        "%d" % spec.vismode,
        repr(float(spec.mu)),
        repr(float(spec.eta0)),
        "time marching",
        "%d" % spec.k_stage,
        repr(float(dt)),
        "%d" % spec.steps,
        "periodic lengths",
        repr(dxc),
        repr(dyc),
        "artificial viscosity",
        "%d" % spec.artiv,
        "output",
        "%d" % spec.nre,
        "%d" % spec.nwrite,
        "restart",
        "0",
        "%d" % spec.N,
        "extension: gamma, problem, B0x, B0y (not read by the reference)",
        repr(spec.gam()),
        "%d" % PROBLEMS[spec.problem],
        repr(float(b0x)),
        repr(float(b0y)),
    ]
    with open(os.path.join(out_dir, "QUAD.INP"), "w") as f:
        f.write("\n".join(lines) + "\n")
    return out_dir


def read_quad_inp(case_dir: str) -> dict:
    """Parse QUAD.INP (same positional layout as readinput.f90:6-36 + extension)."""
    with open(os.path.join(case_dir, "QUAD.INP")) as f:
        L = [ln.rstrip("\n") for ln in f]
    tok = lambda s: s.split()[0].strip("'\"")  # noqa: E731
    real = lambda s: float(tok(s).replace("D", "E").replace("d", "e"))  # noqa: E731
    d = dict(namecel=tok(L[2]), namevrt=tok(L[3]), namebnd=tok(L[5]), namerestart=tok(L[7]),
             N=int(tok(L[9])), curve_wall=int(tok(L[10])), vismode=int(tok(L[11])), mu=real(L[12]),
             eta0=real(L[13]), k_stage=int(tok(L[15])), dt=real(L[16]), maxiter=int(tok(L[17])),
             dxcycl=real(L[19]), dycycl=real(L[20]), artiv=int(tok(L[22])), nre=int(tok(L[24])),
             nwrite=int(tok(L[25])), restart=int(tok(L[27])), restart_ord=int(tok(L[28])),
             gam=5.0 / 3, problem=0, b0x=0.0, b0y=0.0)
    if len(L) >= 31:
        d["gam"] = real(L[30])
    if len(L) >= 32:
        d["problem"] = int(tok(L[31]))
    if len(L) >= 33:
        d["b0x"] = real(L[32])
    if len(L) >= 34:
        d["b0y"] = real(L[33])
    return d
