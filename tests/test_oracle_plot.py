"""Plot output of the oracle (tecplotter2dsetup / tecplotter2d / tecpost_parallel):
known answers for the plot-node topology, exact interpolation, the file layout and the
file name.  CPU only."""
import struct

import numpy as np
import pytest

import oracle
from helpers import make_case


def read_tecplot(path):
    """Parse the #!TDV111 layout that tecpost_parallel writes (tecplotter.f90:186-395)."""
    b = open(path, "rb").read()
    pos = 0

    def take(fmt):
        nonlocal pos
        v = struct.unpack_from("<" + fmt, b, pos)
        pos += struct.calcsize("<" + fmt)
        return v

    def string():
        chars = []
        while True:
            (c,) = take("i")
            if c == 0:
                return "".join(map(chr, chars))
            chars.append(c)

    magic = b[:8].decode()
    pos = 8
    one, ftype = take("2i")
    title = string()
    (nvar,) = take("i")
    names = [string() for _ in range(nvar)]
    (zm,) = take("f")
    zone = string()
    parent, strand = take("2i")
    (t,) = take("d")
    zh = take("12i")
    eoh, zm2 = take("2f")
    fmt = take("%di" % (nvar + 3))
    minmax = np.array(take("%dd" % (2 * nvar))).reshape(nvar, 2)
    nodes, cells = zh[6], zh[7]
    data = np.frombuffer(b, "<f4", nvar * nodes, pos).reshape(nvar, nodes)
    pos += 4 * nvar * nodes
    con = np.frombuffer(b, "<i4", 4 * cells, pos).reshape(cells, 4)
    pos += 16 * cells
    return dict(magic=magic, one=one, ftype=ftype, title=title, names=names, zonemarker=zm, zone=zone,
                parent=parent, strand=strand, time=t, zoneheader=zh, eoh=eoh, zonemarker2=zm2, fmt=fmt,
                minmax=minmax, data=data, con=con, trailing=len(b) - pos)


@pytest.mark.parametrize("nx,ny,N,nre,jitter", [(4, 3, 4, 4, 0.1), (3, 3, 3, 1, 0.0), (5, 2, 5, 3, 0.15)])
def test_plot_topology_known_answers(case_root, nx, ny, N, nre, jitter):
    d = make_case(case_root, problem="orszag_tang", nx=nx, ny=ny, N=N, jitter=jitter, seed=4)
    o = oracle.Oracle(d)
    assert o.plot_setup(nre) == 0
    nodes, cells = o.geti("plotnodes"), o.geti("plotcells")
    assert nodes == (nre * nx + 1) * (nre * ny + 1)  # shared vertices and edge nodes
    assert cells == nx * ny * nre * nre
    fac = o.array("gnode_factor")
    assert fac.sum() == (nre + 1) ** 2 * nx * ny
    assert set(np.unique(fac)) <= {1, 2, 4}
    con = o.array("connec_c2n").reshape(cells, 4)
    assert con.min() == 1 and con.max() == nodes
    assert len(np.unique(con)) == nodes
    X = o.array("plotX").reshape(nodes, 2)
    if jitter == 0.0:  # a uniform mesh: the nodes are the lattice of spacing h/nre
        h = 2 * np.pi / nx / nre
        k = X[:, 0] / h
        assert np.allclose(k, np.round(k), atol=1e-9)


def test_plot_interpolation_is_exact_for_the_state(case_root):
    """A uniform state comes back as its primitive variables at every node."""
    d = make_case(case_root, problem="orszag_tang", nx=3, ny=4, N=4, jitter=0.12, seed=9)
    o = oracle.Oracle(d)
    Q = o.array("Q")
    q0 = np.array([1.7, 0.3, -0.2, 0.1, 3.0, 0.4, -0.5, 0.25, 0.6])
    Q[:] = np.tile(q0, Q.size // 9)
    o.compresid()
    o.plot_setup(3)
    o.plot_eval()
    P = o.array("plotQ").reshape(-1, 9)
    rho, u = q0[0], q0[1:4] / q0[0]
    p = (q0[4] - 0.5 * rho * (u ** 2).sum() - 0.5 * (q0[5:8] ** 2).sum()) * (5.0 / 3 - 1)
    expect = np.concatenate([[rho], u, [p], q0[5:9]])
    assert np.allclose(P, expect[None, :], rtol=1e-13, atol=1e-14)


def test_plot_file_layout(case_root, tmp_path):
    d = make_case(case_root, problem="orszag_tang", nx=4, ny=4, N=4, jitter=0.1, seed=3)
    o = oracle.Oracle(d)
    o.run(2)
    o.plot_setup(2)
    o.plot_eval()
    path = str(tmp_path / oracle.plot_filename(0.625))
    o.plot_write(0.625, path)
    f = read_tecplot(path)
    nodes, cells = o.geti("plotnodes"), o.geti("plotcells")
    assert f["magic"] == "#!TDV111" and f["one"] == 1 and f["ftype"] == 0
    assert f["title"] == "step data"
    assert f["names"] == ["X", "Y", "RHO", "U", "V", "W", "P", "Bx", "By", "Bz", "Az", "muAV", "etaAV"]
    assert f["zonemarker"] == 299.0 and f["zonemarker2"] == 299.0 and f["eoh"] == 357.0
    assert f["zone"] == "ZONE 001" and (f["parent"], f["strand"]) == (-1, 0)
    assert f["time"] == 0.625
    assert f["zoneheader"] == (-1, 3, 0, 0, 0, 0, nodes, cells, 0, 0, 0, 0)
    assert f["fmt"] == tuple([1] * 13 + [0, 0, -1])
    assert f["trailing"] == 0
    X = o.array("plotX").reshape(nodes, 2)
    Q = o.array("plotQ").reshape(nodes, 9)
    AV = o.array("plotAV").reshape(nodes, 2)
    full = np.concatenate([X, Q, AV], axis=1).T
    assert np.array_equal(f["data"], full.astype(np.float32))
    assert np.array_equal(f["minmax"][:, 0], full.min(axis=1))
    assert np.array_equal(f["minmax"][:, 1], full.max(axis=1))
    assert np.array_equal(f["con"], o.array("connec_c2n").reshape(cells, 4) - 1)


@pytest.mark.parametrize("t,name", [(0.1234, "TEC0000000.123.plt"), (12.9996, "TEC0000012.000.plt"),
                                    (3.5, "TEC0000003.500.plt"), (1234567.25, "TEC1234567.250.plt")])
def test_plot_filename(t, name):
    assert oracle.plot_filename(t) == name


@pytest.mark.parametrize("t", [0.0, 0.1234, 12.9996, 3.5, 0.0625, 99.9994, 1234567.25])
def test_product_filename_matches_oracle(t):
    """chorus_plot_filename is host code: callable without a GPU."""
    from chorus_mhd import plot_filename
    assert plot_filename(t) == oracle.plot_filename(t)
