"""The chunk plan of the host-state step (chorus_mesh_host_chunks, the plan chorus_gpu_step_host
follows), checked on the host against the mesh's own face lists: the first stage's face pass
may take a face once both its cells have been through E1, and a run of cells may be
downloaded once it and all its face neighbours are through the last stage's E3 and CT
passes.  CPU only."""
import ctypes

import numpy as np
import pytest

from chorus_mhd import Mesh, _lib
from helpers import make_case, shuffled_case

CASES = [dict(problem="orszag_tang", nx=72, ny=64, N=4, jitter=0.1, seed=21),
         dict(problem="orszag_tang", nx=256, ny=240, N=4, jitter=0.1, seed=21),
         dict(problem="rotor", nx=256, ny=240, N=3, jitter=0.1, seed=2),
         dict(problem="orszag_tang", nx=3, ny=2, N=3)]


def plan(mesh, chunks):
    L = _lib.load()
    K, nseg = ctypes.c_int32(), ctypes.c_int32()
    cut, f2, f1 = (ctypes.c_int32 * 33)(), (ctypes.c_int32 * 33)(), (ctypes.c_int32 * 33)()
    seg = (ctypes.c_int32 * 198)()
    _lib.check(L.chorus_mesh_host_chunks(mesh._h, chunks, ctypes.byref(K), cut, f2, f1, ctypes.byref(nseg), seg))
    k = K.value
    return (k, np.array(cut[:k + 1]), np.array(f2[:k + 1]), np.array(f1[:k + 1]),
            np.array(seg[:3 * nseg.value]).reshape(-1, 3))


def faces(mesh):
    """Two-sided faces (interior and periodic pairs) as 0-based cell pairs, FREE faces' cells."""
    if2c = mesh.iarray("IF2C")
    nf = if2c.size // 4
    if2c = if2c.reshape(4, nf)
    inter = mesh.iarray("IBFINTER") - 1
    pairs = [(if2c[0, f] - 1, if2c[1, f] - 1) for f in inter]
    cyc = mesh.iarray("CYC2FPAIR")
    npair = cyc.size // 2
    pairs += [(if2c[0, cyc[i] - 1] - 1, if2c[0, cyc[i + npair] - 1] - 1) for i in range(npair)]
    free = [if2c[0, f - 1] - 1 for f in mesh.iarray("IBFREE")]
    return np.array(pairs, np.int64).reshape(-1, 2), np.array(free, np.int64)


@pytest.fixture(scope="module")
def meshes(tmp_path_factory):
    """The cases above, then the periodic 256x240 case and the rotor with their cells
    numbered in a random order (the plan's fallback to whole chunks)."""
    root = str(tmp_path_factory.mktemp("chunks"))
    out = [Mesh(make_case(root, **c)) for c in CASES]
    out += [Mesh(shuffled_case(root, 3, **CASES[1])), Mesh(shuffled_case(root, 4, **CASES[2]))]
    yield out
    for m in out:
        m.close()


@pytest.mark.parametrize("which", range(len(CASES) + 2))
@pytest.mark.parametrize("chunks", [1, 3, 8, 16, 32])
def test_plan_respects_face_dependencies(meshes, which, chunks):
    m = meshes[which]
    nc = m.ncell
    K, cut, f2cut, f1cut, seg = plan(m, chunks)
    assert K == max(1, min(chunks, nc // 1024))
    assert cut[0] == 0 and cut[-1] == nc and np.all(np.diff(cut) > 0)
    pairs, free = faces(m)
    big = pairs.max(axis=1) if len(pairs) else np.zeros(0, np.int64)
    # the face pass of chunk k takes exactly the faces whose cells are all in chunks 0..k
    for k in range(K + 1):
        assert f2cut[k] == np.count_nonzero(big < cut[k])
        assert f1cut[k] == np.count_nonzero(free < cut[k])
    # the download runs cover every cell once, in order
    assert seg[0, 0] == 0 and seg[-1, 1] == nc
    assert np.all(seg[1:, 0] == seg[:-1, 1]) and np.all(seg[:, 1] > seg[:, 0])
    # a run is released only once its cells and their face neighbours are through
    rel = np.arange(nc)
    if len(pairs):
        np.maximum.at(rel, pairs[:, 0], pairs[:, 1])
        np.maximum.at(rel, pairs[:, 1], pairs[:, 0])
    chunk_of = np.searchsorted(cut[1:], np.arange(nc), side="right")
    for a, b, k in seg:
        assert 0 <= k < K
        assert rel[a:b].max() < cut[k + 1], (a, b, k)
        assert chunk_of[b - 1] <= k


def test_plan_releases_runs_with_their_chunk(meshes):
    """On the generator's row-major numbering each chunk's cells (bar the rows that touch the
    next chunk or, with periodic faces, the last row) are released right after that chunk:
    the downloads follow the last stage's passes instead of waiting for the end."""
    for m in meshes[1:3]:
        K, cut, _, _, seg = plan(m, 16)
        early = sum(b - a for a, b, k in seg if k < K - 1)
        assert early >= 0.8 * m.ncell


def test_scattered_numbering_falls_back_to_whole_chunks(meshes):
    """With cells numbered at random nearly every cell has a neighbour in the last chunk, so
    the runs fragment and the plan downloads whole chunks, each when its last neighbour is
    through (still checked above)."""
    for m in meshes[len(CASES):]:
        K, cut, _, _, seg = plan(m, 16)
        assert len(seg) == K
        assert np.array_equal(seg[:, 0], cut[:-1]) and np.array_equal(seg[:, 1], cut[1:])


def test_plan_rejects_bad_counts(meshes):
    L = _lib.load()
    z = (ctypes.c_int32 * 198)()
    n = ctypes.c_int32()
    for bad in (0, 33):
        assert L.chorus_mesh_host_chunks(meshes[0]._h, bad, ctypes.byref(n), z, z, z, ctypes.byref(n), z) != 0
