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
