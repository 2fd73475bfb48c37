"""The product path has no CPU fallback and never reaches the oracle: the package imports
no oracle module, the library links no oracle code, and loading it fails loudly when the
built library is missing."""
import ast
import glob
import os
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
PKG = os.path.join(ROOT, "chorus-mhd_gb300", "chorus_mhd")


def test_package_never_imports_the_oracle():
    for path in glob.glob(os.path.join(PKG, "*.py")):
        tree = ast.parse(open(path).read())
        for node in ast.walk(tree):
            names = []
            if isinstance(node, ast.Import):
                names = [a.name for a in node.names]
            elif isinstance(node, ast.ImportFrom):
                names = [node.module or ""]
            assert not any(n.split(".")[0] == "oracle" for n in names), path


def test_library_links_no_oracle_code():
    from chorus_mhd import _lib
    lib = _lib.LIB_PATH
    if not os.path.exists(lib):
        pytest.skip("library not built")
    syms = subprocess.run(["nm", "-D", lib], capture_output=True, text=True).stdout
    assert "orc_" not in syms
    deps = subprocess.run(["ldd", lib], capture_output=True, text=True).stdout
    assert "liborc" not in deps


def test_missing_library_fails_loudly(tmp_path):
    from chorus_mhd import _lib
    with pytest.raises(RuntimeError, match="not built"):
        _lib.load(str(tmp_path / "libchorus_gpu.so"))
