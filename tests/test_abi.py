"""The C-ABI library loads and exports every entry point include/gh1.h declares
(no compute calls: this runs without a GPU)."""
import ctypes
import os
import re

from tests.conftest import ROOT


def _declared():
    src = open(os.path.join(ROOT, "include", "gh1.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(gh1_[a-z0-9_]+)\s*\(", src)))


def test_header_symbols_exported():
    from ngsolve_gb300 import build
    path = build.build()
    lib = ctypes.CDLL(path)
    names = _declared()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, "not exported: %s" % missing


def test_python_binding_covers_header():
    from ngsolve_gb300 import _lib
    assert set(_declared()) <= set(_lib.SIGNATURES), set(_declared()) - set(_lib.SIGNATURES)


def test_no_cpu_fallback_without_gpu():
    import torch
    import pytest
    if torch.cuda.is_available():
        pytest.skip("has a GPU")
    import ngsolve_gb300 as ng
    from ngsolve_gb300._lib import GH1Error
    with pytest.raises(GH1Error):
        ng.H1(ng.MakeStructured3DMesh(nx=2), order=2)
