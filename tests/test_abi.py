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


def _prototypes():
    """name -> list of parameter declarations, from include/gh1.h."""
    src = open(os.path.join(ROOT, "include", "gh1.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    out = {}
    for m in re.finditer(r"\b(?:int|const char\s*\*)\s+(gh1_[a-z0-9_]+)\s*\(([^)]*)\)\s*;", src):
        params = [p.strip() for p in m.group(2).replace("\n", " ").split(",")]
        out[m.group(1)] = [] if params in ([""], ["void"]) else params
    return out


def test_header_compiles_as_c_and_cpp(tmp_path):
    """The boundary header is plain C99 (a cgo or C caller includes it as is)
    and valid C++."""
    import subprocess
    src = tmp_path / "use.c"
    src.write_text('#include "gh1.h"\nint main(void) { return GH1_OK; }\n')
    inc = os.path.join(ROOT, "include")
    subprocess.run(["gcc", "-std=c99", "-pedantic", "-Wall", "-Wextra", "-Werror", "-fsyntax-only", "-I", inc, str(src)],
                   check=True)
    subprocess.run(["g++", "-std=c++17", "-pedantic", "-Wall", "-Wextra", "-Werror", "-fsyntax-only", "-x", "c++",
                    "-I", inc, str(src)], check=True)


def test_binding_matches_prototypes():
    """Every ctypes signature has the header's arity and parameter kinds: a
    pointer for each pointer (or handle), c_int for int / int32, c_int64 for
    int64_t, c_double for double."""
    from ngsolve_gb300 import _lib
    protos = _prototypes()
    assert set(protos) == set(_declared())
    for name, params in protos.items():
        args = _lib.SIGNATURES[name]
        assert len(args) == len(params), (name, params, args)
        for p, a in zip(params, args):
            if "*" in p or p.split()[0] in ("cudaStream_t",):
                assert a is ctypes.c_void_p or issubclass(a, ctypes._Pointer), (name, p, a)
            elif re.match(r"(const\s+)?int64_t\b", p):
                assert a is ctypes.c_int64, (name, p, a)
            elif re.match(r"(const\s+)?(int|int32_t)\b", p):
                assert a is ctypes.c_int, (name, p, a)
            elif re.match(r"(const\s+)?double\b", p):
                assert a is ctypes.c_double, (name, p, a)
            else:
                raise AssertionError("unclassified parameter %r of %s" % (p, name))
