"""The C-ABI library builds, loads and exports every symbol that include/nyles_gb300.h
declares (no compute call: this runs without a GPU)."""
import ctypes
import os
import re

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(REPO, "include", "nyles_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(nyles_[A-Za-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    from nyles_gb300 import build, _native
    try:
        build.nvcc()
    except RuntimeError:
        pytest.skip("no CUDA toolkit to build the library")
    build.build()
    lib = ctypes.CDLL(build.LIB)
    syms = declared_symbols()
    assert len(syms) >= 25
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing
    # the Python binding covers the same set
    assert set(syms) == set(_native.SIGNATURES)
    assert lib.nyles_version() == 10000
