"""CPU checks of the shipped library: it loads, and exports every function that
include/*.h declares (no compute calls: there is no GPU here)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "kspace-neutrinos_gb300")
LIB = os.path.join(PKG, "libkspace_gb300.so")


def declared():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            text = open(os.path.join(inc, f)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            for m in re.finditer(r"\b(kspace_gpu_\w+)\s*\(", text):
                names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(LIB):
        import sys
        sys.path.insert(0, PKG)
        import build
        build.build()
    return ctypes.CDLL(LIB)


def test_every_declared_symbol_is_exported(lib):
    names = declared()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_the_abi():
    import kspace_gpu
    assert set(declared()) == set(kspace_gpu.exported_symbols())


def test_error_strings(lib):
    lib.kspace_gpu_error_string.restype = ctypes.c_char_p
    assert lib.kspace_gpu_error_string(0) == b"success"
    assert b"nan" in lib.kspace_gpu_error_string(2004)
