"""The C-ABI library builds, loads and exports every declared symbol (no GPU needed)."""
import ctypes
import os
import re

from pdspy_gb300 import _build, _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            text = open(os.path.join(ROOT, "include", f)).read()
            names |= set(re.findall(r"\b(pdgpu_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_library_exports_declared_symbols():
    path = _build.build()
    lib = ctypes.CDLL(path)
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing
    assert set(declared_symbols()) <= set(_lib.EXPORTS)


def test_abi_version_and_status_strings():
    L = _lib.lib()
    assert L.pdgpu_abi_version() == 2
    assert L.pdgpu_status_string(2) == b"time limit reached"
