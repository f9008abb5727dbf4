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
    assert L.pdgpu_abi_version() == 4
    assert L.pdgpu_status_string(2) == b"time limit reached"


def test_run_thermal_keyword_mapping():
    """radmc3d.write.control keywords map onto plan options; host-only keywords are
    accepted silently, unknown ones warn."""
    import warnings
    from pdspy_gb300 import thermal
    o = thermal._options(dict(iseed=7, modified_random_walk=True, mrw_gamma=3.0,
                              mrw_tauthres=5.0, mrw_count_trigger=50, timelimit=12.0,
                              setthreads=16, nice=5, verbose=False))
    assert o == dict(seed=7, mrw=True, mrw_gamma=3.0, mrw_tauthres=5.0, mrw_count_trigger=50,
                     timelimit=12.0)
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        thermal._options(dict(not_a_keyword=1))
    assert any("not_a_keyword" in str(x.message) for x in w)
