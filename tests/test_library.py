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


def _scat_plan(L, nlam=3, nspec=1, nphot=1000, kabs=None, r=None):
    import ctypes as C
    import numpy as np
    r = np.logspace(12, 15, 11) if r is None else r
    t = np.linspace(0, np.pi / 2, 9)
    p = np.array([0.0, 2 * np.pi])
    rad, tem = np.array([1.4e11]), np.array([4000.0])
    lam = np.logspace(0, 1, nlam)
    ka = np.ones((nspec, nlam)) if kabs is None else kabs
    ks = np.ones((nspec, nlam))
    keep = [np.ascontiguousarray(a, dtype=np.float64) for a in (r, t, p, rad, tem, lam, ka, ks)]
    dp = C.POINTER(C.c_double)
    ptr = [a.ctypes.data_as(dp) for a in keep]
    desc = _lib.ModelDesc(len(r) - 1, len(t) - 1, len(p) - 1, ptr[0], ptr[1], ptr[2], 1, ptr[3],
                          ptr[4], 0)
    opts = _lib.ScatOptions(1, nphot, 5.0, 0, 0, 0)
    plan = C.c_void_p()
    st = L.pdgpu_scat_plan_create(C.byref(desc), nlam, ptr[5], nspec, ptr[6], ptr[7],
                                  C.byref(opts), C.byref(plan))
    return st, plan


def test_scattering_plan_validates_arguments_and_sizes_its_workspace():
    """Host-side plan logic of the scattering Monte Carlo (no kernels launched)."""
    import ctypes as C
    import numpy as np
    L = _lib.lib()
    st, plan = _scat_plan(L)
    assert st == 0
    ws, nc = C.c_size_t(), C.c_int64()
    assert L.pdgpu_scat_plan_info(plan, C.byref(ws), C.byref(nc)) == 0
    assert nc.value == 10 * 8 * 1
    # cell CDF (float) and path sums (int64) per wavelength and cell dominate the workspace
    assert ws.value >= 3 * nc.value * (4 + 8)
    L.pdgpu_scat_plan_destroy(plan)
    assert _scat_plan(L, nlam=0)[0] == 1                                  # no wavelengths
    assert _scat_plan(L, nphot=0)[0] == 1                                 # no packets
    assert _scat_plan(L, kabs=-np.ones((1, 3)))[0] == 1                   # negative opacity
    assert _scat_plan(L, nspec=5, kabs=np.ones((5, 3)))[0] == 1           # too many species
    assert _scat_plan(L, r=np.array([1e13, 1e12, 1e14]))[0] == 1          # unsorted radii
