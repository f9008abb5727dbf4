"""Loads pdspy's own Model, Grid, Star, Dust, Disk and UlrichEnvelopeExtended classes from a
pdspy source checkout, for tests that bind this package to the real classes.

pdspy cannot be imported as a package in this environment: pdspy/__init__.py imports every
subpackage, some of which need h5py, compiled Cython modules (imaging, interferometry,
radmc3d readers), hyperion, and scipy.integrate.trapz / numpy.trapz, which recent SciPy and
NumPy removed.  The loader registers empty package modules, stubs h5py and the compiled
subpackages with the names Model.py imports, aliases trapz to trapezoid, and loads the
needed files by path.  Nothing is written to the checkout.

The checkout is named by the PDSPY_SOURCE environment variable; ``load()`` returns None
when it is not set or does not hold pdspy.
"""
import importlib.util
import os
import sys
import types

import numpy as np
import scipy.integrate


def source_dir():
    src = os.environ.get("PDSPY_SOURCE")
    if src and os.path.isfile(os.path.join(src, "pdspy", "modeling", "Model.py")):
        return src
    return None


class _Stub:
    """Stand-in for a compiled pdspy class the modules import by name only."""

    def __init__(self, *a, **k):
        self.args, self.kwargs = a, k


def load(src=None):
    """A namespace with pdspy's real Model, Grid, Star, Dust, Disk, UlrichEnvelopeExtended
    and constants modules, or None without a checkout."""
    src = src or source_dir()
    if src is None:
        return None
    saved = {k: v for k, v in sys.modules.items() if k == "pdspy" or k.startswith("pdspy.")}
    had_h5py = "h5py" in sys.modules
    if not hasattr(scipy.integrate, "trapz"):
        scipy.integrate.trapz = scipy.integrate.trapezoid
    if not hasattr(np, "trapz"):
        np.trapz = np.trapezoid
    sys.modules.setdefault("h5py", types.ModuleType("h5py"))

    def package(name):
        mod = types.ModuleType(name)
        mod.__path__ = [os.path.join(src, *name.split("."))]
        sys.modules[name] = mod
        return mod

    def load_file(name):
        path = os.path.join(src, *name.split(".")) + ".py"
        spec = importlib.util.spec_from_file_location(name, path)
        mod = importlib.util.module_from_spec(spec)
        sys.modules[name] = mod
        spec.loader.exec_module(mod)
        return mod

    try:
        for name in ("pdspy", "pdspy.constants", "pdspy.modeling"):
            package(name)
        const = sys.modules["pdspy.constants"]
        for c in ("math", "physics", "astronomy", "time"):
            setattr(const, c, load_file("pdspy.constants." + c))
        dust_pkg = package("pdspy.dust")
        dust_mod = load_file("pdspy.dust.Dust")
        dust_pkg.Dust = dust_mod.Dust
        gas_pkg = package("pdspy.gas")
        gas_pkg.Gas = type("Gas", (), {})
        # compiled or external subpackages Model.py imports by name
        rad = package("pdspy.radmc3d")
        rad.write = types.ModuleType("pdspy.radmc3d.write")
        rad.run = types.ModuleType("pdspy.radmc3d.run")
        rad.read = types.ModuleType("pdspy.radmc3d.read")
        img = package("pdspy.imaging")
        img.Image = img.UnstructuredImage = _Stub
        img.imtovis = lambda *a, **k: None
        inter = package("pdspy.interferometry")
        inter.Visibilities = _Stub
        spec = package("pdspy.spectroscopy")
        spec.Spectrum = _Stub
        star = load_file("pdspy.modeling.Star")
        grid = load_file("pdspy.modeling.Grid")
        model = load_file("pdspy.modeling.Model")
        disk = load_file("pdspy.modeling.Disk")
        env = load_file("pdspy.modeling.UlrichEnvelopeExtended")
        ns = types.SimpleNamespace(Model=model.Model, Grid=grid.Grid, Star=star.Star,
                                   Dust=dust_mod.Dust, Disk=disk.Disk,
                                   UlrichEnvelopeExtended=env.UlrichEnvelopeExtended,
                                   constants=const, model_module=model)
    finally:
        for k in [k for k in sys.modules if k == "pdspy" or k.startswith("pdspy.")]:
            del sys.modules[k]
        sys.modules.update(saved)
        if not had_h5py:
            sys.modules.pop("h5py", None)
    return ns
