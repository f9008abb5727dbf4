"""Generate golden fixtures from the reference pdspy's own density builders.

Run where a pdspy source checkout is available, naming it on the command line or in
PDSPY_SOURCE:

    python tests/golden/make_golden.py <path to the pdspy checkout>

pdspy cannot be imported as a package here (pdspy/__init__.py imports every subpackage,
some of which need h5py, compiled Cython modules and scipy.integrate.trapz, removed in
recent SciPy).  The shim below registers empty package modules, stubs h5py, aliases
scipy.integrate.trapz/numpy.trapz to trapezoid and loads the needed files by path:
pdspy/constants/*.py, pdspy/modeling/Star.py, Disk.py, UlrichEnvelopeExtended.py.
The outputs (tests/golden/pdspy_builders.npz) pin this package's restatements of the
same builders (pdspy_gb300/modeling/), which is what the GPU path is fed with.
"""
import importlib.util
import os
import sys
import types

import numpy as np
import scipy.integrate

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = None


def source_dir(argv=None):
    """The pdspy checkout: the first command-line argument, else $PDSPY_SOURCE."""
    argv = sys.argv[1:] if argv is None else argv
    src = argv[0] if argv else os.environ.get("PDSPY_SOURCE")
    if not src or not os.path.isfile(os.path.join(src, "pdspy", "modeling", "Disk.py")):
        raise SystemExit("usage: make_golden.py <pdspy checkout> (or set PDSPY_SOURCE); "
                         "got %r" % (src,))
    return src


def _shim():
    if not hasattr(scipy.integrate, "trapz"):
        scipy.integrate.trapz = scipy.integrate.trapezoid
    if not hasattr(np, "trapz"):
        np.trapz = np.trapezoid
    sys.modules.setdefault("h5py", types.ModuleType("h5py"))
    for name in ("pdspy", "pdspy.constants", "pdspy.dust", "pdspy.gas", "pdspy.modeling"):
        mod = types.ModuleType(name)
        mod.__path__ = [os.path.join(SRC, *name.split("."))]
        sys.modules[name] = mod

    def load(name):
        path = os.path.join(SRC, *name.split(".")) + ".py"
        spec = importlib.util.spec_from_file_location(name, path)
        mod = importlib.util.module_from_spec(spec)
        sys.modules[name] = mod
        spec.loader.exec_module(mod)
        return mod

    for c in ("math", "physics", "astronomy", "time"):
        setattr(sys.modules["pdspy.constants"], c, load("pdspy.constants." + c))
    # Disk/envelope import Dust and Gas by name only
    dmod = types.ModuleType("pdspy.dust")
    dmod.Dust = type("Dust", (), {})
    sys.modules["pdspy.dust"] = dmod
    gmod = types.ModuleType("pdspy.gas")
    gmod.Gas = type("Gas", (), {})
    sys.modules["pdspy.gas"] = gmod
    star = load("pdspy.modeling.Star")
    disk = load("pdspy.modeling.Disk")
    env = load("pdspy.modeling.UlrichEnvelopeExtended")
    return star, disk, env, sys.modules["pdspy.constants"]


def main():
    global SRC
    SRC = source_dir()
    star, disk, env, const = _shim()
    out = {}
    # small axisymmetric disk on 100 log-r cells over 0.1-100 au and 100 theta cells over [0, pi]
    w1 = np.logspace(-1, 2, 101)
    w2 = np.linspace(0, np.pi, 101)
    w3 = np.array([0.0, 2 * np.pi])
    r, th, ph = [0.5 * (w[1:] + w[:-1]) for w in (w1, w2, w3)]
    d = disk.Disk(mass=1e-4, rmin=0.1, rmax=100.0, plrho=2.25, h0=0.1, plh=1.25)
    out["disk_w1"], out["disk_w2"], out["disk_w3"] = w1, w2, w3
    out["disk_rho"] = d.density(r, th, ph)
    # heavier disk with a different flaring on a mirrored theta grid (pdspy's radmc3d grids)
    w2m = np.linspace(0, np.pi / 2, 41)
    thm = 0.5 * (w2m[1:] + w2m[:-1])
    d2 = disk.Disk(mass=3e-3, rmin=0.5, rmax=60.0, plrho=2.1, h0=0.05, plh=1.1)
    out["disk2_w2"] = w2m
    out["disk2_rho"] = d2.density(r, thm, ph)
    # Ulrich envelope with a 20 degree cavity on log-r cells over 0.1-1e4 au
    e1 = np.logspace(-1, 4, 65)
    e2 = np.linspace(0, np.pi, 65)
    er, eth = 0.5 * (e1[1:] + e1[:-1]), 0.5 * (e2[1:] + e2[:-1])
    e = env.UlrichEnvelopeExtended(mass=0.05, rmin=0.1, rmax=1e4, rcent=100.0, cavpl=1.0,
                                   cavrfact=0.2, theta_open=20.0, zoffset=1.0)
    out["env_w1"], out["env_w2"] = e1, e2
    out["env_rho"] = e.density(er, eth, ph)
    # stars
    s = star.Star(mass=0.5, luminosity=0.9064, temperature=4000.0)
    out["star_radius_rsun"] = np.array([s.radius])
    out["constants"] = np.array([const.astronomy.AU, const.astronomy.M_sun,
                                 const.astronomy.R_sun, const.astronomy.L_sun,
                                 const.physics.sigma, const.physics.h, const.physics.k,
                                 const.physics.c, const.astronomy.pc, const.astronomy.Jy,
                                 const.math.pi])
    path = os.path.join(HERE, "pdspy_builders.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, {k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main()
