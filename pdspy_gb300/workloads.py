"""Synthetic disk models used by the tests and the benchmark.

Each builder returns pdspy-style Model objects (this package's mirror of
pdspy.modeling) built the way a pdspy user would build them: a spherical grid, a
blackbody star, power-law disks / Ulrich envelopes from the density builders, and dust
opacities defined analytically on a log wavelength grid.  No data files are read.
"""
import numpy as np

from .constants import AU, R_sun, L_sun, sigma
from .dust import Dust
from .modeling import Disk, Model, Star, UlrichEnvelopeExtended


def star_luminosity(radius_rsun, temperature):
    """L in L_sun of a blackbody of the given radius (inverse of Star.py:12-13)."""
    return 4 * np.pi * (radius_rsun * R_sun)**2 * sigma * temperature**4 / L_sun


def lam_grid(nlam=100):
    return np.logspace(-1, 4, nlam)


def analytic_dust(lam_um=None, g=0.6):
    """Small-grain dust: kabs = 1e3 cm^2/g below 10 um and 2 (1300 um / lam) beyond; albedo
    0.5 up to 10 um falling log-linearly to 0 at 1 mm; Henyey-Greenstein g."""
    lam_um = lam_grid() if lam_um is None else np.asarray(lam_um, dtype=np.float64)
    kabs = np.where(lam_um < 10.0, 1.0e3, 2.0 * (1300.0 / lam_um))
    alb = np.where(lam_um <= 10.0, 0.5,
                   np.where(lam_um >= 1000.0, 0.0,
                            0.5 * (3.0 - np.log10(lam_um)) / (3.0 - 1.0)))
    ksca = kabs * alb / (1.0 - alb)
    d = Dust()
    d.set_properties(lam_um * 1.0e-4, kabs, ksca, g=None if g is None else np.full_like(kabs, g))
    return d


def large_grain_dust(lam_um=None, g=0.6):
    """Large grains: kabs = 10 cm^2/g flat up to 1 mm and ~ lam^-1 beyond; albedo as the
    small grains."""
    lam_um = lam_grid() if lam_um is None else np.asarray(lam_um, dtype=np.float64)
    kabs = np.where(lam_um <= 1000.0, 10.0, 10.0 * (1000.0 / lam_um))
    alb = np.where(lam_um <= 10.0, 0.5,
                   np.where(lam_um >= 1000.0, 0.0,
                            0.5 * (3.0 - np.log10(lam_um)) / (3.0 - 1.0)))
    ksca = kabs * alb / (1.0 - alb)
    d = Dust()
    d.set_properties(lam_um * 1.0e-4, kabs, ksca, g=None if g is None else np.full_like(kabs, g))
    return d


def _base_model(r_edges_au, ntheta, nphi=1, theta_max=np.pi, lam_um=None, tstar=4000.0,
                rstar=2.0):
    m = Model()
    th = np.linspace(0.0, theta_max, ntheta + 1)
    ph = np.linspace(0.0, 2 * np.pi, nphi + 1)
    m.grid.set_spherical_grid(np.asarray(r_edges_au, dtype=np.float64), th, ph)
    m.grid.lam = lam_grid() if lam_um is None else lam_um
    m.grid.add_star(Star(mass=0.5, luminosity=star_luminosity(rstar, tstar), temperature=tstar))
    return m


def small_disk(nr=100, ntheta=100, mass=1e-4, rin=0.1, rout=100.0, rgrid=100.0, plrho=2.25,
               h0=0.1, plh=1.25, theta_max=np.pi, g=0.6, lam_um=None):
    """Axisymmetric power-law disk around a 4000 K, 2 R_sun star on an nr x ntheta grid
    (log r from rin to rgrid au, theta over [0, theta_max])."""
    m = _base_model(np.logspace(np.log10(rin), np.log10(rgrid), nr + 1), ntheta,
                    theta_max=theta_max, lam_um=lam_um)
    dust = analytic_dust(m.grid.lam, g=g)
    disk = Disk(mass=mass, rmin=rin, rmax=rout, plrho=plrho, h0=h0, plh=plh, dust=dust)
    m.disk = disk
    m.grid.add_density(disk.density(m.grid.r, m.grid.theta, m.grid.phi), dust)
    return m


def disk_envelope(nr=256, ntheta=256, mdisk=1e-2, menv=0.05, renv=1.0e4, rcent=100.0,
                  theta_open=20.0, g=0.6):
    """Disk (as small_disk, heavier) plus an Ulrich envelope with a 20 degree cavity: two
    species, grid log r over [0.1, 1e4] au."""
    m = _base_model(np.logspace(-1, np.log10(renv), nr + 1), ntheta)
    dust = analytic_dust(m.grid.lam, g=g)
    disk = Disk(mass=mdisk, rmin=0.1, rmax=100.0, plrho=2.25, h0=0.1, plh=1.25, dust=dust)
    env = UlrichEnvelopeExtended(mass=menv, rmin=0.1, rmax=renv, rcent=rcent, cavpl=1.0,
                                 cavrfact=0.2, theta_open=theta_open, zoffset=1.0, dust=dust)
    m.disk, m.envelope = disk, env
    m.grid.add_density(disk.density(m.grid.r, m.grid.theta, m.grid.phi), dust)
    m.grid.add_density(env.density(m.grid.r, m.grid.theta, m.grid.phi), dust)
    return m


def walker_params(n=64, seed=0):
    """Disk parameters of n MCMC walkers: log-uniform Mdisk in [1e-5, 1e-2] Msun, Rout in
    [20, 300] au, h0 in [0.03, 0.2], beta in [1.0, 1.3], gamma in [0, 1.5], grid sizes
    nr in 64..256 and ntheta in 64..192."""
    rng = np.random.default_rng(seed)
    return [dict(mass=10 ** rng.uniform(-5, -2), rout=rng.uniform(20, 300),
                 h0=rng.uniform(0.03, 0.2), beta=rng.uniform(1.0, 1.3),
                 gamma=rng.uniform(0.0, 1.5), nr=int(rng.integers(64, 257)),
                 ntheta=int(rng.integers(64, 193))) for _ in range(n)]


def walker_models(n=64, seed=0, g=0.6, scale=1.0):
    """Models of n walkers (grids outer edge 5 Rout as pdspy's run_disk_model.py:122).
    ``scale`` shrinks the grids (for fast tests)."""
    out = []
    for p in walker_params(n, seed):
        nr = max(8, int(p["nr"] * scale))
        nt = max(8, int(p["ntheta"] * scale))
        m = small_disk(nr=nr, ntheta=nt, mass=p["mass"], rin=0.1, rout=p["rout"],
                       rgrid=5 * p["rout"], plrho=p["gamma"] + p["beta"], h0=p["h0"],
                       plh=p["beta"], g=g)
        m.params = p
        out.append(m)
    return out


def walker_model(i, n=64, seed=0, g=0.6):
    """Walker i of walker_models(n, seed)."""
    return walker_models(n=n, seed=seed, g=g)[i]


def spiral_disk(nr=128, ntheta=128, nphi=128, phase=0.0, mass=1e-3, rout=100.0, h0=0.1,
                plh=1.25, plrho=2.25, pitch_deg=15.0, amp=0.3, large_fraction=0.9, g=0.6):
    """3-D disk with a two-armed logarithmic spiral, small grains at h and large grains
    at 0.2 h holding ``large_fraction`` of the mass (two species)."""
    m = _base_model(np.logspace(-1, np.log10(rout), nr + 1), ntheta, nphi=nphi)
    small = analytic_dust(m.grid.lam, g=g)
    large = large_grain_dust(m.grid.lam, g=g)
    d_s = Disk(mass=mass * (1 - large_fraction), rmin=0.1, rmax=rout, plrho=plrho, h0=h0, plh=plh)
    d_l = Disk(mass=mass * large_fraction, rmin=0.1, rmax=rout, plrho=plrho, h0=0.2 * h0, plh=plh)
    rr, tt, pp = np.meshgrid(m.grid.r, m.grid.theta, m.grid.phi, indexing='ij')
    R = rr * np.sin(tt)
    with np.errstate(divide="ignore"):
        pert = 1.0 + amp * np.cos(2 * pp - 2 * np.log(np.maximum(R, 1e-30)) /
                                  np.tan(np.radians(pitch_deg)) - phase)
    m.grid.add_density(d_s.density(m.grid.r, m.grid.theta, m.grid.phi) * pert, small)
    m.grid.add_density(d_l.density(m.grid.r, m.grid.theta, m.grid.phi) * pert, large)
    return m
