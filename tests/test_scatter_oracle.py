"""Scattering Monte Carlo oracle: known answers for the mean intensity J (CPU only).

The oracle restates the monochromatic scattering Monte Carlo of RADMC-3D's image and
spectrum modes (pdspy/modeling/Model.py:258-322, :515-577; mc_scat_maxtauabs from
pdspy/radmc3d/write.py:141-142).  With no RADMC-3D to compare against, it is pinned by
cases with closed-form answers:
  - an optically thin shell around a point source: J averaged over a shell is
    L (r1 - r0) 3 / (16 pi^2 (r1^3 - r0^3));
  - a pure absorber of uniform opacity: the same times the attenuation e^-tau(r)
    integrated over the shell;
  - uniform thermal emission in an optically thin ball of radius R: sum_c 4 pi J_c V_c
    = L_dust <chord> with the mean chord from a uniform point of a ball to its surface
    along a random direction, 3R/4;
  - no absorption: every packet escapes, however thick the scattering medium.
"""
import numpy as np
import pytest

from oracle import orc

AU = 1.495978707e13
R_SUN = 6.957e10
R_STAR, T_STAR = 2.0 * R_SUN, 4000.0


def planck(nu, T):
    h, k, c = 6.6260755e-27, 1.380658e-16, 2.99792458e10
    return 2 * h * nu ** 3 / c ** 2 / np.expm1(h * nu / (k * T))


def _shell_grid(nr=20, nt=10, rin=1.0, rout=100.0, nphi=1, mirror=True):
    r = np.logspace(np.log10(rin), np.log10(rout), nr + 1) * AU
    th = np.linspace(0.0, np.pi / 2 if mirror else np.pi, nt + 1)
    ph = np.linspace(0.0, 2.0 * np.pi, nphi + 1)
    Vr = (r[1:] ** 3 - r[:-1] ** 3) / 3.0
    Vt = (2.0 if mirror else 1.0) * (np.cos(th[:-1]) - np.cos(th[1:]))
    V = Vr[:, None, None] * Vt[None, :, None] * np.diff(ph)[None, None, :]
    return r, th, ph, V.reshape(nr, -1)


def _lstar(lam):
    nu = 2.99792458e10 / (np.asarray(lam) * 1e-4)
    return 4.0 * np.pi ** 2 * R_STAR ** 2 * planck(nu, T_STAR)


def _shell_mean(J, V, nl):
    J = J.reshape((nl,) + V.shape)
    return (J * V[None]).sum(2) / V.sum(1)[None]


def test_math_helpers_accuracy():
    xs = np.linspace(0.0, 86.0, 3001).astype(np.float32)
    e = np.array([orc.expm(float(x)) for x in xs])
    assert np.max(np.abs(e / np.exp(-xs.astype(np.float64)) - 1)) < 2e-7
    assert orc.expm(0.0) == 1.0 and orc.expm(90.0) == 0.0
    xs = np.logspace(-8, 2, 1001).astype(np.float32)
    f = np.array([orc.expm_frac(float(x), orc.expm(float(x))) for x in xs])
    ref = -np.expm1(-xs.astype(np.float64)) / xs.astype(np.float64)
    assert np.max(np.abs(f / ref - 1)) < 1e-6
    xs = np.logspace(-9, 0, 1001).astype(np.float32)
    c = np.array([orc.cbrt01(float(x)) for x in xs])
    assert np.max(np.abs(c / np.cbrt(xs.astype(np.float64)) - 1)) < 3e-7


@pytest.mark.parametrize("nphi,mirror", [(1, True), (6, False)])
def test_thin_shell_point_source(nphi, mirror):
    r, th, ph, V = _shell_grid(nphi=nphi, mirror=mirror)
    lam = np.array([1.0, 3.0])
    ncell = V.size
    o = orc.mcscat(r, th, ph, np.full((1, ncell), 1e-25), lam, np.zeros((1, 2)),
                   np.ones((1, 2)), R_STAR, T_STAR, 20000, seed=1)
    assert o["stats"]["escaped"] == 40000 and o["stats"]["dropped"] == 0
    r0, r1 = r[:-1], r[1:]
    expect = _lstar(lam)[:, None] * (r1 - r0)[None] * 3 / (16 * np.pi ** 2 * (r1 ** 3 - r0 ** 3))[None]
    got = _shell_mean(o["J"], V, 2)
    # every packet crosses every shell once, radially: only fixed-point rounding remains
    assert np.allclose(got, expect, rtol=1e-6)


def test_pure_absorber_attenuation():
    r, th, ph, V = _shell_grid()
    lam = np.array([1.0, 3.0])
    ncell = V.size
    rho = np.full((1, ncell), 1e-15)
    ka = np.array([[1.0, 2.0]])
    o = orc.mcscat(r, th, ph, rho, lam, ka, np.zeros((1, 2)), R_STAR, T_STAR, 20000, seed=2)
    assert o["stats"]["scatterings"] == 0 and o["stats"]["dropped"] == 0
    r0, r1 = r[:-1], r[1:]
    a = (np.float32(1e-15) * np.float32(1.0) * np.array([1.0, 2.0]))[:, None]
    tau0 = a * (r0 - r[0])[None]
    expect = _lstar(lam)[:, None] * np.exp(-tau0) * -np.expm1(-a * (r1 - r0)[None]) / a * \
        3 / (16 * np.pi ** 2 * (r1 ** 3 - r0 ** 3))[None]
    assert np.allclose(_shell_mean(o["J"], V, 2), expect, rtol=2e-6)


def test_maxtauabs_drops_packets():
    r, th, ph, V = _shell_grid()
    ncell = V.size
    rho = np.full((1, ncell), 1e-15)
    o = orc.mcscat(r, th, ph, rho, [1.0], [[3.0]], [[0.0]], R_STAR, T_STAR, 2000,
                   maxtauabs=2.0)
    # tau from the inner edge to r is a (r - r_in); the cut at 2 falls inside the grid
    assert o["stats"]["dropped"] == 2000 and o["stats"]["escaped"] == 0
    J = o["J"].reshape(V.shape)
    a = np.float32(1e-15) * np.float32(3.0)
    beyond = (r[:-1] - r[0]) * a > 2.0 + 1e-6
    assert np.all(J[beyond] == 0) and np.all(J[~beyond] > 0)


def test_thin_ball_uniform_emission():
    rr = np.logspace(-2, 2, 41) * AU
    th = np.linspace(0.0, np.pi / 2, 11)
    ph = np.array([0.0, 2.0 * np.pi])
    Vr = (rr[1:] ** 3 - rr[:-1] ** 3) / 3.0
    V = Vr[:, None] * (2.0 * (np.cos(th[:-1]) - np.cos(th[1:])))[None] * 2.0 * np.pi
    emis = np.full((2, V.size), 1e-20)
    o = orc.mcscat(rr, th, ph, np.full((1, V.size), 1e-25), [1.0, 3.0], np.zeros((1, 2)),
                   np.ones((1, 2)), [], [], 40000, emis=emis, seed=3)
    J = o["J"].reshape((2,) + V.shape)
    Ld = (emis.reshape(J.shape) * V[None] * 4 * np.pi).sum((1, 2))
    total = (4 * np.pi * J * V[None]).sum((1, 2))
    assert np.allclose(total / (Ld * 0.75 * rr[-1]), 1.0, atol=0.015)


def test_conservative_scattering_all_escape_and_deterministic():
    r, th, ph, V = _shell_grid(nr=10, nt=6)
    ncell = V.size
    rho = np.full((1, ncell), 1e-14)
    args = (r, th, ph, rho, [1.0], [[0.0]], [[1.0]], R_STAR, T_STAR, 3000)
    a = orc.mcscat(*args, seed=5, nthreads=1)
    b = orc.mcscat(*args, seed=5, nthreads=4)
    assert a["stats"]["escaped"] == 3000 and a["stats"]["scatterings"] > 3000
    assert np.array_equal(a["acc"], b["acc"]) and np.array_equal(a["J"], b["J"])
    c = orc.mcscat(*args, seed=6)
    assert not np.array_equal(a["acc"], c["acc"])


def test_rejects_invalid_input():
    r, th, ph, V = _shell_grid(nr=4, nt=3)
    with pytest.raises(ValueError):
        orc.mcscat(r, th, ph, np.zeros((1, V.size)), [1.0], [[0.0]], [[1.0]], R_STAR, T_STAR, 0)
