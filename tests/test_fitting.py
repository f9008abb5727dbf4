"""Parameter resolution, priors and model set-up of the batched lnprob (CPU): pdspy's
run_disk_model.py:39-56 and utils/emcee.py:64-150."""
import numpy as np
import torch

from pdspy_gb300 import fitting
from tests.test_fitting_gpu import parameters


def test_resolve_follows_run_disk_model():
    P = parameters()
    P["logR_c"] = {"fixed": True, "value": "logR_disk", "limits": [-1., 4.]}
    p = fitting.resolve({"h_0": 0.1, "i": 40.0, "logM_disk": -3.0}, P)
    assert p["M_disk"] == 10.0 ** -3.0 and p["R_disk"] == 10.0 ** 1.5
    assert p["logR_c"] == 1.5 and p["R_c"] == 10.0 ** 1.5      # a fixed value naming a key
    assert p["alpha"] == p["gamma"] + p["beta"]
    assert p["theta_open"] == "45"


def test_lnprior_radii_and_density_checks():
    P = parameters()
    assert fitting.lnprior({"h_0": 0.1, "i": 40.0, "logM_disk": -3.0}, P, {}, 1) == 0.0
    assert fitting.lnprior({"h_0": 0.6, "i": 40.0, "logM_disk": -3.0}, P, {}, 1) == -np.inf
    Q = dict(P, logR_disk={"fixed": True, "value": 3.5, "limits": [0., 4.]})
    assert fitting.lnprior({"h_0": 0.1, "i": 40.0, "logM_disk": -3.0}, Q, {}, 1) == -np.inf


def test_build_model_grid_and_densities():
    P = parameters()
    P["envelope_type"] = {"fixed": True, "value": "ulrich-extended", "limits": [0., 0.]}
    p = fitting.resolve({"h_0": 0.1, "i": 40.0, "logM_disk": -3.0}, P)
    from pdspy_gb300.workloads import analytic_dust, lam_grid
    lam = lam_grid()
    m = fitting.build_model(p, analytic_dust(lam), lam, torch.device("cpu"))
    g = m.grid
    assert len(g.w1) == 100 and len(g.w2) == 101 and len(g.w3) == 2
    assert np.isclose(g.w1[-1], p["R_env"]) and np.isclose(g.w2[-1], np.pi / 2)
    assert len(g.density) == 2 and g.density[0].shape == (99, 100, 1)
    assert np.all(g.density[1] >= 0) and g.density[1].max() > 0


def test_lnlike_visibility_term_as_pdspy_writes_it():
    """utils/emcee.py:31-43: -0.5 sum (Re_d - Re_m)^2 w - sum log(w_good / 2 pi), the same
    for Im, zero-weight points excluded from the log terms."""
    from pdspy_gb300 import vis
    rng = np.random.default_rng(4)
    n = 50
    w = rng.uniform(1.0, 5.0, n)
    w[:5] = 0.0
    d = vis.UVData(rng.normal(size=n), rng.normal(size=n), rng.normal(size=n),
                   rng.normal(size=n), w)
    re, im = rng.normal(size=n), rng.normal(size=n)
    good = w > 0
    expect = (-0.5 * np.sum((d.real - re) ** 2 * w) - np.sum(np.log(w[good] / (2 * np.pi))) +
              -0.5 * np.sum((d.imag - im) ** 2 * w) - np.sum(np.log(w[good] / (2 * np.pi))))
    assert fitting._lnlike_vis(re, im, d) == expect


def test_freefree_matches_pdspy_formula():
    """pdspy/spectroscopy/freefree.py:3-17 and the point source of
    interferometry/model.py:102-104 (real part)."""
    nu = np.array([1e8, 1e9, 3e10, 2e13])
    F, nt, pl = 1e-3, 5e9, 0.6
    expect = np.where(nu < nt, F * (nu / nt) ** pl, F * (nu / nt) ** -0.1)
    expect = np.where(nu > 1e13, 0.0, expect)
    assert np.array_equal(fitting.freefree(nu, F, nt, pl), expect)
    p = {"F_nu_ff": F, "nu_turn": 5.0, "pl_turn": pl, "x0": 0.02, "y0": -0.01}
    u, v = np.array([1e5, -3e5]), np.array([2e5, 4e4])
    from pdspy_gb300.constants import arcsec
    ff = fitting.freefree(2.3e11, F, 5e9, pl)
    pt = ff * np.exp(-2 * 3.14159 * (0 + 1j * (u * 0.02 * arcsec + v * -0.01 * arcsec)))
    assert np.allclose(fitting.freefree_real(u, v, [2.3e11], p), pt.real, rtol=1e-14)


def test_beam_convolution_matches_scipy_fftconvolve():
    """run_disk_model's beam convolution (run_disk_model.py:468-476): the beam of pdspy's
    gaussian2d on the 512 x 512 grid, and fftconvolve(..., mode="same") of a model plane."""
    import scipy.signal
    beam = fitting.gaussian_beam(0.12, 0.08, 30.0, 0.02)
    assert beam.shape == (512, 512) and beam.max() == 1.0
    rng = np.random.default_rng(2)
    for shape in [(64, 64), (63, 80)]:
        plane = rng.random(shape)
        got = fitting.convolve_same(plane, beam, device=torch.device("cpu"))
        ref = scipy.signal.fftconvolve(plane, beam, mode="same")
        assert got.shape == ref.shape
        assert np.abs(got - ref).max() <= 1e-10 * np.abs(ref).max()


def test_redden_follows_pdspy():
    """dust.redden (dust/redden.py:6-63): identity at A = 0, otherwise the law interpolated
    in log-log with extrapolation, as interp1d(fill_value="extrapolate") does."""
    from scipy.interpolate import interp1d
    wave = np.logspace(-0.5, 3.5, 40)
    flux = np.logspace(-3, 1, 40)
    assert np.array_equal(fitting.redden(wave, flux, 0.0), flux)
    lw = np.array([1.0, 2.2, 5.0, 20.0, 100.0])
    lc = np.array([7.0, 1.0, 0.45, 0.3, 0.05])
    got = fitting.redden(wave, flux, 0.4, law=(lw, lc))
    f = interp1d(np.log10(lw), np.log10(lc), fill_value="extrapolate")
    ref = flux / 10. ** (0.4 * 10. ** f(np.log10(wave)) / 2.5)
    assert np.allclose(got, ref, rtol=1e-12, atol=0)
