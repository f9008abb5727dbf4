"""Batched MCMC log-probability (pdspy/utils/emcee.py lnprob/lnprior/lnlike over
run_disk_model.py) on the GPU: one batched thermal launch for the ensemble."""
import numpy as np
import pytest
import torch

from pdspy_gb300 import fitting, vis

pytestmark = pytest.mark.gpu


def parameters():
    """pdspy's defaults with h_0, i and logM_disk free (a 31 au disk, inclined and offset)."""
    P = fitting.base_parameters()
    for k in ("h_0", "i", "logM_disk"):
        P[k]["fixed"] = False
    P["logR_disk"]["value"] = 1.5
    P["beta"]["value"] = 1.1
    P["pa"]["value"] = 30.
    P["x0"]["value"] = 0.01
    P["y0"]["value"] = -0.02
    return P


def test_lnprob_batched_orders_walkers(cuda):
    P = parameters()
    keys = fitting.free_keys(P)
    assert keys == ["h_0", "i", "logM_disk"]
    truth = [0.1, 40.0, -3.0]
    npix, pixelsize = 64, 0.02
    # data: the truth's own model visibilities (noise-free), 1 mJy errors
    u, v = vis.synthetic_uv(400, seed=3, bmin_klam=10, bmax_klam=1500)
    freq = 2.99792458e10 / 0.13
    dust = None
    p = fitting.resolve(dict(zip(keys, truth)), P)
    from pdspy_gb300 import thermal
    from pdspy_gb300.workloads import analytic_dust, lam_grid
    lam = lam_grid()
    dust = analytic_dust(lam)
    m = fitting.build_model(p, dust, lam, cuda)
    thermal.run_thermal_batched([m], nphot=20000, iseed=5, **fitting.THERMAL)
    data = vis.UVData(u, v, np.zeros(400), np.zeros(400), np.full(400, 1e6), freq=freq)
    vs = dict(data=data, npix=npix, pixelsize=pixelsize, index=1)
    re, im = fitting.model_visibilities(m, p, vs, cuda)
    data.real, data.imag = re, im
    sets = [dict(data=data, npix=npix, pixelsize=pixelsize)]
    walkers = np.array([truth, [0.15, 40.0, -3.0], [0.1, 40.0, -1.0], [0.1, 60.0, -3.2]])
    lp = fitting.lnprob_batched(walkers, sets, P, dust=dust, lam_um=lam, nphot=20000, seed=5,
                                device=cuda)
    assert lp[2] == -np.inf                         # logM_disk beyond its limit
    best = -2 * np.sum(np.log(data.weights / (2 * np.pi)))
    assert lp[0] == pytest.approx(best, rel=1e-12)  # the data's own model: chi^2 = 0
    assert np.isfinite(lp[1]) and np.isfinite(lp[3])
    assert lp[1] < lp[0] and lp[3] < lp[0]
    # a per-walker time limit: walker 3 runs out of time alone and scores -inf; the other
    # walkers' values are unchanged bit for bit
    lp2 = fitting.lnprob_batched(walkers, sets, P, dust=dust, lam_um=lam, nphot=20000, seed=5,
                                 device=cuda, timelimit=[3600.0, 3600.0, 3600.0, 1e-9])
    assert lp2[3] == -np.inf and lp2[2] == -np.inf
    assert lp2[0] == lp[0] and lp2[1] == lp[1]


def test_lnprob_image_and_sed_terms(cuda):
    """lnlike's image and SED terms (utils/emcee.py:45-58): data made from the truth's own
    beam-convolved image and log10 SED give zero chi^2, so the truth's lnprob is the
    visibility optimum; a walker away from the truth scores lower."""
    from pdspy_gb300 import image, thermal
    from pdspy_gb300.workloads import analytic_dust, lam_grid
    P = parameters()
    keys = fitting.free_keys(P)
    truth = [0.1, 40.0, -3.0]
    lam = lam_grid()
    dust = analytic_dust(lam)
    p = fitting.resolve(dict(zip(keys, truth)), P)
    m = fitting.build_model(p, dust, lam, cuda)
    thermal.run_thermal_batched([m], nphot=20000, iseed=5, **fitting.THERMAL)
    u, v = vis.synthetic_uv(200, seed=3, bmin_klam=10, bmax_klam=1500)
    freq = 2.99792458e10 / 0.13
    data = vis.UVData(u, v, np.zeros(200), np.zeros(200), np.full(200, 1e6), freq=freq)
    vs = dict(data=data, npix=64, pixelsize=0.02, index=1)
    re, im = fitting.model_visibilities(m, p, vs, cuda)
    data.real, data.imag = re, im
    img_set = dict(npix=48, pixelsize=0.03, lam="1300", bmaj=0.1, bmin=0.08, bpa=20.0)
    mi = fitting.model_image(m, p, img_set, cuda)
    assert mi.image.shape == (48, 48, 1, 1) and mi.image.max() > 0
    img_set["data"] = image.Image(mi.image.copy(), x=mi.x, y=mi.y, wave=mi.wave,
                                  unc=np.full(mi.image.shape, 1e-3))
    sed_wave = np.array([5.0, 30.0, 300.0, 1300.0])
    sd = fitting.model_sed(m, p, image.Spectrum(wave=sed_wave, flux=np.zeros(4)))
    assert np.all(np.isfinite(sd.flux))
    spectra = {"total": image.Spectrum(wave=sed_wave, flux=sd.flux.copy(), unc=np.full(4, 0.1))}
    sets = [dict(data=data, npix=64, pixelsize=0.02)]
    walkers = np.array([truth, [0.14, 40.0, -3.0]])
    lp = fitting.lnprob_batched(walkers, sets, P, dust=dust, lam_um=lam, nphot=20000, seed=5,
                                device=cuda, images=[img_set], spectra=spectra)
    best = -2 * np.sum(np.log(data.weights / (2 * np.pi)))
    assert lp[0] == pytest.approx(best, rel=1e-12)
    assert np.isfinite(lp[1]) and lp[1] < lp[0]
