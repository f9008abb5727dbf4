"""Batched log-probability of an MCMC ensemble on one GPU.

pdspy fits a model by emcee: ``lnprob`` (pdspy/utils/emcee.py:183-203) = ``lnprior``
(:64-150) + ``lnlike`` (:6-61), evaluated one walker at a time, each walker running
``run_disk_model`` (pdspy/modeling/run_disk_model.py: parameters :39-56, model set-up
:112-205, the RADMC-3D thermal run :251-255, images and galario sampling per visibility
set :285-330) in its own process (bin/disk_model_emcee3.py:177-184 farms the walkers
over an MPI pool).  ``lnprob_batched`` evaluates a whole ensemble in one go:

  1. every walker's parameters are resolved as run_disk_model does and its prior checked;
  2. the models of the walkers with a finite prior are built with the device density
     builders (``builders``) on run_disk_model's grid (set_spherical_grid(R_in, R_grid,
     100, 101, 2): 99 x 100 x 1 cells, theta mirrored, R_grid = R_env with an envelope,
     else 5 R_disk);
  3. ONE batched thermal launch (``thermal.run_thermal_batched``) computes all their
     temperatures with run_disk_model's settings (1e6 packets, MRW gamma 2, tauthres 10,
     count trigger 100); a walker whose run times out gets -inf, as run_disk_model's
     TimeoutExpired branch returns 0 and lnlike then -inf;
  4. per walker and visibility set: the image at the set's wavelength (``image``), scaled
     by flux_unc, sampled at the data's (u, v) by the gridded FFT (``vis.VisFFT``,
     galario's method) with the (x0, y0) offset, and lnlike's visibility term.

Scope: the "truncated" power-law disk with an optional "ulrich-extended" envelope (its
centrifugal radius = R_disk, as YSOModel does unless rcent_ne_rdisk), lnlike's visibility,
image (beam-convolved model images) and SED (free-free added, reddened, log10) terms, and
one dust model for disk and envelope (pdspy's DustGenerator tables are not available).  The
free-free point source run_disk_model adds to the real part of the visibilities
(:325-334, pdspy/spectroscopy/freefree.py, interferometry/model.py:102-104) is added the
same way.
"""
import subprocess

import numpy as np
import torch

from . import builders, image, thermal, vis
from .constants import arcsec, c as C_LIGHT
from .modeling import Model, Star

# run_disk_model's thermal settings (run_disk_model.py:251-255)
THERMAL = dict(modified_random_walk=True, mrw_gamma=2, mrw_tauthres=10, mrw_count_trigger=100)


def base_parameters():
    """pdspy's default parameter table (pdspy/modeling/base_parameters.py) for the keys of
    this model family: every entry fixed at pdspy's default value and limits."""
    def e(v, lo, hi, **kw):
        return dict(fixed=True, value=v, limits=[lo, hi], **kw)
    return {
        "logM_star": e(0.0, -1., 1.), "T_star": e(4000., 500., 10000.),
        "logL_star": e(0.0, -1., 2.), "disk_type": e("truncated", 0., 0.),
        "logM_disk": e(-4., -10., -2.5), "logR_in": e(-1., -1., 4.), "logR_disk": e(2., 0., 4.),
        "h_0": e(0.1, 0.01, 0.5), "gamma": e(1.0, -0.5, 2.0), "beta": e(1.0, 0.5, 1.5),
        "envelope_type": e("none", 0., 0.), "logM_env": e(-3., -10., -2.),
        "logR_env": e(3., 2., 5.), "logR_c": e("logR_disk", -1., 4.), "f_cav": e(0.5, 0., 1.),
        "ksi": e(1.0, 0.5, 1.5), "theta_open": e("45", 0., 90.), "zoffset": e(1, 0., 5.),
        "i": e(45., 0., 180.), "pa": e(0., 0., 360.), "x0": e(0., -0.1, 0.1),
        "y0": e(0., -0.1, 0.1), "dpc": e(140., 1., 1e6, prior="box", sigma=0.),
        "flux_unc1": e(1., 0.5, 1.5, prior="box", sigma=0.),
        "logF_nu_ff": e(-20., -30., 0.), "lognu_turn": e(0., -1., 2.), "pl_turn": e(0.6, 0., 2.),
        "Ak": e(0., 0., 1.),
    }


def resolve(params, parameters):
    """run_disk_model's parameter dictionary (run_disk_model.py:39-56): fixed values (or
    the value of the parameter they name), free values from ``params``, 10**x for every
    "log" key, alpha = gamma + beta."""
    p = {}
    for key in parameters:
        if parameters[key]["fixed"]:
            v = parameters[key]["value"]
            if isinstance(v, str) and v in parameters:
                v = parameters[v]["value"] if parameters[v]["fixed"] else params[v]
        else:
            v = params[key]
        p[key] = v
        if key[:3] == "log":
            p[key[3:]] = 10.0 ** float(v)
    p["alpha"] = p["gamma"] + p["beta"]
    return p


def free_keys(parameters):
    return [k for k in sorted(parameters) if not parameters[k]["fixed"]]


def lnprior(params, parameters, priors, nvis):
    """pdspy's lnprior (utils/emcee.py:64-150) for the parameters this family has."""
    for key in parameters:
        if not parameters[key]["fixed"]:
            lo, hi = parameters[key]["limits"]
            if not lo <= params[key] <= hi:
                return -np.inf

    def val(k):
        return params[k] if k in params else parameters[k]["value"]

    R_in, R_disk, R_env = (10.0 ** float(val(k)) for k in ("logR_in", "logR_disk", "logR_env"))
    if not R_in <= R_disk <= R_env:
        return -np.inf
    if "logR_env" in params and "logM_env" in params:
        if params["logR_env"] < 0.5 * params["logM_env"] + 4.0:
            return -np.inf
    lp = 0.0
    for i in range(nvis):
        k = "flux_unc%d" % (i + 1)
        if k in parameters and not parameters[k]["fixed"] and \
                parameters[k].get("prior") == "gaussian":
            lp += -0.5 * (params[k] - parameters[k]["value"]) ** 2 / parameters[k]["sigma"] ** 2
    if "dpc" in parameters and not parameters["dpc"]["fixed"]:
        if "parallax" in priors:
            plx = 1.0 / params["dpc"] * 1000
            lp += -0.5 * (plx - priors["parallax"]["value"]) ** 2 / priors["parallax"]["sigma"] ** 2
        elif "dpc" in priors:
            lp += -0.5 * (params["dpc"] - priors["dpc"]["value"]) ** 2 / priors["dpc"]["sigma"] ** 2
    return lp


def build_model(p, dust, lam_um, device):
    """The walker's Model: star, run_disk_model's grid, disk (+ envelope) densities from
    the device builders."""
    m = Model()
    m.grid.add_star(Star(mass=p.get("M_star", 1.0), luminosity=p["L_star"],
                         temperature=p["T_star"]))
    env = p.get("envelope_type", "none") == "ulrich-extended"
    R_grid = p["R_env"] if env else 5 * p["R_disk"]
    r = np.logspace(np.log10(p["R_in"]), np.log10(R_grid), 100)
    th = np.linspace(0.0, np.pi / 2, 101)
    ph = np.linspace(0.0, 2 * np.pi, 2)
    m.grid.set_spherical_grid(r, th, ph)
    m.grid.lam = lam_um
    g = m.grid
    rho = builders.disk_density(g.r, g.theta, g.phi, p["M_disk"], p["R_in"], p["R_disk"],
                                p["alpha"], p["h_0"], p["beta"], device=device)
    g.add_density(rho.cpu().numpy(), dust)
    if env:
        rho = builders.ulrich_envelope_density(g.r, g.theta, g.phi, p["M_env"], p["R_in"],
                                               p["R_env"], p["R_disk"], p["ksi"], p["f_cav"],
                                               float(p["theta_open"]), p["zoffset"],
                                               device=device)
        g.add_density(rho.cpu().numpy(), dust)
    return m


def freefree(nu, F_nu_ff, nu_turn, pl_turn):
    """pdspy's free-free spectrum (pdspy/spectroscopy/freefree.py:3-17), Jy."""
    nu = np.asarray(nu, dtype=np.float64)
    flux = np.where(nu < nu_turn, F_nu_ff * (nu / nu_turn) ** pl_turn,
                    F_nu_ff * (nu / nu_turn) ** -0.1)
    return np.where(nu > 1.0e13, 0.0, flux)


def freefree_real(u, v, freq, p):
    """Real part of the free-free point source at (x0, y0) run_disk_model adds to the model
    visibilities (run_disk_model.py:325-334; point_model, interferometry/model.py:102-104,
    with its 3.14159)."""
    f = float(freefree(np.mean(freq), p.get("F_nu_ff", 0.0), p.get("nu_turn", 1.0) * 1e9,
                       p.get("pl_turn", 0.6)))
    x0 = float(p.get("x0", 0.0)) * arcsec
    y0 = float(p.get("y0", 0.0)) * arcsec
    return f * np.cos(2 * 3.14159 * (np.asarray(u) * x0 + np.asarray(v) * y0))


def gaussian_beam(bmaj, bmin, bpa, pixelsize):
    """The beam run_disk_model convolves model images with (run_disk_model.py:468-472):
    pdspy's misc.gaussian2d (misc/gaussian2d.py:3-8) on a 512 x 512 pixel grid, sigmas
    bmaj/2.355 and bmin/2.355 in pixels, position angle (90 - bpa) degrees, peak 1."""
    x, y = np.meshgrid(np.linspace(-256, 255, 512), np.linspace(-256, 255, 512))
    sx = bmaj / 2.355 / pixelsize
    sy = bmin / 2.355 / pixelsize
    pa = (90 - bpa) * np.pi / 180.
    xp = x * np.cos(pa) - y * np.sin(pa)
    yp = x * np.sin(pa) + y * np.cos(pa)
    return np.exp(-1 * xp ** 2 / (2 * sx ** 2)) * np.exp(-1 * yp ** 2 / (2 * sy ** 2))


def convolve_same(plane, kernel, device=None):
    """scipy.signal.fftconvolve(plane, kernel, mode="same") in float64 with torch.fft on
    ``device``: the linear convolution through zero-padded transforms, cropped to the
    plane's shape about the centre of the full result."""
    dev = torch.device("cuda", torch.cuda.current_device()) if device is None else device
    a = torch.as_tensor(np.asarray(plane, dtype=np.float64), device=dev)
    k = torch.as_tensor(np.asarray(kernel, dtype=np.float64), device=dev)
    full = (a.shape[0] + k.shape[0] - 1, a.shape[1] + k.shape[1] - 1)
    f = torch.fft.irfft2(torch.fft.rfft2(a, s=full) * torch.fft.rfft2(k, s=full), s=full)
    y0 = (full[0] - a.shape[0]) // 2
    x0 = (full[1] - a.shape[1]) // 2
    return f[y0:y0 + a.shape[0], x0:x0 + a.shape[1]].cpu().numpy()


def redden(wave_um, flux, Av, law=None):
    """pdspy's dust.redden (dust/redden.py:6-63): flux / 10**(Av coeff / 2.5) with coeff the
    extinction law interpolated linearly in log-log (extrapolated from the end segments).
    ``law`` = (wavelengths in um, coefficients) of the tabulated law pdspy reads from its
    data files (McClure 2009 for run_disk_model); with Av = 0 the flux passes unchanged and
    no table is needed."""
    flux = np.asarray(flux, dtype=np.float64)
    if Av == 0:
        return flux / 10. ** (0. * np.ones_like(flux) / 2.5)
    if law is None:
        raise ValueError("redden: Av = %g needs the extinction law table (wavelengths, "
                         "coefficients)" % Av)
    lw = np.log10(np.asarray(law[0], dtype=np.float64))
    lc = np.log10(np.asarray(law[1], dtype=np.float64))
    order = np.argsort(lw)
    lw, lc = lw[order], lc[order]
    x = np.log10(np.asarray(wave_um, dtype=np.float64))
    y = np.interp(x, lw, lc)
    lo, hi = x < lw[0], x > lw[-1]
    y[lo] = lc[0] + (lc[1] - lc[0]) / (lw[1] - lw[0]) * (x[lo] - lw[0])
    y[hi] = lc[-2] + (lc[-1] - lc[-2]) / (lw[-1] - lw[-2]) * (x[hi] - lw[-2])
    return flux / 10. ** (Av * 10. ** y / 2.5)


def model_image(m, p, img_set, device):
    """run_disk_model's model image for one image data set (run_disk_model.py:457-476):
    run_image at the set's wavelength (1e5 scattering packets, mc_scat_maxtauabs 5),
    convolved with the set's beam; returns the Image.  (The reference reads the beam's
    second pixel size from an undefined name, ``image["pixelsize"]``; the set's pixel size
    is used for both axes here.)"""
    lam = img_set["lam"]
    im = image.run_image(m, name=lam, nphot=1e5, npix=int(img_set["npix"]),
                         pixelsize=float(img_set["pixelsize"]),
                         lam=[float(lam)], incl=p["i"], pa=p["pa"], dpc=p["dpc"],
                         mc_scat_maxtauabs=5)
    beam = gaussian_beam(img_set["bmaj"], img_set["bmin"], img_set["bpa"],
                         float(img_set["pixelsize"]))
    im.image = convolve_same(im.image[:, :, 0, 0], beam, device).reshape(im.image.shape)
    return im


def model_sed(m, p, spectrum, extinction_law=None):
    """run_disk_model's model SED (run_disk_model.py:480-504): run_sed at the data's
    wavelengths (1e4 packets, scattering at every wavelength, mc_scat_maxtauabs 5), plus the
    free-free spectrum, reddened by A_k, as log10 flux."""
    m.set_camera_wavelength(np.asarray(spectrum.wave, dtype=np.float64))
    sed = image.run_sed(m, name="SED", nphot=1e4, loadlambda=True, incl=p["i"], pa=p["pa"],
                        dpc=p["dpc"], camera_scatsrc_allfreq=True, mc_scat_maxtauabs=5)
    sed.flux = sed.flux + freefree(sed.freq, p.get("F_nu_ff", 0.0), p.get("nu_turn", 1.0) * 1e9,
                                   p.get("pl_turn", 0.6))
    sed.flux = redden(sed.wave, sed.flux, p.get("Ak", 0.0), law=extinction_law)
    sed.flux = np.log10(sed.flux)
    return sed


def _lnlike_vis(re, im, data):
    """lnlike's visibility term (utils/emcee.py:31-43), numerically as pdspy writes it."""
    w = data.weights
    good = w > 0
    norm = np.sum(np.log(w[good] / (2 * np.pi)))
    return (-0.5 * np.sum((data.real - re) ** 2 * w) - norm +
            -0.5 * np.sum((data.imag - im) ** 2 * w) - norm)


def model_visibilities(m, p, vis_set, device, pad=2, nphot_image=1e5):
    """Model visibilities (re, im) of walker m for one visibility set: run_image at the
    set's wavelength with run_disk_model's settings (npix, pixelsize, incl i, pa, dpc,
    1e5 scattering packets, mc_scat_maxtauabs 5; run_disk_model.py:299-306), times flux_unc,
    sampled with the (x0, y0) offset.  One frequency channel per set (continuum data)."""
    data = vis_set["data"]
    lam_um = C_LIGHT / np.atleast_1d(data.freq)[0] / 1.0e-4
    npix, pixelsize = int(vis_set["npix"]), float(vis_set["pixelsize"])
    img = image.run_image(m, name="vis", nphot=nphot_image, npix=npix, pixelsize=pixelsize,
                          lam=[lam_um], incl=p["i"], pa=p["pa"], dpc=p["dpc"],
                          mc_scat_maxtauabs=5)
    scale = float(p.get("flux_unc%d" % vis_set["index"], 1.0))
    plane = torch.as_tensor(img.image[:, :, 0, 0] * scale, dtype=torch.float32, device=device)
    geo = vis.pixel_grid(npix, pixelsize)
    geo = (geo[0] + float(p.get("x0", 0.0)) * arcsec, geo[1],
           geo[2] + float(p.get("y0", 0.0)) * arcsec, geo[3])
    u = torch.as_tensor(data.u, dtype=torch.float32, device=device)
    v = torch.as_tensor(data.v, dtype=torch.float32, device=device)
    re, im = vis.VisFFT.apply(plane, u, v, geo, pad)
    re = re.cpu().numpy() + freefree_real(data.u, data.v, data.freq, p)
    return re, im.cpu().numpy()


def lnprob_batched(P, visibilities, parameters, priors=None, dust=None, lam_um=None,
                   nphot=1e6, device=None, pad=2, timelimit=3600.0, seed=0, images=None,
                   spectra=None, extinction_law=None):
    """lnprob of every walker (rows of P, the free parameters in sorted key order as
    pdspy's lnprob orders them) with one batched thermal launch; returns float64 [nwalker].

    timelimit: seconds of device time per walker (one number or one per row of P); a
    walker whose thermal run has not finished in time scores -inf alone.

    images: list of dicts with "data" (an Image with ``image`` and ``unc``), "npix",
    "pixelsize", "lam", "bmaj", "bmin", "bpa" (pdspy's images[...][j]); spectra: dict with
    "total" (a Spectrum of log10 flux with ``unc`` at the data wavelengths).  They add
    lnlike's image and SED terms (utils/emcee.py:45-58).  extinction_law: the (wavelength
    um, coefficient) table redden needs when A_k is not 0.

    visibilities: list of dicts with "data" (vis.UVData plus ``freq``), "npix" and
    "pixelsize" (arcsec), one per visibility set (pdspy's visibilities["data"][j],
    ["npix"][j], ["pixelsize"][j])."""
    from .workloads import analytic_dust, lam_grid
    priors = priors or {}
    dev = device or torch.device("cuda", torch.cuda.current_device())
    lam_um = lam_grid() if lam_um is None else lam_um
    dust = analytic_dust(lam_um) if dust is None else dust
    keys = free_keys(parameters)
    out = np.full(len(P), -np.inf)
    live, models, res, lps = [], [], [], []
    for w, row in enumerate(P):
        params = dict(zip(keys, [float(x) for x in row]))
        lp = lnprior(params, parameters, priors, len(visibilities))
        if not np.isfinite(lp):
            continue
        p = resolve(params, parameters)
        live.append(w)
        models.append(build_model(p, dust, lam_um, dev))
        res.append(p)
        lps.append(lp)
    if not models:
        return out
    # each walker has its own time limit (run_disk_model.py:251-273): a walker that runs out
    # of time scores -inf alone (utils/emcee.py:22-23), the others are scored as usual
    limits = timelimit
    if limits is not None and np.ndim(limits) > 0:
        limits = [np.asarray(limits, dtype=object)[w] for w in live]   # one per walker of P
    try:
        thermal.run_thermal_batched(models, nphot=nphot, iseed=seed, model_timelimit=limits,
                                    **THERMAL)
    except subprocess.TimeoutExpired:
        return out
    for w, m, p, lp in zip(live, models, res, lps):
        if m.grid.temperature is None:
            continue
        ll = 0.0
        for j, vs in enumerate(visibilities):
            vs = dict(vs, index=j + 1)
            re, im = model_visibilities(m, p, vs, dev, pad=pad)
            ll += _lnlike_vis(re, im, vs["data"])
        for img_set in images or []:
            mi = model_image(m, p, img_set, dev)
            d = img_set["data"]
            ll += -0.5 * (np.sum((d.image - mi.image) ** 2 / d.unc ** 2))
        if spectra and "total" in spectra:
            sed = model_sed(m, p, spectra["total"], extinction_law)
            d = spectra["total"]
            ll += -0.5 * (np.sum((d.flux - sed.flux) ** 2 / d.unc ** 2))
        out[w] = lp + ll
    return out
