"""Ray-traced images and SEDs behind ``Model.run_image`` / ``Model.run_sed`` (code="gb300").

Replaces pdspy's radmc3d branch (pdspy/modeling/Model.py:515-577 and :608-650): instead of
writing the model and a density-weighted mean temperature to RADMC-3D input files
(Model.py:723-825, the mean at :759-769), running ``radmc3d image`` / ``radmc3d spectrum``
(pdspy/radmc3d/run.py:69-289) and reading ``image.out`` (pdspy/radmc3d/read.pyx:25-152),
the per-cell extinction and source function go to device buffers and the CUDA ray tracer
integrates the formal solution.  Results land where the reference puts them:
``model.images[name]`` (an Image with ``image[ny, nx, nlam, 1]`` in Jy/pixel, ``x``/``y``
in arcsec and ``wave`` in cm, Model.py:566-572) and ``model.spectra[name]`` (a Spectrum
with wavelengths in microns and fluxes in Jy at ``dpc``, Model.py:646-648).

The source function is S = [B_nu(T) sum_s rho_s kabs_s + J sum_s rho_s ksca_s] / alpha with
alpha = sum_s rho_s (kabs_s + ksca_s): thermal emission plus, where the dust scatters,
the isotropic scattering of the mean intensity J that the GPU scattering Monte Carlo
(``scatter.ScatterPlan``) computes with ``nphot`` packets per wavelength, as RADMC-3D
does before "radmc3d image" / "radmc3d spectrum" (nphot_scat / nphot_spec,
mc_scat_maxtauabs; pdspy/radmc3d/write.py:33-38, :141-142).  ``scattering_mode_max=0``
switches scattering off as in RADMC-3D.

``RayTrace`` is a ``torch.autograd.Function`` whose backward is the hand-written adjoint
of the ray trace (``pdgpu_image_adjoint``).
"""
import ctypes as C

import numpy as np
import torch

from . import _lib
from .constants import AU, Jy, R_sun, c as C_LIGHT, h as H_PLANCK, k as K_BOLTZ, pc
from .thermal import _stars, grid_arrays, opacity_on_grid


class Image:
    """Mirror of pdspy's imaging.Image container (pdspy/imaging/libimaging.pyx:7-45)."""

    def __init__(self, image=None, x=None, y=None, wave=None, freq=None, unc=None):
        self.image = image
        self.x = x
        self.y = y
        self.unc = unc
        if wave is not None:
            self.wave = wave
            self.freq = C_LIGHT / wave if freq is None else freq
        elif freq is not None:
            self.freq = freq
            self.wave = C_LIGHT / freq


class Spectrum:
    """Mirror of pdspy's spectroscopy.Spectrum (pdspy/spectroscopy/spectroscopy.py:7-19):
    ``wave`` in microns, ``flux`` in Jy."""

    def __init__(self, wave=None, flux=None, unc=None):
        if wave is not None:
            self.wave = wave
            self.freq = C_LIGHT / wave / 1.0e-4
            self.flux = flux
            self.unc = np.zeros(wave.size) if unc is None else unc


def planck_nu(nu, T):
    """B_nu(T) in erg/s/cm^2/Hz/ster (pdspy/misc/B_nu.py:4-6), zero where T <= 0."""
    Tpos = torch.where(T > 0, T, torch.ones_like(T))
    x = H_PLANCK * nu / (K_BOLTZ * Tpos)
    B = (2.0 * H_PLANCK * nu ** 3 / C_LIGHT ** 2) / torch.expm1(torch.clamp(x, max=700.0))
    B = torch.where(x > 700.0, torch.zeros_like(B), B)
    return torch.where(T > 0, B, torch.zeros_like(B))


def mean_temperature(rho, T):
    """Density-weighted mean temperature shared by all species, as pdspy writes it for
    RADMC-3D's image mode (Model.py:759-769): rho = 0 counts as 1e-30."""
    r = torch.where(rho == 0, torch.full_like(rho, 1.0e-30), rho)
    return (r * T).sum(0) / r.sum(0)


def thermal_emissivity(rho, T, kabs, lam_um):
    """sum_s rho_s kabs_s B_nu(Tm) [nlam, ncell] (erg/s/cm^3/Hz/ster) at the density-weighted
    mean temperature Tm pdspy writes for image mode."""
    nu = (C_LIGHT / (torch.as_tensor(lam_um, dtype=rho.dtype, device=rho.device) * 1.0e-4))
    Tm = mean_temperature(rho, T)
    jab = torch.einsum("sl,sc->lc", kabs, rho)
    return planck_nu(nu[:, None], Tm[None, :]) * jab


def source_terms(rho, T, kabs, ksca, lam_um, J=None):
    """(alpha, S) [nlam, ncell] from rho, T [nspec, ncell] and opacities [nspec, nlam];
    J [nlam, ncell] (the mean intensity) adds the isotropic scattering source."""
    alpha = torch.einsum("sl,sc->lc", kabs + ksca, rho)
    emis = thermal_emissivity(rho, T, kabs, lam_um)
    if J is not None:
        emis = emis + torch.einsum("sl,sc->lc", ksca, rho) * J
    safe = torch.where(alpha > 0, alpha, torch.ones_like(alpha))
    S = torch.where(alpha > 0, emis / safe, torch.zeros_like(alpha))
    return alpha, S


def star_flux_1pc(grid, lam_um):
    """Flux of the stars at 1 pc (erg/s/cm^2/Hz): sum pi R^2 B_nu(T*) / pc^2."""
    radius, temp = _stars(grid)
    nu = torch.as_tensor(C_LIGHT / (np.asarray(lam_um, dtype=np.float64) * 1.0e-4))
    f = torch.zeros_like(nu)
    for R, T in zip(radius, temp):
        f = f + np.pi * R * R * planck_nu(nu, torch.full_like(nu, T)) / pc ** 2
    return f.numpy()


def camera_wavelengths(model, lam="1300", loadlambda=False):
    """Camera wavelengths in microns: ``model.camera_wavelength`` when loadlambda is set,
    else the ``lam`` keyword (a string or number in microns, as radmc3d's "lambda")."""
    if loadlambda:
        return np.atleast_1d(np.asarray(model.camera_wavelength, dtype=np.float64))
    if isinstance(lam, str):
        return np.array([float(x) for x in lam.split()], dtype=np.float64)
    return np.atleast_1d(np.asarray(lam, dtype=np.float64))


def opacities(grid, lam_um):
    ka, ks = [], []
    for d in grid.dust:
        a, s, _ = opacity_on_grid(d, lam_um)
        ka.append(a)
        ks.append(s)
    return np.stack(ka), np.stack(ks)


class ImagePlan:
    """One camera over one spherical grid; ``run`` and ``adjoint`` work on device tensors."""

    def __init__(self, grid, npix, pixel_cm, lam_um, incl=0.0, pa=0.0, phi=0.0, nostar=False,
                 max_refine=6, refine_factor=0.5, star_flux=None, device=None):
        self.L = _lib.lib()
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None
                                   else torch.device(device).index or 0)
        r, t, p = grid_arrays(grid)
        self._keep = [np.ascontiguousarray(a, dtype=np.float64) for a in (r, t, p)]
        self.lam_um = np.atleast_1d(np.asarray(lam_um, dtype=np.float64))
        self.nlam = len(self.lam_um)
        if star_flux is None:
            star_flux = star_flux_1pc(grid, self.lam_um) if not nostar else np.zeros(self.nlam)
        self._star = np.ascontiguousarray(np.broadcast_to(star_flux, (self.nlam,)), dtype=np.float64)
        self.npix = int(npix)
        self.ncell = (len(r) - 1) * (len(t) - 1) * (len(p) - 1)
        cam = _lib.Camera(self.npix, self.npix, float(pixel_cm), float(incl), float(pa), float(phi),
                          int(bool(nostar)), int(max_refine), float(refine_factor))
        dp = C.POINTER(C.c_double)
        self._plan = C.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(self.L.pdgpu_image_plan_create(
                len(r) - 1, len(t) - 1, len(p) - 1, self._keep[0].ctypes.data_as(dp),
                self._keep[1].ctypes.data_as(dp), self._keep[2].ctypes.data_as(dp), C.byref(cam),
                self.nlam, self._star.ctypes.data_as(dp), C.byref(self._plan)),
                "pdgpu_image_plan_create")
            ws, nr = C.c_size_t(), C.c_int64()
            self.levels = np.zeros((self.npix, self.npix), np.int32)
            _lib.check(self.L.pdgpu_image_plan_info(self._plan, C.byref(ws), C.byref(nr),
                                                    self.levels.ctypes.data_as(C.c_void_p)),
                       "pdgpu_image_plan_info")
            self.ws_bytes, self.nrays = ws.value, nr.value
            self.workspace = torch.empty(self.ws_bytes, dtype=torch.uint8, device=self.device)
            _lib.check(self.L.pdgpu_image_plan_upload(
                self._plan, self.workspace.data_ptr(), self.ws_bytes,
                torch.cuda.current_stream(self.device).cuda_stream), "pdgpu_image_plan_upload")

    def __del__(self):
        try:
            if self._plan:
                self.L.pdgpu_image_plan_destroy(self._plan)
                self._plan = C.c_void_p()
        except Exception:
            pass

    def _check_inputs(self, alpha, S):
        for a in (alpha, S):
            assert a.dtype == torch.float32 and a.is_contiguous() and a.device == self.device
            assert a.shape == (self.nlam, self.ncell)

    def run(self, alpha, S, out=None):
        """Pixel-averaged intensity at 1 pc, float64 [nlam, ny, nx]."""
        self._check_inputs(alpha, S)
        if out is None:
            out = torch.empty((self.nlam, self.npix, self.npix), dtype=torch.float64,
                              device=self.device)
        _lib.check(self.L.pdgpu_image_run(self._plan, alpha.data_ptr(), S.data_ptr(),
                                          out.data_ptr(), self.workspace.data_ptr(),
                                          self.ws_bytes,
                                          torch.cuda.current_stream(self.device).cuda_stream),
                   "pdgpu_image_run")
        return out

    def flux(self, image_1pc):
        """Whole-field flux per wavelength at 1 pc (erg/s/cm^2/Hz), float64 [nlam]."""
        img = image_1pc.to(torch.float64).contiguous()
        out = torch.empty(self.nlam, dtype=torch.float64, device=self.device)
        _lib.check(self.L.pdgpu_image_flux(self._plan, img.data_ptr(), out.data_ptr(),
                                           torch.cuda.current_stream(self.device).cuda_stream),
                   "pdgpu_image_flux")
        return out

    def adjoint(self, alpha, S, grad_image):
        """(dL/dalpha, dL/dS) float64 [nlam, ncell] for dL/dimage."""
        self._check_inputs(alpha, S)
        g = grad_image.to(torch.float64).contiguous()
        ga = torch.empty((self.nlam, self.ncell), dtype=torch.float64, device=self.device)
        gs = torch.empty_like(ga)
        _lib.check(self.L.pdgpu_image_adjoint(self._plan, alpha.data_ptr(), S.data_ptr(),
                                              g.data_ptr(), ga.data_ptr(), gs.data_ptr(),
                                              self.workspace.data_ptr(), self.ws_bytes,
                                              torch.cuda.current_stream(self.device).cuda_stream),
                   "pdgpu_image_adjoint")
        return ga, gs


class RayTrace(torch.autograd.Function):
    """image = RayTrace.apply(alpha, S, plan): ray-traced intensity [nlam, ny, nx] whose
    backward is the adjoint ray trace; alpha and S may carry gradients."""

    @staticmethod
    def forward(ctx, alpha, S, plan):
        a = alpha.detach().to(torch.float32).contiguous()
        s = S.detach().to(torch.float32).contiguous()
        ctx.save_for_backward(a, s)
        ctx.plan = plan
        ctx.dtypes = (alpha.dtype, S.dtype)
        return plan.run(a, s)

    @staticmethod
    def backward(ctx, grad):
        a, s = ctx.saved_tensors
        ga, gs = ctx.plan.adjoint(a, s, grad)
        return ga.to(ctx.dtypes[0]), gs.to(ctx.dtypes[1]), None


def model_state(model, device):
    """(rho, T) float64 [nspec, ncell] on the device."""
    g = model.grid
    if len(g.temperature) != len(g.density):
        raise ValueError("run_image needs grid.temperature (run run_thermal first)")
    rho = torch.as_tensor(np.stack([np.asarray(d, dtype=np.float64).reshape(-1)
                                    for d in g.density]), device=device)
    T = torch.as_tensor(np.stack([np.asarray(t, dtype=np.float64).reshape(-1)
                                  for t in g.temperature]), device=device)
    return rho, T


def model_sources(model, lam_um, device, nphot_scat=0, scattering=True,
                  maxtauabs=30.0, seed=0):
    """(alpha, S) float32 on the device for the model's densities and temperatures.  With
    nphot_scat > 0 and scattering dust the scattering source is computed by the GPU
    scattering Monte Carlo; scattering=False drops scattering altogether."""
    from .scatter import ScatterPlan
    g = model.grid
    rho, T = model_state(model, device)
    ka, ks = opacities(g, lam_um)
    if not scattering:
        ks = np.zeros_like(ks)
    kat = torch.as_tensor(ka, device=device)
    J = None
    if nphot_scat > 0 and np.any(ks > 0):
        plan = ScatterPlan(g, lam_um, ka, ks, int(nphot_scat), maxtauabs=maxtauabs, seed=seed,
                           device=device)
        J = plan.run(rho, thermal_emissivity(rho, T, kat, lam_um))
    alpha, S = source_terms(rho, T, kat, torch.as_tensor(ks, device=device), lam_um, J=J)
    return alpha.to(torch.float32).contiguous(), S.to(torch.float32).contiguous()


def _scat_keywords(keywords):
    from .scatter import maxtauabs_of, scattering_enabled
    return dict(scattering=scattering_enabled(keywords), maxtauabs=maxtauabs_of(keywords),
                seed=int(keywords.get("iseed", 0) or 0))


def run_image(model, name=None, nphot=1e6, npix=256, pixelsize=1.0, lam="1300",
              loadlambda=False, incl=0, pa=0, phi=0, dpc=1, nostar=False, max_refine=6,
              refine_factor=0.5, **keywords):
    """``Model.run_image`` for code="gb300"; fills ``model.images[name]``."""
    lam_um = camera_wavelengths(model, lam, loadlambda)
    dev = torch.device("cuda", torch.cuda.current_device())
    pixel_cm = float(pixelsize) * float(dpc) * AU
    plan = ImagePlan(model.grid, npix, pixel_cm, lam_um, incl=incl, pa=pa, phi=phi,
                     nostar=nostar, max_refine=max_refine, refine_factor=refine_factor,
                     device=dev)
    alpha, S = model_sources(model, lam_um, dev, nphot_scat=int(nphot), **_scat_keywords(keywords))
    inten = plan.run(alpha, S).cpu().numpy()              # [nlam, ny, nx] at 1 pc
    omega = (pixel_cm / (dpc * pc)) ** 2
    image = np.ascontiguousarray(np.transpose(inten, (1, 2, 0))[:, :, :, None]) / Jy * omega
    x = (np.arange(npix) - npix // 2) * float(pixelsize)
    model.images[name] = Image(image, x=x.astype(np.float64), y=x.astype(np.float64).copy(),
                               wave=lam_um * 1.0e-4)
    return model.images[name]


def run_visibilities(model, name=None, nphot=1e6, npix=256, pixelsize=1.0, lam="1300",
                     loadlambda=False, incl=0, pa=0, phi=0, dpc=1, nostar=False, **keywords):
    """``Model.run_visibilities`` for code="gb300" (Model.py:682-721): the image of
    run_image (Jy/pixel at ``dpc``, arcsec offsets) transformed by imtovis on the GPU;
    fills ``model.visibilities[name]`` and leaves ``model.images`` untouched, as the
    reference does."""
    from .vis import imtovis
    saved = model.images.get("__run_visibilities__")
    im = run_image(model, name="__run_visibilities__", nphot=nphot, npix=npix,
                   pixelsize=pixelsize, lam=lam, loadlambda=loadlambda, incl=incl, pa=pa,
                   phi=phi, dpc=dpc, nostar=nostar, **keywords)
    if saved is None:
        del model.images["__run_visibilities__"]
    else:
        model.images["__run_visibilities__"] = saved
    model.visibilities[name] = imtovis(im)
    return model.visibilities[name]


def run_sed(model, name=None, nphot=1e6, incl=0, pa=0, phi=0, dpc=1, loadlambda=False,
            npix=129, max_refine=6, refine_factor=0.5, nest_block=17, **keywords):
    """``Model.run_sed`` for code="gb300": flux in Jy at ``dpc`` of the whole grid (plus the
    stars) at every wavelength; fills ``model.spectra[name]``.

    The field is covered by nested square cameras of ``npix`` (odd) pixels: level 0 spans
    the grid; each next level spans the central ``nest_block`` pixels of the one before
    (about 7.6 times finer for 129 / 17) and replaces them, down to a pixel smaller than
    half the inner radius, so the inner rim, which carries the short-wavelength flux, is
    resolved however large the grid is (RADMC-3D's spectrum mode uses circular images for
    the same reason).  Each level refines pixels near small cells as run_image does.  The
    flux is the sum over levels of the pixels outside the next level's block, times the
    pixel solid angle."""
    g = model.grid
    lam_um = camera_wavelengths(model, None, True) if loadlambda else np.asarray(g.lam, np.float64)
    dev = torch.device("cuda", torch.cuda.current_device())
    npix = int(npix) | 1
    nest_block = min(int(nest_block) | 1, npix)
    r, _, _ = grid_arrays(g)
    pixel_cm = 2.02 * r[-1] / npix
    alpha, S = model_sources(model, lam_um, dev, nphot_scat=int(nphot), **_scat_keywords(keywords))
    flux_1pc = torch.zeros(len(lam_um), dtype=torch.float64, device=dev)
    c, h = npix // 2, nest_block // 2
    while True:
        plan = ImagePlan(g, npix, pixel_cm, lam_um, incl=incl, pa=pa, phi=phi, nostar=False,
                         max_refine=max_refine, refine_factor=refine_factor, device=dev)
        inten = plan.run(alpha, S)                              # [nlam, ny, nx] at 1 pc
        finest = pixel_cm <= 0.5 * r[0] or nest_block >= npix
        if not finest:
            inten = inten.clone()
            inten[:, c - h:c + h + 1, c - h:c + h + 1] = 0.0    # covered by the next level
        flux_1pc += inten.sum(dim=(1, 2)) * (pixel_cm / pc) ** 2  # erg/s/cm^2/Hz at 1 pc
        if finest:
            break
        pixel_cm = pixel_cm * nest_block / npix
    flux = flux_1pc.cpu().numpy() / Jy * (1.0 / dpc) ** 2
    model.spectra[name] = Spectrum(wave=lam_um, flux=flux)
    return model.spectra[name]
