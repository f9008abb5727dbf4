"""Monte Carlo scattering source behind ``Model.run_scattering(code="gb300")`` and the
albedo > 0 images and spectra of ``run_image`` / ``run_sed``.

RADMC-3D computes the scattering source by a monochromatic Monte Carlo at every camera
wavelength before it ray-traces an image or a spectrum of dust that scatters, with
``nphot_scat`` (images, pdspy/modeling/Model.py:520 passes run_image's ``nphot``) or
``nphot_spec`` (spectra, Model.py:639) packets and the ``mc_scat_maxtauabs`` cut
(pdspy/radmc3d/write.py:33-38, :141-142); ``radmc3d mcscat`` runs it alone for
``Model.run_scattering`` (Model.py:258-322).  Here ``ScatterPlan`` runs it on the GPU
(``pdgpu_scat_*``): the result is the mean intensity J of every cell at every
wavelength.  Scattering is isotropic -- pdspy writes no asymmetry parameter to RADMC-3D
(Model.py:774-776) -- so the scattering emissivity of a cell is sum_s rho_s ksca_s J and
its scattering source function is J itself.

Photon sources are the stars and the thermal emission of the dust at the density-weighted
mean temperature pdspy writes for image mode (Model.py:759-769).
"""
import ctypes as C

import numpy as np
import torch

from . import _lib
from .constants import c as C_LIGHT
from .thermal import _stars, grid_arrays

MAXTAUABS = 30.0


class ScatterPlan:
    """Scattering Monte Carlo of one grid at the wavelengths ``lam_um`` (microns) with
    opacities ``kabs``/``ksca`` [nspec, nlam] (cm^2/g); ``run`` works on device tensors."""

    def __init__(self, grid, lam_um, kabs, ksca, nphot, maxtauabs=MAXTAUABS, seed=0,
                 max_scatter=0, device=None):
        self.L = _lib.lib()
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None
                                   else torch.device(device).index or 0)
        r, t, p = grid_arrays(grid)
        radius, temp = _stars(grid)
        self.lam_um = np.ascontiguousarray(np.atleast_1d(lam_um), dtype=np.float64)
        self.nlam = len(self.lam_um)
        ka = np.ascontiguousarray(np.atleast_2d(kabs), dtype=np.float64)
        ks = np.ascontiguousarray(np.atleast_2d(ksca), dtype=np.float64)
        if ka.shape != ks.shape or ka.shape[1] != self.nlam:
            raise ValueError("kabs/ksca must be [nspec, nlam]")
        self.nspec = ka.shape[0]
        self._keep = [np.ascontiguousarray(a, dtype=np.float64)
                      for a in (r, t, p, radius, temp)] + [ka, ks]
        dp = C.POINTER(C.c_double)
        k = self._keep
        desc = _lib.ModelDesc(len(r) - 1, len(t) - 1, len(p) - 1, k[0].ctypes.data_as(dp),
                              k[1].ctypes.data_as(dp), k[2].ctypes.data_as(dp), len(radius),
                              k[3].ctypes.data_as(dp), k[4].ctypes.data_as(dp), 0)
        opts = _lib.ScatOptions(int(seed), int(nphot), float(maxtauabs), int(max_scatter), 0, 0)
        self.nphot = int(nphot)
        self._plan = C.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(self.L.pdgpu_scat_plan_create(
                C.byref(desc), self.nlam, self.lam_um.ctypes.data_as(dp), self.nspec,
                ka.ctypes.data_as(dp), ks.ctypes.data_as(dp), C.byref(opts),
                C.byref(self._plan)), "pdgpu_scat_plan_create")
            ws, nc = C.c_size_t(), C.c_int64()
            _lib.check(self.L.pdgpu_scat_plan_info(self._plan, C.byref(ws), C.byref(nc)),
                       "pdgpu_scat_plan_info")
            self.ws_bytes, self.ncell = ws.value, nc.value
            self.workspace = torch.empty(self.ws_bytes, dtype=torch.uint8, device=self.device)
            _lib.check(self.L.pdgpu_scat_plan_upload(
                self._plan, self.workspace.data_ptr(), self.ws_bytes,
                torch.cuda.current_stream(self.device).cuda_stream), "pdgpu_scat_plan_upload")

    def __del__(self):
        try:
            if self._plan:
                self.L.pdgpu_scat_plan_destroy(self._plan)
                self._plan = C.c_void_p()
        except Exception:
            pass

    def run(self, rho, emis=None, out=None):
        """Mean intensity J, float64 [nlam, ncell] (erg/s/cm^2/Hz/ster), for densities
        ``rho`` (float32 [nspec, ncell]) and the thermal emissivity ``emis`` (float64
        [nlam, ncell], erg/s/cm^3/Hz/ster) or None for stellar photons only."""
        rho = rho.to(device=self.device, dtype=torch.float32).contiguous()
        if rho.shape != (self.nspec, self.ncell):
            raise ValueError("rho must be [nspec, ncell] = %s" % ((self.nspec, self.ncell),))
        eptr = None
        if emis is not None:
            emis = emis.to(device=self.device, dtype=torch.float64).contiguous()
            if emis.shape != (self.nlam, self.ncell):
                raise ValueError("emis must be [nlam, ncell]")
            eptr = emis.data_ptr()
        if out is None:
            out = torch.empty((self.nlam, self.ncell), dtype=torch.float64, device=self.device)
        _lib.check(self.L.pdgpu_scat_run(self._plan, rho.data_ptr(), eptr, out.data_ptr(),
                                         self.workspace.data_ptr(), self.ws_bytes,
                                         torch.cuda.current_stream(self.device).cuda_stream),
                   "pdgpu_scat_run")
        self._last = (rho, emis)   # keep the inputs alive until the stream has used them
        return out

    def stats(self):
        s = _lib.ScatStats()
        _lib.check(self.L.pdgpu_scat_plan_stats(self._plan, self.workspace.data_ptr(),
                                                torch.cuda.current_stream(self.device).cuda_stream,
                                                C.byref(s)), "pdgpu_scat_plan_stats")
        return s.asdict()


def maxtauabs_of(keywords):
    v = keywords.get("mc_scat_maxtauabs")
    return MAXTAUABS if v is None else float(v)


def scattering_enabled(keywords):
    """RADMC-3D's scattering_mode_max = 0 (pdspy/radmc3d/write.py:53-54) switches
    scattering off: no scattering source and no scattering extinction."""
    v = keywords.get("scattering_mode_max")
    return v is None or int(v) != 0


def mean_intensity(model, lam_um, nphot, device=None, maxtauabs=MAXTAUABS, seed=0):
    """J [nlam, ncell] on the device for the model's densities and temperatures, with
    packets from the stars and from the dust's thermal emission."""
    from .image import model_state, opacities, thermal_emissivity
    g = model.grid
    dev = torch.device("cuda", torch.cuda.current_device()) if device is None else device
    rho, T = model_state(model, dev)
    ka, ks = opacities(g, lam_um)
    emis = thermal_emissivity(rho, T, torch.as_tensor(ka, device=dev), lam_um)
    plan = ScatterPlan(g, lam_um, ka, ks, nphot, maxtauabs=maxtauabs, seed=seed, device=dev)
    return plan.run(rho, emis)


def run_scattering(model, nphot=1e6, loadlambda=None, **keywords):
    """``Model.run_scattering`` for code="gb300": fills ``grid.scattering_phase_freq`` (Hz)
    and ``grid.scattering_phase`` (float64 [nfreq, nr, ntheta, nphi], the isotropic
    scattering source function J of every cell, erg/s/cm^2/Hz/ster), the layout
    Model.py:312-320 leaves.  Wavelengths: ``model.camera_wavelength`` when loadlambda is
    set, else ``grid.lam``."""
    g = model.grid
    lam_um = np.asarray(model.camera_wavelength if loadlambda else g.lam, dtype=np.float64)
    lam_um = np.atleast_1d(lam_um)
    J = mean_intensity(model, lam_um, int(nphot), maxtauabs=maxtauabs_of(keywords),
                       seed=int(keywords.get("iseed", 0) or 0))
    shape = np.asarray(g.density[0]).shape
    g.scattering_phase_freq = C_LIGHT / (lam_um * 1.0e-4)
    g.scattering_phase = J.cpu().numpy().reshape((len(lam_um),) + tuple(shape))
    return g.scattering_phase
