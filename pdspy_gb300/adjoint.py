"""Gradients of an interferometric chi^2 through the ray-traced image.

The chain, all in torch autograd with two hand-written GPU adjoints:

    (Mdisk, h0, beta, gamma) --disk_density_torch--> rho_disk (float64)
    rho = [rho_disk, rho_envelope], T frozen --source_terms--> alpha, S
    --RayTrace (adjoint ray trace)--> intensity --x Omega / Jy--> image (Jy/pixel)
    --VisDFT (adjoint DFT)--> Re V, Im V --chisq--> chi^2

``disk_density_torch`` restates pdspy's power-law disk (pdspy/modeling/Disk.py:48-135) in
float64 torch so that d rho/d(parameters) comes from autograd; with Monte Carlo
temperatures held frozen, the gradient w.r.t. every cell density and the four disk
parameters is one backward pass.
"""
import math

import numpy as np
import torch

from .constants import AU, Jy, M_sun, arcsec, pc, pi_pdspy
from .image import ImagePlan, RayTrace, opacities, source_terms, star_flux_1pc
from .thermal import grid_arrays
from .vis import VisDFT, chisq, pixel_grid


def disk_density_torch(r_au, theta, phi, mass, rmin, rmax, h0, beta, gamma):
    """pdspy Disk.density with plrho = gamma + beta and plh = beta, differentiable in
    mass (Msun), h0, beta and gamma.  Returns float64 [nr, ntheta, nphi]."""
    dev = mass.device
    r = torch.as_tensor(np.asarray(r_au, np.float64), device=dev)
    th = torch.as_tensor(np.asarray(theta, np.float64), device=dev)
    ph = torch.as_tensor(np.asarray(phi, np.float64), device=dev)
    rt, tt, _ = torch.meshgrid(r * AU, th, ph, indexing="ij")
    rr = rt * torch.sin(tt)
    zz = rt * torch.cos(tt)

    def surface(rau, normalize):
        rin, rout = rmin * AU, rmax * AU
        m = mass * M_sun
        Sigma0 = (2 - gamma) * m / (2 * pi_pdspy * (1 * AU) ** gamma) / \
            (rout ** (-gamma + 2) - rin ** (-gamma + 2))
        Sig = Sigma0 * rau ** (-gamma)
        inside = ~((rau >= rout / AU) ^ (rau <= rin / AU))
        Sig = torch.where(inside, Sig, torch.zeros_like(Sig))
        if normalize:
            rh = torch.logspace(math.log10(rmin), math.log10(rmax), 1000, dtype=torch.float64,
                                device=dev)
            Sh = surface(rh, False)
            scale = m / (2 * math.pi * torch.trapezoid(rh * AU * Sh, rh * AU))
            Sig = Sig * scale
        return Sig

    Sigma = surface(rr / AU, True)
    h = h0 * AU * (rr / AU) ** beta
    return Sigma / (math.sqrt(2 * math.pi) * h) * torch.exp(-0.5 * (zz / h) ** 2)


class Chi2Problem:
    """chi^2 of a model image against visibility data, with gradients.

    ``rho_fixed`` holds the densities of the species that are not recomputed from disk
    parameters (e.g. an envelope); ``disk`` (dict rmin, rmax) describes species 0 when
    ``chi2_params`` is used."""

    def __init__(self, model, uv, npix, pixelsize, dpc, incl=0.0, pa=0.0, phi=0.0,
                 lam_um=1300.0, max_refine=3, refine_factor=0.5, device=None):
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None
                                   else torch.device(device).index or 0)
        g = model.grid
        self.grid = g
        self.lam_um = np.atleast_1d(np.asarray(lam_um, dtype=np.float64))
        self.npix = npix
        self.pixel_cm = float(pixelsize) * float(dpc) * AU
        self.omega = (self.pixel_cm / (dpc * pc)) ** 2
        self.plan = ImagePlan(g, npix, self.pixel_cm, self.lam_um, incl=incl, pa=pa, phi=phi,
                              max_refine=max_refine, refine_factor=refine_factor,
                              device=self.device)
        ka, ks = opacities(g, self.lam_um)
        self.kabs = torch.as_tensor(ka, device=self.device)
        self.ksca = torch.as_tensor(ks, device=self.device)
        self.T = torch.as_tensor(np.stack([np.asarray(t, np.float64).reshape(-1)
                                           for t in g.temperature]), device=self.device)
        self.rho0 = torch.as_tensor(np.stack([np.asarray(d, np.float64).reshape(-1)
                                              for d in g.density]), device=self.device)
        self.geometry = pixel_grid(npix, pixelsize)
        self.u = torch.as_tensor(uv.u, dtype=torch.float32, device=self.device)
        self.v = torch.as_tensor(uv.v, dtype=torch.float32, device=self.device)
        self.re_d = torch.as_tensor(uv.real, device=self.device)
        self.im_d = torch.as_tensor(uv.imag, device=self.device)
        self.w = torch.as_tensor(uv.weights, device=self.device)
        self.shape = np.asarray(g.density[0]).shape

    def image(self, rho):
        """Image in Jy/pixel [nlam, ny, nx] for densities rho [nspec, ncell] (float64)."""
        alpha, S = source_terms(rho, self.T, self.kabs, self.ksca, self.lam_um)
        return RayTrace.apply(alpha, S, self.plan) * (self.omega / Jy)

    def visibilities(self, rho):
        img = self.image(rho)
        return VisDFT.apply(img[0], self.u, self.v, self.geometry)

    def chi2(self, rho):
        re, im = self.visibilities(rho)
        return chisq(re, im, self.re_d, self.im_d, self.w)

    def rho_from_params(self, params, rmin, rmax):
        """Species 0 from (Mdisk, h0, beta, gamma); other species from the model."""
        r, th, ph = grid_arrays(self.grid)
        rc = 0.5 * (r[1:] + r[:-1]) / AU
        # pdspy evaluates densities at the arithmetic cell centres (Grid.py:71-80)
        rho_d = disk_density_torch(rc, 0.5 * (th[1:] + th[:-1]), 0.5 * (ph[1:] + ph[:-1]),
                                   params[0], rmin, rmax, params[1], params[2], params[3])
        return torch.cat([rho_d.reshape(1, -1), self.rho0[1:]], dim=0)

    def chi2_params(self, params, rmin, rmax):
        return self.chi2(self.rho_from_params(params, rmin, rmax))
