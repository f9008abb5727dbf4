"""Model visibilities by direct Fourier transform and the interferometric chi^2.

``VisDFT`` samples an image (Jy per pixel) at (u, v) points on the GPU
(``pdgpu_vis_dft``) with a hand-written adjoint (``pdgpu_vis_dft_adjoint``) as its
backward.  ``chisq`` is pdspy's chi^2 (pdspy/interferometry/libinterferometry.pyx:610-633):
sum w [(Re_d - Re_m)^2 + (Im_d - Im_m)^2].  Pixel (i, j) of an image sits at
x = (i - nx/2) dx, y = (j - ny/2) dy radians, the offsets pdspy's Image carries in arcsec
(pdspy/modeling/Model.py:569-570).
"""
import numpy as np
import torch

from . import _lib
from .constants import arcsec


class UVData:
    """Visibility data: u, v in wavelengths; real, imag in Jy; weights 1/sigma^2."""

    def __init__(self, u, v, real, imag, weights):
        self.u = np.asarray(u, dtype=np.float64)
        self.v = np.asarray(v, dtype=np.float64)
        self.real = np.asarray(real, dtype=np.float64)
        self.imag = np.asarray(imag, dtype=np.float64)
        self.weights = np.asarray(weights, dtype=np.float64)


def synthetic_uv(n=20000, seed=0, bmin_klam=10.0, bmax_klam=2000.0):
    """(u, v) in wavelengths: baseline length uniform in [bmin, bmax] klambda, position
    angle uniform in [0, pi)."""
    rng = np.random.default_rng(seed)
    b = rng.uniform(bmin_klam, bmax_klam, n) * 1e3
    pa = rng.uniform(0.0, np.pi, n)
    return b * np.sin(pa), b * np.cos(pa)


def pixel_grid(npix, pixelsize_arcsec):
    d = float(pixelsize_arcsec) * arcsec
    x0 = -(npix // 2) * d
    return x0, d, x0, d


class VisDFT(torch.autograd.Function):
    """(re, im) = VisDFT.apply(image, u, v, geometry): image [ny, nx] (Jy/pixel),
    u, v float32 device tensors, geometry = (x0, dx, y0, dy) in radians."""

    @staticmethod
    def forward(ctx, image, u, v, geometry):
        L = _lib.lib()
        img = image.detach().to(torch.float32).contiguous()
        ny, nx = img.shape
        n = u.numel()
        re = torch.empty(n, dtype=torch.float64, device=img.device)
        im = torch.empty_like(re)
        st = torch.cuda.current_stream(img.device).cuda_stream
        x0, dx, y0, dy = geometry
        _lib.check(L.pdgpu_vis_dft(nx, ny, x0, dx, y0, dy, img.data_ptr(), n, u.data_ptr(),
                                   v.data_ptr(), re.data_ptr(), im.data_ptr(), st),
                   "pdgpu_vis_dft")
        ctx.save_for_backward(u, v)
        ctx.meta = (nx, ny, geometry, image.dtype)
        return re, im

    @staticmethod
    def backward(ctx, gre, gim):
        L = _lib.lib()
        u, v = ctx.saved_tensors
        nx, ny, (x0, dx, y0, dy), dtype = ctx.meta
        gre = (torch.zeros_like(u, dtype=torch.float64) if gre is None else gre).to(torch.float64).contiguous()
        gim = (torch.zeros_like(u, dtype=torch.float64) if gim is None else gim).to(torch.float64).contiguous()
        gimg = torch.empty((ny, nx), dtype=torch.float64, device=u.device)
        st = torch.cuda.current_stream(u.device).cuda_stream
        _lib.check(L.pdgpu_vis_dft_adjoint(nx, ny, x0, dx, y0, dy, u.numel(), u.data_ptr(),
                                           v.data_ptr(), gre.data_ptr(), gim.data_ptr(),
                                           gimg.data_ptr(), st), "pdgpu_vis_dft_adjoint")
        return gimg.to(dtype), None, None, None


def chisq(re, im, data_re, data_im, weights):
    """pdspy's chi^2 (libinterferometry.pyx:610-633), accumulated in float64."""
    return (((data_re - re) ** 2 + (data_im - im) ** 2) * weights).sum()
