"""Model visibilities by direct Fourier transform or gridded FFT sampling, and the
interferometric chi^2.

``VisDFT`` samples an image (Jy per pixel) at (u, v) points on the GPU
(``pdgpu_vis_dft``) with a hand-written adjoint (``pdgpu_vis_dft_adjoint``) as its
backward: exact at every point, O(pixels x points).  ``VisFFT`` is the method of
galario's sampleImage, which pdspy's interpolate_model calls
(pdspy/interferometry/interpolate_model.py:11-57): a 2-D FFT of the zero-padded image
(cuFFT through torch.fft) and bilinear interpolation at each point
(``pdgpu_vis_grid_sample``, adjoint ``pdgpu_vis_grid_sample_adjoint``): O(pixels log
pixels + points), accurate to the interpolation error, which padding reduces.
``interpolate_model`` mirrors pdspy's function of that name.  ``chisq`` is pdspy's chi^2
(pdspy/interferometry/libinterferometry.pyx:610-633): sum w [(Re_d - Re_m)^2 +
(Im_d - Im_m)^2].  Pixel (i, j) of an image sits at
x = (i - nx/2) dx, y = (j - ny/2) dy radians, the offsets pdspy's Image carries in arcsec
(pdspy/modeling/Model.py:569-570).
"""
import numpy as np
import torch

from . import _lib
from .constants import arcsec


class UVData:
    """Visibility data: u, v in wavelengths; real, imag in Jy; weights 1/sigma^2; freq in
    Hz (optional)."""

    def __init__(self, u, v, real, imag, weights, freq=None):
        self.u = np.asarray(u, dtype=np.float64)
        self.v = np.asarray(v, dtype=np.float64)
        self.real = np.asarray(real, dtype=np.float64)
        self.imag = np.asarray(imag, dtype=np.float64)
        self.weights = np.asarray(weights, dtype=np.float64)
        self.freq = None if freq is None else np.atleast_1d(np.asarray(freq, dtype=np.float64))


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


def _grid_frame(n, pad, geometry):
    x0, dx, y0, dy = geometry
    N = int(pad) * n
    return N, 1.0 / (N * dx), 1.0 / (N * dy), x0 + (n // 2) * dx, y0 + (n // 2) * dy


def grid_transform(image, pad=1):
    """2-D FFT (complex64 [N, N], N = pad n) of an n x n image zero-padded about its centre
    pixel (n/2, n/2)."""
    n = image.shape[-1]
    if image.shape[-2] != n or n % 2:
        raise ValueError("gridded sampling needs a square image with an even side")
    N = int(pad) * n
    F = torch.zeros((N, N), dtype=torch.complex64, device=image.device)
    o = (N - n) // 2
    F[o:o + n, o:o + n] = image.to(torch.float32)
    return torch.fft.fft2(F)


def _check_band(u, v, N, du, dv):
    lim = 0.5 * N - 1.0
    if float(u.abs().max()) / du >= lim or float(v.abs().max()) / dv >= lim:
        raise ValueError("uv points beyond the sampled band (|u| < (n pad / 2 - 1) du): "
                         "use smaller pixels")


class VisFFT(torch.autograd.Function):
    """(re, im) = VisFFT.apply(image, u, v, geometry, pad): gridded sampling of a square
    image [n, n] (Jy/pixel), geometry = (x0, dx, y0, dy) in radians as for VisDFT."""

    @staticmethod
    def forward(ctx, image, u, v, geometry, pad=1):
        L = _lib.lib()
        n = image.shape[-1]
        N, du, dv, xc, yc = _grid_frame(n, pad, geometry)
        _check_band(u, v, N, du, dv)
        G = grid_transform(image.detach(), pad).contiguous()
        nuv = u.numel()
        re = torch.empty(nuv, dtype=torch.float64, device=image.device)
        im = torch.empty_like(re)
        st = torch.cuda.current_stream(image.device).cuda_stream
        _lib.check(L.pdgpu_vis_grid_sample(N, G.data_ptr(), du, dv, xc, yc, nuv, u.data_ptr(),
                                           v.data_ptr(), re.data_ptr(), im.data_ptr(), st),
                   "pdgpu_vis_grid_sample")
        ctx.save_for_backward(u, v)
        ctx.meta = (n, N, du, dv, xc, yc, image.dtype)
        return re, im

    @staticmethod
    def backward(ctx, gre, gim):
        L = _lib.lib()
        u, v = ctx.saved_tensors
        n, N, du, dv, xc, yc, dtype = ctx.meta
        gre = (torch.zeros_like(u, dtype=torch.float64) if gre is None else gre).to(torch.float64).contiguous()
        gim = (torch.zeros_like(u, dtype=torch.float64) if gim is None else gim).to(torch.float64).contiguous()
        H = torch.zeros((N, N), dtype=torch.complex128, device=u.device)
        st = torch.cuda.current_stream(u.device).cuda_stream
        _lib.check(L.pdgpu_vis_grid_sample_adjoint(N, du, dv, xc, yc, u.numel(), u.data_ptr(),
                                                   v.data_ptr(), gre.data_ptr(), gim.data_ptr(),
                                                   H.data_ptr(), st),
                   "pdgpu_vis_grid_sample_adjoint")
        o = (N - n) // 2
        g = torch.fft.fft2(H).real[o:o + n, o:o + n]
        return g.to(dtype), None, None, None, None


class Visibilities:
    """Mirror of pdspy's interferometry.Visibilities fields that interpolate_model fills
    (pdspy/interferometry/libinterferometry.pyx): u, v (wavelengths), freq (Hz),
    real/imag [nuv, nfreq] (Jy), weights."""

    def __init__(self, u, v, freq, real, imag, weights):
        self.u, self.v, self.freq = u, v, freq
        self.real, self.imag, self.weights = real, imag, weights


def imtovis(image, device=None):
    """``imtovis`` (pdspy/imaging/imtovis.py:6-27) on the GPU: the visibilities on the
    image's own Fourier grid, per frequency fftshift(fft2(ifftshift(plane))) in complex128
    (cuFFT through torch.fft, a plain library transform), u and v from
    fftshift(fftfreq(n, pixel [rad])), flattened row by row as pdspy's meshgrid/reshape does
    (u runs along x, v along y), unit weights.  ``image`` is an Image with
    ``image[ny, nx, nfreq, 1]`` in Jy/pixel and ``x``/``y`` in arcsec."""
    dev = torch.device("cuda", torch.cuda.current_device()) if device is None else device
    img = torch.as_tensor(np.asarray(image.image[:, :, :, 0], dtype=np.float64), device=dev)
    ny, nx, nf = img.shape
    planes = img.permute(2, 0, 1)                                  # [nfreq, ny, nx]
    V = torch.fft.fftshift(torch.fft.fft2(torch.fft.ifftshift(planes, dim=(-2, -1))),
                           dim=(-2, -1))
    real = V.real.reshape(nf, ny * nx).T.contiguous().cpu().numpy()
    imag = V.imag.reshape(nf, ny * nx).T.contiguous().cpu().numpy()
    x = np.asarray(image.x, dtype=np.float64)
    y = np.asarray(image.y, dtype=np.float64)
    uu = np.fft.fftshift(np.fft.fftfreq(x.size, (x[1] - x[0]) * arcsec))
    vv = np.fft.fftshift(np.fft.fftfreq(y.size, (y[1] - y[0]) * arcsec))
    u, v = np.meshgrid(uu, vv)
    return Visibilities(u.reshape(-1), v.reshape(-1), np.atleast_1d(image.freq), real, imag,
                        np.ones(real.shape))


def interpolate_model(u, v, freq, model, dRA=0.0, dDec=0.0, code="fft", pad=1, device=None):
    """``interpolate_model`` (pdspy/interferometry/interpolate_model.py:11-57) on the GPU:
    model visibilities of an Image (``image[ny, nx, nfreq, 1]`` Jy/pixel, ``x``/``y`` in
    arcsec) at (u, v) wavelengths, the image shifted by (dRA, dDec) arcsec.  code="fft"
    samples the gridded FFT (galario's method, ``pad``-times zero padding), code="dft" sums
    directly.  The sign convention is pdgpu_vis_dft's, V = sum F exp(-2 pi i (u x + v y))
    (galario itself is not available to pin its conventions against)."""
    dev = torch.device("cuda", torch.cuda.current_device()) if device is None else device
    img = np.asarray(model.image, dtype=np.float64)
    ny, nx, nf = img.shape[0], img.shape[1], img.shape[2]
    dx = (float(model.x[1]) - float(model.x[0])) * arcsec
    dy = (float(model.y[1]) - float(model.y[0])) * arcsec
    geo = (float(model.x[0]) * arcsec + dRA * arcsec, dx, float(model.y[0]) * arcsec + dDec * arcsec, dy)
    ut = torch.as_tensor(np.asarray(u, dtype=np.float32).ravel(), device=dev)
    vt = torch.as_tensor(np.asarray(v, dtype=np.float32).ravel(), device=dev)
    real = np.empty((ut.numel(), nf))
    imag = np.empty((ut.numel(), nf))
    for i in range(nf):
        plane = torch.as_tensor(img[:, :, i, 0], dtype=torch.float32, device=dev)
        if code == "fft":
            re, im = VisFFT.apply(plane, ut, vt, geo, pad)
        elif code == "dft":
            re, im = VisDFT.apply(plane, ut, vt, geo)
        else:
            raise ValueError("code must be 'fft' or 'dft'")
        real[:, i] = re.cpu().numpy()
        imag[:, i] = im.cpu().numpy()
    return Visibilities(np.asarray(u), np.asarray(v), np.atleast_1d(freq), real, imag,
                        np.ones(real.shape))
