"""Gridded FFT visibility sampling (galario's method behind pdspy's interpolate_model,
pdspy/interferometry/interpolate_model.py:11-57) against the direct sum and against a
float64 torch restatement of the same operation (forward and adjoint)."""
import numpy as np
import pytest
import torch

from pdspy_gb300 import image, vis

pytestmark = pytest.mark.gpu


def relerr(a, b):
    return float(torch.linalg.norm(a - b) / torch.linalg.norm(b))


def _ref(img, u, v, geo, pad):
    """float64 restatement: zero-pad, FFT, (-1)^(k+l), bilinear, centre phase."""
    n = img.shape[-1]
    N, du, dv, xc, yc = vis._grid_frame(n, pad, geo)
    o = (N - n) // 2
    F = torch.zeros((N, N), dtype=torch.complex128)
    F[o:o + n, o:o + n] = img.to(torch.complex128)
    G = torch.fft.fft2(F)
    fu, fv = u / du, v / dv
    k0, l0 = torch.floor(fu), torch.floor(fv)
    t, s = fu - k0, fv - l0
    W = torch.zeros(u.shape, dtype=torch.complex128)
    for a, wl in ((0, 1 - s), (1, s)):
        for c, wk in ((0, 1 - t), (1, t)):
            k = (k0 + c).long()
            l = (l0 + a).long()
            sg = 1.0 - 2.0 * ((k + l) % 2).double()
            W = W + (sg * wk * wl) * G[l % N, k % N]
    V = W * torch.exp(-2j * np.pi * (u * xc + v * yc))
    return V.real, V.imag


def _setup(n, nuv, seed, frac=0.45):
    rng = np.random.default_rng(seed)
    geo = vis.pixel_grid(n, 0.02)
    _, du, dv, _, _ = vis._grid_frame(n, 1, geo)
    u = rng.uniform(-frac, frac, nuv) * n * du
    v = rng.uniform(-frac, frac, nuv) * n * dv
    return geo, torch.as_tensor(u, dtype=torch.float32), torch.as_tensor(v, dtype=torch.float32)


def test_exact_on_grid_points(cuda):
    n = 64
    rng = np.random.default_rng(1)
    img = torch.as_tensor(rng.random((n, n)), dtype=torch.float32, device=cuda)
    geo = vis.pixel_grid(n, 0.02)
    N, du, dv, _, _ = vis._grid_frame(n, 2, geo)
    k = rng.integers(-N // 2 + 2, N // 2 - 2, 500)
    l = rng.integers(-N // 2 + 2, N // 2 - 2, 500)
    u = torch.as_tensor(k * du, dtype=torch.float32, device=cuda)
    v = torch.as_tensor(l * dv, dtype=torch.float32, device=cuda)
    # float32 u, v are within 1e-7 of the grid: the interpolation weight is ~1e-5 at most
    re, im = vis.VisFFT.apply(img, u, v, geo, 2)
    rd, idd = vis.VisDFT.apply(img, u, v, geo)
    assert relerr(re, rd) < 1e-4 and relerr(im, idd) < 1e-4


def test_centred_source_matches_direct_sum(cuda):
    n = 64
    x = np.arange(n) - n // 2
    img = np.exp(-0.5 * (x[None, :] ** 2 + x[:, None] ** 2) / 3.0 ** 2)
    img = torch.as_tensor(img, dtype=torch.float32, device=cuda)
    geo, u, v = _setup(n, 2000, 2, frac=0.1)
    u, v = u.to(cuda), v.to(cuda)
    re, im = vis.VisFFT.apply(img, u, v, geo, 4)
    rd, idd = vis.VisDFT.apply(img, u, v, geo)
    scale = float(torch.sqrt(rd ** 2 + idd ** 2).max())
    assert float((re - rd).abs().max()) / scale < 2e-3
    assert float((im - idd).abs().max()) / scale < 2e-3


@pytest.mark.parametrize("pad", [1, 2])
def test_forward_and_adjoint_vs_float64(cuda, pad):
    n, nuv = 32, 400
    rng = np.random.default_rng(5)
    img = torch.tensor(rng.random((n, n)), dtype=torch.float32, device=cuda, requires_grad=True)
    geo, u, v = _setup(n, nuv, 6)
    re, im = vis.VisFFT.apply(img, u.to(cuda), v.to(cuda), geo, pad)
    gr = torch.as_tensor(rng.normal(size=nuv))
    gi = torch.as_tensor(rng.normal(size=nuv))
    ((re * gr.to(cuda)).sum() + (im * gi.to(cuda)).sum()).backward()
    i64 = img.detach().double().cpu().requires_grad_(True)
    rr, ii = _ref(i64, u.double(), v.double(), geo, pad)
    ((rr * gr).sum() + (ii * gi).sum()).backward()
    assert relerr(re.detach().cpu(), rr.detach()) < 1e-5
    assert relerr(im.detach().cpu(), ii.detach()) < 1e-5
    assert relerr(img.grad.double().cpu(), i64.grad) < 1e-5


def test_out_of_band_raises(cuda):
    n = 16
    img = torch.ones((n, n), device=cuda)
    geo = vis.pixel_grid(n, 0.02)
    _, du, _, _, _ = vis._grid_frame(n, 1, geo)
    u = torch.tensor([0.5 * n * du], dtype=torch.float32, device=cuda)
    with pytest.raises(ValueError):
        vis.VisFFT.apply(img, u, torch.zeros_like(u), geo, 1)


def test_interpolate_model_api(cuda):
    n = 64
    x = (np.arange(n) - n // 2) * 0.02
    rng = np.random.default_rng(7)
    cube = np.zeros((n, n, 2, 1))
    g = np.exp(-0.5 * (x[None, :] ** 2 + x[:, None] ** 2) / 0.06 ** 2)
    cube[:, :, 0, 0] = g
    cube[:, :, 1, 0] = 2 * g
    model = image.Image(cube, x=x, y=x.copy(), wave=np.array([0.13, 0.087]))
    u, v = vis.synthetic_uv(500, seed=8, bmin_klam=10, bmax_klam=500)
    a = vis.interpolate_model(u, v, [2.3e11, 3.4e11], model, dRA=0.05, dDec=-0.03, code="fft",
                              pad=4, device=cuda)
    b = vis.interpolate_model(u, v, [2.3e11, 3.4e11], model, dRA=0.05, dDec=-0.03, code="dft",
                              device=cuda)
    assert a.real.shape == (500, 2) and a.imag.shape == (500, 2)
    scale = np.abs(b.real).max()
    assert np.abs(a.real - b.real).max() / scale < 3e-3
    assert np.abs(a.imag - b.imag).max() / scale < 3e-3
    assert np.allclose(b.real[:, 1], 2 * b.real[:, 0], rtol=1e-5, atol=1e-6 * scale)
    # the shift is a phase: amplitudes do not change
    c = vis.interpolate_model(u, v, [2.3e11, 3.4e11], model, code="dft", device=cuda)
    assert np.allclose(np.hypot(b.real, b.imag), np.hypot(c.real, c.imag), rtol=1e-4,
                       atol=1e-6 * scale)
