"""The ray-tracing oracle against analytic answers (no GPU)."""
import numpy as np
import torch

from oracle import orc
from pdspy_gb300 import adjoint, constants as K, image, workloads
from tests import _cases, _imageref


def test_uniform_sphere_with_hole():
    """Pixel-centre rays through a uniform shell: I = S (1 - exp(-alpha * chord))."""
    r = np.linspace(1.0, 10.0, 11) * K.AU
    t = np.linspace(0, np.pi, 9)
    p = np.array([0, 2 * np.pi])
    nc = 10 * 8
    a0, S0 = 2e-14, 3.0
    alpha = np.full((1, nc), a0, np.float32)
    S = np.full((1, nc), S0, np.float32)
    npix = 21
    d = 2.2 * r[-1] / npix
    img = orc.image(r, t, p, alpha, S, [0.0], npix, d, incl=37.0, nostar=True, max_refine=0)[0]
    X = (np.arange(npix) - npix // 2) * d
    b = np.hypot(*np.meshgrid(X, X))
    chord = 2 * np.sqrt(np.clip(r[-1] ** 2 - b ** 2, 0, None)) - \
        2 * np.sqrt(np.clip(r[0] ** 2 - b ** 2, 0, None))
    expect = S0 * (1 - np.exp(-float(np.float32(a0)) * chord))
    assert np.allclose(img, expect, rtol=2e-6, atol=1e-12)


def test_source_terms_match_pdspy_conventions():
    """alpha, S from the density-weighted mean temperature (pdspy Model.py:759-769) and
    B_nu (pdspy/misc/B_nu.py:4-6), restated in numpy."""
    m = _cases.image_model("envelope", nr=8, ntheta=8)
    lam = np.array([1300.0, 100.0])
    g = m.grid
    rho = np.stack([d.reshape(-1) for d in g.density])
    T = np.stack([t.reshape(-1) for t in g.temperature])
    rr = np.where(rho == 0, 1e-30, rho)
    Tm = (rr * T).sum(0) / rr.sum(0)
    ka, ks = image.opacities(g, lam)
    nu = K.c / (lam * 1e-4)
    B = (2 * K.h * nu[:, None] ** 3 / K.c ** 2) / (np.exp(K.h * nu[:, None] / (K.k * Tm[None])) - 1)
    alpha = (ka + ks).T @ rho
    S = B * (ka.T @ rho) / np.where(alpha > 0, alpha, 1)
    ta, ts = image.source_terms(torch.as_tensor(rho), torch.as_tensor(T), torch.as_tensor(ka),
                                torch.as_tensor(ks), lam)
    assert np.allclose(ta.numpy(), alpha, rtol=1e-12)
    assert np.allclose(ts.numpy(), S, rtol=1e-10)


def test_dense_dft_reference_against_numpy():
    rng = np.random.default_rng(0)
    img = rng.random((6, 5))
    u, v = rng.normal(size=7) * 1e5, rng.normal(size=7) * 1e5
    x0, dx = -2e-6, 1e-6
    re, im = _imageref.dft(torch.as_tensor(img), torch.as_tensor(u), torch.as_tensor(v),
                           x0, dx, x0, dx)
    X = x0 + np.arange(5) * dx
    Y = x0 + np.arange(6) * dx
    V = np.array([(img * np.exp(-2j * np.pi * (uk * X[None, :] + vk * Y[:, None]))).sum()
                  for uk, vk in zip(u, v)])
    assert np.allclose(re.numpy(), V.real) and np.allclose(im.numpy(), V.imag)


def test_disk_density_torch_matches_numpy_builder():
    m = workloads.small_disk(nr=20, ntheta=16, mass=3e-4, plrho=2.3, h0=0.07, plh=1.2)
    t = adjoint.disk_density_torch(m.grid.r, m.grid.theta, m.grid.phi,
                                   torch.tensor(3e-4, dtype=torch.float64), 0.1, 100.0,
                                   torch.tensor(0.07, dtype=torch.float64),
                                   torch.tensor(1.2, dtype=torch.float64),
                                   torch.tensor(1.1, dtype=torch.float64))
    assert np.allclose(t.numpy(), m.grid.density[0], rtol=1e-12, atol=0)
