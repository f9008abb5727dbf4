"""GPU ray tracer against the CPU oracle and analytic answers (run_image, run_sed)."""
import numpy as np
import pytest
import torch

from oracle import orc
from pdspy_gb300 import constants as K, image, thermal
from tests import _cases

pytestmark = pytest.mark.gpu

# image tolerance: FP32 per-segment transfer against the float64 oracle on the same
# float32 (alpha, S) inputs and identical FP64 ray geometry
RTOL = 2e-5

CASES = [
    ("disk", dict(incl=0.0, pa=0.0, phi=0.0), [1300.0]),
    ("disk", dict(incl=60.0, pa=30.0, phi=20.0), [1300.0, 100.0, 10.0]),
    ("mirror", dict(incl=75.0, pa=0.0, phi=0.0), [870.0]),
    ("spiral", dict(incl=45.0, pa=-20.0, phi=10.0), [1300.0, 30.0]),
    ("envelope", dict(incl=30.0, pa=45.0, phi=0.0), [1300.0]),
]


def _gpu_and_oracle(kind, cam, lam, npix=24, nostar=False, max_refine=3):
    m = _cases.image_model(kind, nr=12, ntheta=12, nphi=8 if kind == "spiral" else 1)
    dev = torch.device("cuda", 0)
    r, t, p = thermal.grid_arrays(m.grid)
    pixel_cm = 2.1 * r[-1] / npix
    lam = np.asarray(lam)
    plan = image.ImagePlan(m.grid, npix, pixel_cm, lam, nostar=nostar, max_refine=max_refine,
                           **cam)
    alpha, S = image.model_sources(m, lam, dev)
    gpu = plan.run(alpha, S).cpu().numpy()
    sf = image.star_flux_1pc(m.grid, lam)
    ref = orc.image(r, t, p, alpha.cpu().numpy(), S.cpu().numpy(), sf, npix, pixel_cm,
                    nostar=nostar, max_refine=max_refine, refine_factor=0.5,
                    incl=cam["incl"], pa=cam["pa"], phi=cam["phi"])
    levels = orc.refine_levels(r, t, p, npix, pixel_cm, max_refine=max_refine)
    return m, plan, gpu, ref, levels


@pytest.mark.parametrize("kind,cam,lam", CASES)
def test_image_matches_oracle(cuda, kind, cam, lam):
    m, plan, gpu, ref, levels = _gpu_and_oracle(kind, cam, lam)
    assert np.array_equal(plan.levels, levels)
    assert np.all(np.isfinite(gpu))
    scale = np.abs(ref).max()
    assert np.allclose(gpu, ref, rtol=RTOL, atol=RTOL * 1e-3 * scale), \
        np.abs(gpu - ref).max() / scale


def test_nostar_and_star_pixel(cuda):
    _, _, a, ref_a, _ = _gpu_and_oracle("disk", dict(incl=20.0, pa=0.0, phi=0.0), [10.0],
                                        nostar=False)
    _, _, b, ref_b, _ = _gpu_and_oracle("disk", dict(incl=20.0, pa=0.0, phi=0.0), [10.0],
                                        nostar=True)
    diff = a - b
    c = a.shape[-1] // 2
    assert diff[0, c, c] > 0
    diff[0, c, c] = 0
    assert np.allclose(diff, 0.0)


def test_run_image_api_units(cuda):
    m = _cases.image_model("disk", nr=12, ntheta=12)
    img = m.run_image(name="1300", npix=16, pixelsize=0.05, lam="1300", incl=30, pa=10,
                      dpc=140, code="gb300")
    assert m.images["1300"] is img
    assert img.image.shape == (16, 16, 1, 1) and img.image.dtype == np.float64
    assert np.allclose(img.x, (np.arange(16) - 8) * 0.05) and np.allclose(img.wave, 0.13)
    # Jy/pixel = intensity at 1 pc x pixel solid angle at dpc / 1e-23
    pixel_cm = 0.05 * 140 * K.AU
    plan = image.ImagePlan(m.grid, 16, pixel_cm, [1300.0], incl=30, pa=10)
    a, s = image.model_sources(m, np.array([1300.0]), torch.device("cuda", 0))
    inten = plan.run(a, s).cpu().numpy()[0]
    expect = inten * (pixel_cm / (140 * K.pc)) ** 2 / K.Jy
    assert np.allclose(img.image[:, :, 0, 0], expect, rtol=1e-12)


def test_sed_optically_thin_matches_volume_emission(cuda):
    """Optically thin dust: F_nu = sum_c j_c V_c / d^2 plus the star (within 2%)."""
    m = _cases.image_model("disk", nr=24, ntheta=24, mass=1e-9)
    lam = np.array([300.0, 1000.0, 3000.0])
    m.set_camera_wavelength(lam)
    sed = m.run_sed(name="SED", loadlambda=True, dpc=140, npix=96, code="gb300")
    g = m.grid
    r, t, p = thermal.grid_arrays(g)
    V = ((r[1:] ** 3 - r[:-1] ** 3) / 3)[:, None, None] * \
        (np.cos(t[:-1]) - np.cos(t[1:]))[None, :, None] * (p[1:] - p[:-1])[None, None, :]
    ka, _ = image.opacities(g, lam)
    nu = K.c / (lam * 1e-4)
    T = g.temperature[0]
    B = (2 * K.h * nu[:, None, None, None] ** 3 / K.c ** 2) / \
        np.expm1(K.h * nu[:, None, None, None] / (K.k * T[None]))
    L = (4 * np.pi * ka[0][:, None, None, None] * g.density[0][None] * B * V[None]).sum((1, 2, 3))
    d = 140 * K.pc
    expect = L / (4 * np.pi * d ** 2) / K.Jy + image.star_flux_1pc(g, lam) / 140 ** 2 / K.Jy
    assert np.allclose(sed.flux, expect, rtol=0.02), sed.flux / expect


def test_image_flux_is_omega_times_pixel_sum(cuda):
    m = _cases.image_model("disk", nr=12, ntheta=12)
    lam = np.array([1300.0, 100.0, 10.0])
    r, _, _ = thermal.grid_arrays(m.grid)
    npix = 40
    pixel_cm = 2.02 * r[-1] / npix
    plan = image.ImagePlan(m.grid, npix, pixel_cm, lam, incl=35.0, device=cuda)
    a, s = image.model_sources(m, lam, cuda)
    img = plan.run(a, s)
    got = plan.flux(img).cpu().numpy()
    expect = img.sum(dim=(1, 2)).cpu().numpy() * (pixel_cm / K.pc) ** 2
    assert np.allclose(got, expect, rtol=1e-12, atol=0)


def test_run_visibilities_is_imtovis_of_the_image(cuda):
    """Model.run_visibilities (Model.py:682-721): the image of run_image transformed like
    pdspy's imtovis (imaging/imtovis.py:6-27): fftshift(fft2(ifftshift(plane))) per
    frequency, u/v from fftshift(fftfreq(n, pixel)), flattened row by row, unit weights.
    Checked against numpy's transform of the same image (complex128 both)."""
    m = _cases.image_model("disk", nr=12, ntheta=12)
    kw = dict(nphot=2000, npix=32, pixelsize=0.05, lam=[1300.0, 870.0], incl=40.0, pa=20.0,
              dpc=140.0)
    im = m.run_image(name="img", **kw)
    vis = m.run_visibilities(name="vis", **kw)
    assert "vis" in m.visibilities and list(m.images) == ["img"]
    n = 32
    for i in range(2):
        ref = np.fft.fftshift(np.fft.fft2(np.fft.ifftshift(im.image[:, :, i, 0])))
        scale = np.abs(ref).max()
        assert np.abs(vis.real[:, i] - ref.real.reshape(-1)).max() <= 1e-12 * scale
        assert np.abs(vis.imag[:, i] - ref.imag.reshape(-1)).max() <= 1e-12 * scale
    uu = np.fft.fftshift(np.fft.fftfreq(n, (im.x[1] - im.x[0]) * K.arcsec))   # as pdspy
    vv = np.fft.fftshift(np.fft.fftfreq(n, (im.y[1] - im.y[0]) * K.arcsec))
    u, v = np.meshgrid(uu, vv)
    assert np.array_equal(vis.u, u.reshape(-1)) and np.array_equal(vis.v, v.reshape(-1))
    assert vis.real.shape == (n * n, 2) and np.all(vis.weights == 1.0)
    assert np.allclose(vis.freq, im.freq)
    # the zero-spacing visibility is the total flux
    k = (n // 2) * n + n // 2
    assert vis.real[k, 0] == pytest.approx(im.image[:, :, 0, 0].sum(), rel=1e-12)


@pytest.mark.parametrize("config", ["config0", "config1"])
def test_sed_converged_at_its_defaults(cuda, config):
    """run_sed at its defaults (nested 129-pixel cameras, max_refine 6) against a much finer
    trace of the same model (257 pixels per level, max_refine 9), 1 um to 1 cm, within 2%
    (the SED accuracy criterion).  Config 0 is also checked against one 1025-pixel camera
    refined to 4^10 sub-rays (no nesting).  The disk + envelope grid reaches 1e4 au while
    its inner rim, which carries the 1-10 um flux, sits at 0.1 au."""
    from pdspy_gb300 import workloads
    m = workloads.small_disk() if config == "config0" else workloads.disk_envelope(nr=256, ntheta=256)
    g = m.grid
    rr = np.meshgrid(g.r, g.theta, g.phi, indexing="ij")[0]
    g.temperature = [np.maximum(1400.0 * (rr / 0.1) ** -0.5, 10.0)] * len(g.density)
    lam = np.logspace(0, 4, 13)
    m.set_camera_wavelength(lam)
    kw = dict(nphot=100000, loadlambda=True, dpc=140, incl=45.0)
    sed = image.run_sed(m, name="SED", **kw).flux
    fine = image.run_sed(m, name="fine", npix=257, max_refine=9, **kw).flux
    assert np.all(sed > 0)
    assert np.allclose(sed, fine, rtol=0.02, atol=0), sed / fine - 1
    if config == "config0":
        single = image.run_sed(m, name="single", npix=1025, max_refine=10, nest_block=1025,
                               **kw).flux
        assert np.allclose(sed, single, rtol=0.02, atol=0), sed / single - 1
