"""GPU scattering Monte Carlo against the CPU oracle, and its use by run_image / run_sed /
run_scattering (pdspy/modeling/Model.py:258-322, :515-577, :608-650)."""
import numpy as np
import pytest
import torch

from oracle import orc
from pdspy_gb300 import image, scatter, thermal
from tests import _cases

pytestmark = pytest.mark.gpu

LAM = np.array([0.5, 2.0, 10.0])


def _inputs(kind, dev, nphi=1):
    m = _cases.image_model(kind, nr=12, ntheta=12, nphi=nphi)
    rho, T = image.model_state(m, dev)
    ka, ks = image.opacities(m.grid, LAM)
    emis = image.thermal_emissivity(rho, T, torch.as_tensor(ka, device=dev), LAM)
    return m, rho, ka, ks, emis


def _oracle(m, rho, ka, ks, emis, nphot, **kw):
    r, t, p = thermal.grid_arrays(m.grid)
    radius, temp = thermal._stars(m.grid)
    return orc.mcscat(r, t, p, rho.to(torch.float32).cpu().numpy(), LAM, ka, ks, radius, temp,
                      nphot, emis=None if emis is None else emis.cpu().numpy(), **kw)


@pytest.mark.parametrize("kind,nphi,dust,maxtauabs", [
    ("mirror", 1, True, 30.0),
    ("envelope", 1, True, 5.0),
    ("spiral", 8, True, 30.0),
    ("disk", 1, False, 30.0),
])
def test_mean_intensity_bit_exact(cuda, kind, nphi, dust, maxtauabs):
    m, rho, ka, ks, emis = _inputs(kind, cuda, nphi)
    e = emis if dust else None
    plan = scatter.ScatterPlan(m.grid, LAM, ka, ks, 4000, maxtauabs=maxtauabs, seed=11,
                               device=cuda)
    J = plan.run(rho, e).cpu().numpy()
    st = plan.stats()
    ref = _oracle(m, rho, ka, ks, e, 4000, seed=11, maxtauabs=maxtauabs)
    assert np.array_equal(J, ref["J"]), np.abs(J - ref["J"]).max() / np.abs(ref["J"]).max()
    for k in ("packets", "escaped", "dropped", "capped", "scatterings", "crossings"):
        assert st[k] == ref["stats"][k], k
    assert st["scatterings"] > 0 and np.all(J >= 0) and J.max() > 0


def test_replay_is_deterministic_and_seeded(cuda):
    m, rho, ka, ks, emis = _inputs("mirror", cuda)
    plan = scatter.ScatterPlan(m.grid, LAM, ka, ks, 20000, seed=3, device=cuda)
    a = plan.run(rho, emis).clone()
    b = plan.run(rho, emis)
    assert torch.equal(a, b)
    other = scatter.ScatterPlan(m.grid, LAM, ka, ks, 20000, seed=4, device=cuda).run(rho, emis)
    assert not torch.equal(a, other)


def test_scattered_light_brightens_short_wavelength_image(cuda):
    m = _cases.image_model("mirror", nr=16, ntheta=16)
    lam = np.array([1.0])
    r, _, _ = thermal.grid_arrays(m.grid)
    npix = 32
    pixel_cm = 2.1 * r[-1] / npix
    plan = image.ImagePlan(m.grid, npix, pixel_cm, lam, incl=60.0, nostar=True, device=cuda)
    a0, s0 = image.model_sources(m, lam, cuda)
    a1, s1 = image.model_sources(m, lam, cuda, nphot_scat=100000)
    assert torch.equal(a0, a1)
    i0 = plan.run(a0, s0).sum().item()
    i1 = plan.run(a1, s1).sum().item()
    assert i1 > 2.0 * i0    # at 1 micron a 150 K (r/au)^-0.5 disk shines by scattered starlight
    # the source function is the thermal part plus ksca rho J / alpha with the plan's J
    rho, T = image.model_state(m, cuda)
    ka, ks = image.opacities(m.grid, lam)
    kat = torch.as_tensor(ka, device=cuda)
    J = scatter.ScatterPlan(m.grid, lam, ka, ks, 100000, device=cuda).run(
        rho, image.thermal_emissivity(rho, T, kat, lam))
    _, s = image.source_terms(rho, T, kat, torch.as_tensor(ks, device=cuda), lam, J=J)
    assert torch.equal(s.to(torch.float32), s1)


def test_scattering_mode_max_zero_drops_scattering(cuda):
    m = _cases.image_model("disk", nr=12, ntheta=12)
    lam = np.array([1.0])
    a_on, _ = image.model_sources(m, lam, cuda, nphot_scat=1000)
    a_off, _ = image.model_sources(m, lam, cuda, nphot_scat=1000, scattering=False)
    rho, _ = image.model_state(m, cuda)
    ka, _ = image.opacities(m.grid, lam)
    assert torch.allclose(a_off.double(), torch.as_tensor(ka, device=cuda).T @ rho, rtol=1e-6)
    assert torch.all(a_on >= a_off) and torch.any(a_on > a_off)


def test_run_scattering_api(cuda):
    m = _cases.image_model("mirror", nr=10, ntheta=8)
    m.set_camera_wavelength(np.array([0.8, 1.6]))
    out = m.run_scattering(nphot=5000, loadlambda=True, code="gb300")
    g = m.grid
    assert out is g.scattering_phase
    assert g.scattering_phase.shape == (2,) + np.asarray(g.density[0]).shape
    assert np.allclose(g.scattering_phase_freq, 2.99792458e10 / (np.array([0.8, 1.6]) * 1e-4))
    J = scatter.mean_intensity(m, np.array([0.8, 1.6]), 5000, device=cuda)
    assert np.array_equal(g.scattering_phase.reshape(2, -1), J.cpu().numpy())


def test_sed_includes_scattered_starlight(cuda):
    m = _cases.image_model("mirror", nr=16, ntheta=16)
    lam = np.array([0.7, 1.0, 1300.0])
    m.set_camera_wavelength(lam)
    with_s = m.run_sed(name="a", nphot=50000, loadlambda=True, dpc=140, incl=30, npix=64,
                       code="gb300").flux.copy()
    # nphot = 0: scattering extinguishes but adds no source
    without = m.run_sed(name="b", nphot=0, loadlambda=True, dpc=140, incl=30, npix=64,
                        code="gb300").flux.copy()
    assert np.all(with_s[:2] > without[:2])
    assert with_s[2] == pytest.approx(without[2], rel=1e-6)   # albedo 0 at 1.3 mm
    # scattering_mode_max = 0 removes the scattering extinction too
    off = m.run_sed(name="c", nphot=50000, loadlambda=True, dpc=140, incl=30, npix=64,
                    scattering_mode_max=0, code="gb300").flux
    assert np.all(off[:2] >= without[:2])
