"""Host-side logic of the Python layer that needs no GPU: keyword handling of run_image /
run_sed / run_scattering, camera wavelengths, pixel grids and the gridded-sampling frame."""
import numpy as np
import pytest

from pdspy_gb300 import image, scatter, vis
from pdspy_gb300.constants import arcsec


class _M:
    camera_wavelength = [870.0, 1300.0]


def test_camera_wavelengths_follow_radmc3d_lambda_and_loadlambda():
    assert np.array_equal(image.camera_wavelengths(_M(), "1300"), [1300.0])
    assert np.array_equal(image.camera_wavelengths(_M(), "870 1300"), [870.0, 1300.0])
    assert np.array_equal(image.camera_wavelengths(_M(), 10.0), [10.0])
    assert np.array_equal(image.camera_wavelengths(_M(), None, loadlambda=True), [870.0, 1300.0])


def test_scattering_keywords():
    assert scatter.maxtauabs_of({}) == 30.0
    assert scatter.maxtauabs_of({"mc_scat_maxtauabs": 5}) == 5.0
    assert scatter.scattering_enabled({})
    assert scatter.scattering_enabled({"scattering_mode_max": 1})
    assert not scatter.scattering_enabled({"scattering_mode_max": 0})
    kw = image._scat_keywords({"mc_scat_maxtauabs": 5, "iseed": 9, "setthreads": 4})
    assert kw == dict(scattering=True, maxtauabs=5.0, seed=9)


def test_pixel_grid_centres_pixel_n_over_2():
    x0, dx, y0, dy = vis.pixel_grid(256, 0.01)
    assert dx == dy == 0.01 * arcsec
    assert x0 + 128 * dx == 0.0 and y0 == x0


def test_grid_frame_puts_the_centre_pixel_on_the_padded_centre():
    geo = vis.pixel_grid(64, 0.02)
    N, du, dv, xc, yc = vis._grid_frame(64, 4, geo)
    assert N == 256 and du == pytest.approx(1.0 / (256 * geo[1]))
    assert xc == pytest.approx(0.0, abs=1e-20) and yc == pytest.approx(0.0, abs=1e-20)


def test_source_terms_add_isotropic_scattering():
    import torch
    rho = torch.tensor([[1e-18, 2e-18, 0.0]], dtype=torch.float64)
    T = torch.tensor([[50.0, 80.0, 10.0]], dtype=torch.float64)
    ka = torch.tensor([[2.0]], dtype=torch.float64)
    ks = torch.tensor([[3.0]], dtype=torch.float64)
    J = torch.tensor([[1e-9, 2e-9, 3e-9]], dtype=torch.float64)
    a0, s0 = image.source_terms(rho, T, ka, ks, [1300.0])
    a1, s1 = image.source_terms(rho, T, ka, ks, [1300.0], J=J)
    assert torch.equal(a0, a1)
    expect = s0 + (3.0 * rho * J) / torch.where(a0 > 0, a0, torch.ones_like(a0))
    assert torch.allclose(s1[:, :2], expect[:, :2], rtol=1e-14)
    assert s1[0, 2] == 0.0     # empty cell: no extinction, no source
