"""The backend bound to pdspy's own classes (pdspy/modeling/Model.py, Grid.py, Star.py,
pdspy/dust/Dust.py, Disk.py), loaded from a pdspy checkout named by PDSPY_SOURCE (see
tests/_pdspy_shim.py); skipped without one.

Everything the GPU plan receives is read from the model through thermal.grid_arrays,
thermal._stars, thermal.opacity_on_grid and thermal.stack_density.  On pdspy's real
objects, built for config 0 the way a pdspy user builds them (Grid.set_spherical_grid in au,
Star from mass/luminosity/temperature, Dust.set_properties in cm, Disk.density), these give
bit for bit the inputs the package's own mirror classes give, so the kernels see identical
grids, stars, opacities and densities; the CPU restatement run on them gives identical
temperatures.  The dispatch branch INTEGRATION.md adds to Model.run_thermal/run_image/
run_sed/run_visibilities reaches this package with pdspy's keywords, and the result is
written back into the real Grid as pdspy's radmc3d branch leaves it."""
import numpy as np
import pytest

from pdspy_gb300 import image, thermal, workloads
from pdspy_gb300.constants import AU
from tests import _cases, _pdspy_shim

pd = _pdspy_shim.load()
pytestmark = pytest.mark.skipif(pd is None, reason="PDSPY_SOURCE does not name a pdspy checkout")

MRW = dict(modified_random_walk=True, mrw_gamma=2, mrw_tauthres=10, mrw_count_trigger=100)


def _real_config0(nr=100, ntheta=100):
    """Config 0 with pdspy's classes: 0.1-100 au log r edges, theta over [0, pi], a 4000 K
    2 R_sun star, the analytic dust (no g: pdspy's radmc3d path has none) and the 1e-4 Msun
    power-law disk."""
    m = pd.Model()
    w1 = np.logspace(-1, 2, nr + 1)
    w2 = np.linspace(0.0, np.pi, ntheta + 1)
    w3 = np.array([0.0, 2 * np.pi])
    m.grid.set_spherical_grid(w1, w2, w3)
    lam = workloads.lam_grid()
    m.grid.lam = lam
    m.grid.add_star(pd.Star(mass=0.5, luminosity=workloads.star_luminosity(2.0, 4000.0),
                            temperature=4000.0))
    mine = workloads.analytic_dust(lam, g=None)
    d = pd.Dust()
    d.set_properties(lam * 1.0e-4, mine.kabs, mine.ksca)
    disk = pd.Disk(mass=1e-4, rmin=0.1, rmax=100.0, plrho=2.25, h0=0.1, plh=1.25)
    m.grid.add_density(disk.density(m.grid.r, m.grid.theta, m.grid.phi), d)
    return m


def test_plan_inputs_from_pdspys_classes_equal_the_mirrors():
    real = _real_config0()
    mirror = workloads.small_disk(g=None)
    for a, b in zip(thermal.grid_arrays(real.grid), thermal.grid_arrays(mirror.grid)):
        assert np.array_equal(a, b)
    for a, b in zip(thermal._stars(real.grid), thermal._stars(mirror.grid)):
        assert np.array_equal(a, b)
    ka, ks, g = thermal.opacity_on_grid(real.grid.dust[0], real.grid.lam)
    kb, kt, h = thermal.opacity_on_grid(mirror.grid.dust[0], mirror.grid.lam)
    assert np.array_equal(ka, kb) and np.array_equal(ks, kt) and g is None and h is None
    assert np.array_equal(thermal.stack_density(real.grid), thermal.stack_density(mirror.grid))
    assert thermal.grid_arrays(real.grid)[0][0] == 0.1 * AU


def test_restatement_on_pdspys_objects_gives_the_mirrors_temperatures():
    real, mirror = _real_config0(24, 24), workloads.small_disk(nr=24, ntheta=24, g=None,
                                                                 rgrid=100.0)
    mirror.grid.density = [thermal.stack_density(real.grid)[0].astype(np.float64)]
    kw = dict(mrw=True, mrw_gamma=2.0, mrw_tauthres=10.0, mrw_count_trigger=100)
    a = _cases.run_oracle(real, 3000, seed=3, **kw)
    b = _cases.run_oracle(mirror, 3000, seed=3, **kw)
    assert np.array_equal(a["temperature"], b["temperature"])


def test_dispatch_branch_and_write_back(monkeypatch):
    """INTEGRATION.md's branch on pdspy's Model: code="gb300" reaches thermal.run_thermal
    with run_disk_model's keywords (run_disk_model.py:251-255), which are all understood;
    the temperatures land in the real Grid as a list of float64 (nr, ntheta, nphi) arrays."""
    Model = pd.Model
    orig = Model.run_thermal

    def run_thermal(self, nphot=1e6, code="radmc3d", **keywords):
        if code == "gb300":
            return thermal.run_thermal(self, nphot=nphot, **keywords)
        return orig(self, nphot=nphot, code=code, **keywords)

    monkeypatch.setattr(Model, "run_thermal", run_thermal)
    seen = {}

    def fake_gpu_run(model, nphot=1e6, **keywords):      # no GPU here: record, then fill
        seen["model"], seen["nphot"] = model, nphot
        seen["opts"] = thermal._options(keywords)
        ref = _cases.run_oracle(model, int(nphot), seed=seen["opts"].get("seed", 0),
                                mrw=True, mrw_gamma=2.0, mrw_tauthres=10.0,
                                mrw_count_trigger=100)
        model.grid.temperature = [np.array(t, dtype=np.float64) for t in ref["temperature"]]
        return {"status": 0}

    monkeypatch.setattr(thermal, "run_thermal", fake_gpu_run)
    m = _real_config0(24, 24)
    import warnings
    with warnings.catch_warnings():
        warnings.simplefilter("error")        # every run_disk_model keyword is understood
        m.run_thermal(code="gb300", nphot=2000, verbose=False, setthreads=16, timelimit=3600,
                      nice=19, iseed=4, **MRW)
    assert seen["model"] is m and seen["nphot"] == 2000
    o = seen["opts"]
    assert o["mrw"] is True and o["mrw_gamma"] == 2 and o["mrw_tauthres"] == 10
    assert o["mrw_count_trigger"] == 100 and o["timelimit"] == 3600 and o["seed"] == 4
    T = m.grid.temperature
    assert isinstance(T, list) and len(T) == 1
    assert T[0].dtype == np.float64 and T[0].shape == m.grid.density[0].shape == (24, 24, 1)
    # run_image reads the real grid's lists the same way (model_state on the host here)
    import torch
    rho, Tt = image.model_state(m, torch.device("cpu"))
    assert rho.shape == Tt.shape == (1, 24 * 24)
    assert image.mean_temperature(rho, Tt).shape == (24 * 24,)
