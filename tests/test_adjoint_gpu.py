"""Adjoint ray trace, adjoint DFT and the chi^2 gradient against float64 torch autograd
and float64 central differences."""
import numpy as np
import pytest
import torch

from pdspy_gb300 import adjoint, image, thermal, vis, workloads
from tests import _cases, _imageref

pytestmark = pytest.mark.gpu

TOL = 1e-4   # relative (2-norm) error of gradients against float64 references


def relerr(a, b):
    a = np.asarray(a, dtype=np.float64).ravel()
    b = np.asarray(b, dtype=np.float64).ravel()
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("kind,incl,nostar", [("disk", 50.0, False), ("envelope", 20.0, True),
                                              ("mirror", 80.0, False)])
def test_image_adjoint_vs_float64_autograd(cuda, kind, incl, nostar):
    m = _cases.image_model(kind, nr=10, ntheta=10)
    npix = 10
    r, t, p = thermal.grid_arrays(m.grid)
    pixel_cm = 2.1 * r[-1] / npix
    lam = np.array([1300.0, 50.0])
    plan = image.ImagePlan(m.grid, npix, pixel_cm, lam, incl=incl, pa=15.0, nostar=nostar,
                           max_refine=1)
    a32, s32 = image.model_sources(m, lam, cuda)
    rng = np.random.default_rng(1)
    w = torch.as_tensor(rng.random((2, npix, npix)), device=cuda)
    # GPU: image + adjoint
    a = a32.clone().requires_grad_(True)
    s = s32.clone().requires_grad_(True)
    (image.RayTrace.apply(a, s, plan) * w).sum().backward()
    # float64 reference on the same float32 inputs
    segs, star = _imageref.segments(m, npix, pixel_cm, plan.levels, incl, 15.0, 0.0)
    a64 = a32.double().cpu().requires_grad_(True)
    s64 = s32.double().cpu().requires_grad_(True)
    ref = _imageref.image(a64, s64, segs, star, image.star_flux_1pc(m.grid, lam), npix,
                          pixel_cm, nostar=nostar)
    (ref * w.cpu()).sum().backward()
    assert relerr(a.grad.cpu(), a64.grad) < TOL
    assert relerr(s.grad.cpu(), s64.grad) < TOL


def test_dft_and_adjoint_vs_float64(cuda):
    rng = np.random.default_rng(3)
    img = torch.tensor(rng.random((24, 20)) * 1e-3, device=cuda, requires_grad=True)
    u, v = vis.synthetic_uv(500, seed=4)
    geo = vis.pixel_grid(20, 0.02)
    ut = torch.as_tensor(u, dtype=torch.float32, device=cuda)
    vt = torch.as_tensor(v, dtype=torch.float32, device=cuda)
    geo = (geo[0], geo[1], -(24 // 2) * geo[3], geo[3])
    re, im = vis.VisDFT.apply(img, ut, vt, geo)
    gr = torch.as_tensor(rng.normal(size=500), device=cuda)
    gi = torch.as_tensor(rng.normal(size=500), device=cuda)
    ((re * gr).sum() + (im * gi).sum()).backward()
    i64 = img.detach().double().cpu().requires_grad_(True)
    rr, ii = _imageref.dft(i64, torch.as_tensor(ut.double().cpu()),
                           torch.as_tensor(vt.double().cpu()), *geo)
    ((rr * gr.cpu()).sum() + (ii * gi.cpu()).sum()).backward()
    assert relerr(re.detach().cpu(), rr.detach()) < 1e-5
    assert relerr(im.detach().cpu(), ii.detach()) < 1e-5
    assert relerr(img.grad.cpu(), i64.grad) < TOL


def _problem(cuda, nuv=300):
    m = workloads.disk_envelope(nr=12, ntheta=12, mdisk=1e-3, menv=0.01, renv=500.0)
    g = m.grid
    rr = np.meshgrid(g.r, g.theta, g.phi, indexing="ij")[0]
    g.temperature = [30.0 * rr ** -0.4, 20.0 * rr ** -0.3]
    u, v = vis.synthetic_uv(nuv, seed=7)
    data = vis.UVData(u, v, np.zeros(nuv), np.zeros(nuv), np.full(nuv, 1e6))
    prob = adjoint.Chi2Problem(m, data, npix=12, pixelsize=0.5, dpc=140.0, incl=40.0,
                               max_refine=1, device=cuda)
    return m, prob


def _reference_chi2(prob, rho64, segs, star):
    alpha, S = image.source_terms(rho64, prob.T.cpu(), prob.kabs.cpu(), prob.ksca.cpu(),
                                  prob.lam_um)
    img = _imageref.image(alpha, S, segs, star, image.star_flux_1pc(prob.grid, prob.lam_um),
                          prob.npix, prob.pixel_cm) * (prob.omega / 1e-23)
    re, im = _imageref.dft(img[0], prob.u.double().cpu(), prob.v.double().cpu(), *prob.geometry)
    return vis.chisq(re, im, prob.re_d.cpu(), prob.im_d.cpu(), prob.w.cpu())


def test_chi2_density_gradient_vs_float64_autograd(cuda):
    m, prob = _problem(cuda)
    rho = prob.rho0.clone().requires_grad_(True)
    chi = prob.chi2(rho)
    chi.backward()
    segs, star = _imageref.segments(m, prob.npix, prob.pixel_cm, prob.plan.levels, 40.0)
    rho64 = prob.rho0.cpu().clone().requires_grad_(True)
    ref = _reference_chi2(prob, rho64, segs, star)
    ref.backward()
    assert abs(chi.item() / ref.item() - 1) < 1e-5
    assert relerr(rho.grad.cpu(), rho64.grad) < TOL


def test_chi2_parameter_gradient_vs_autograd_and_central_differences(cuda):
    m, prob = _problem(cuda)
    p0 = [1e-3, 0.1, 1.25, 1.0]
    params = torch.tensor(p0, dtype=torch.float64, device=cuda, requires_grad=True)
    chi = prob.chi2_params(params, 0.1, 100.0)
    chi.backward()
    segs, star = _imageref.segments(m, prob.npix, prob.pixel_cm, prob.plan.levels, 40.0)

    def ref_chi(pv):
        rho = torch.cat([adjoint.disk_density_torch(
            m.grid.r, m.grid.theta, m.grid.phi, pv[0], 0.1, 100.0, pv[1], pv[2], pv[3]
        ).reshape(1, -1), prob.rho0[1:].cpu()], 0)
        return _reference_chi2(prob, rho, segs, star)

    pr = torch.tensor(p0, dtype=torch.float64, requires_grad=True)
    ref = ref_chi(pr)
    ref.backward()
    assert relerr(params.grad.cpu(), pr.grad) < TOL
    fd = []
    for i in range(4):
        h = 1e-5 * abs(p0[i])
        up = torch.tensor(p0, dtype=torch.float64); up[i] += h
        dn = torch.tensor(p0, dtype=torch.float64); dn[i] -= h
        fd.append((ref_chi(up).item() - ref_chi(dn).item()) / (2 * h))
    assert relerr(pr.grad.numpy(), fd) < 1e-5
    assert relerr(params.grad.cpu().numpy(), fd) < TOL
