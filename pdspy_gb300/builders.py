"""Density builders on the device, differentiable in their parameters.

pdspy builds each model's density on the host in numpy: the power-law disk
(pdspy/modeling/Disk.py:48-135) and the Ulrich envelope with an outflow cavity
(pdspy/modeling/UlrichEnvelopeExtended.py:37-110), whose streamline angle mu0 is found cell
by cell with scipy's brenth in a Python loop (:68-75) -- seconds per walker on a
256 x 256 grid, repeated for every MCMC walker.  Here both are float64 torch expressions
that run on the GPU for a whole grid at once and carry gradients with respect to every
parameter:

* ``disk_density`` -- the same formula, masks and normalisation as Disk.density
  (Sigma ~ R^-(plrho - plh) between rmin and rmax, h = h0 AU (R/AU)^plh, mass fixed by a
  1000-point trapezoid in log R).
* ``ulrich_envelope_density`` -- mu0 in closed form: mu0^3 + p mu0 + q = 0 with
  p = r/Rc - 1 and q = -mu r/Rc has one real root for p >= 0 or a positive discriminant
  (Cardano) and three otherwise (trigonometric form); the streamline root is the one on
  the side of mu with |mu0| >= |mu|, the root brenth returns on [-1, 1] away from the
  midplane (where pdspy replaces the formula by its own limits).  Two Newton steps polish
  it.  Then the reference's density, midplane limits, radial mask
  ((r >= rmax) xor (r <= rmin)), cavity factor and mass normalisation by nested
  trapezoids over theta and r.
"""
import math

import numpy as np
import torch

from .constants import AU, M_sun, pi_pdspy


def _t(x, dev):
    if torch.is_tensor(x):
        return x.to(device=dev, dtype=torch.float64)
    return torch.as_tensor(np.asarray(x, np.float64), device=dev)


def _mesh(r_au, theta, phi, dev):
    r = _t(r_au, dev)
    th = _t(theta, dev)
    ph = _t(phi, dev)
    return torch.meshgrid(r * AU, th, ph, indexing="ij")


def disk_density(r_au, theta, phi, mass, rmin, rmax, plrho, h0, plh, device=None):
    """pdspy Disk(mass, rmin, rmax, plrho, h0, plh).density(r, theta, phi): float64
    [nr, ntheta, nphi] (g/cm^3); mass, plrho, h0, plh may be tensors with gradients."""
    dev = device or (mass.device if torch.is_tensor(mass) else torch.device("cpu"))
    rt, tt, _ = _mesh(r_au, theta, phi, dev)
    mass, plrho, h0, plh = (_t(v, dev) for v in (mass, plrho, h0, plh))
    gamma = plrho - plh
    rr = rt * torch.sin(tt)
    zz = rt * torch.cos(tt)
    rin, rout = rmin * AU, rmax * AU
    m = mass * M_sun
    Sigma0 = (2 - gamma) * m / (2 * pi_pdspy * (1 * AU) ** gamma) / \
        (rout ** (-gamma + 2) - rin ** (-gamma + 2))

    def surface(rau):
        S = Sigma0 * rau ** (-gamma)
        inside = ~((rau >= rout / AU) ^ (rau <= rin / AU))
        return torch.where(inside, S, torch.zeros_like(S))

    rh = torch.logspace(math.log10(rmin), math.log10(rmax), 1000, dtype=torch.float64, device=dev)
    scale = m / (2 * math.pi * torch.trapezoid(rh * AU * surface(rh), rh * AU))
    Sigma = surface(rr / AU) * scale
    h = h0 * AU * (rr / AU) ** plh
    return Sigma / (math.sqrt(2 * math.pi) * h) * torch.exp(-0.5 * (zz / h) ** 2)


def streamline_mu0(x, mu):
    """Root mu0 of mu0^3 - mu0 (1 - x) - mu x = 0 (x = r / Rc) on the side of mu with
    |mu0| >= |mu|: float64 tensors of the broadcast shape.  The root is found without
    gradients; one Newton step taken with gradients carries d mu0 = -(df/dx dx + df/dmu dmu)
    / (df/dmu0), the implicit derivative."""
    with torch.no_grad():
        xd, md = x.detach(), mu.detach()
        p = xd - 1.0
        q = -md * xd
        D = (0.5 * q) ** 2 + (p / 3.0) ** 3
        sD = torch.sqrt(torch.clamp(D, min=0.0))
        cbrt = lambda v: torch.sign(v) * torch.abs(v) ** (1.0 / 3.0)
        one = cbrt(-0.5 * q + sD) + cbrt(-0.5 * q - sD)        # Cardano, one real root
        pn = torch.clamp(p, max=-1e-300)
        m = 2.0 * torch.sqrt(-pn / 3.0)
        ph = torch.arccos(torch.clamp(3.0 * q / (pn * m), -1.0, 1.0)) / 3.0
        roots = torch.stack([m * torch.cos(ph - 2.0 * math.pi * k / 3.0) for k in range(3)])
        big = torch.full_like(roots, 1e300)
        up = torch.where(roots >= md - 1e-9, roots, big).min(0).values
        down = torch.where(roots <= md + 1e-9, roots, -big).max(0).values
        mu0 = torch.where((D >= 0) | (p >= 0), one, torch.where(md >= 0, up, down))
        for _ in range(2):
            f = mu0 ** 3 - mu0 * (1.0 - xd) - md * xd
            df = 3.0 * mu0 ** 2 - (1.0 - xd)
            ok = torch.abs(df) > 1e-8
            mu0 = torch.where(ok, mu0 - f / torch.where(ok, df, torch.ones_like(df)), mu0)
    f = mu0 ** 3 - mu0 * (1.0 - x) - mu * x
    df = 3.0 * mu0 ** 2 - (1.0 - x)
    ok = torch.abs(df) > 1e-8
    return torch.where(ok, mu0 - f / torch.where(ok, df, torch.ones_like(df)), mu0)


def ulrich_envelope_density(r_au, theta, phi, mass, rmin, rmax, rcent, cavpl=1.0,
                            cavrfact=0.2, theta_open=1.0, zoffset=1.0, device=None):
    """pdspy UlrichEnvelopeExtended(mass, rmin, rmax, rcent, cavpl, cavrfact, theta_open,
    zoffset).density(r, theta, phi): float64 [nr, ntheta, nphi] (g/cm^3).  mass, rcent
    and cavrfact may be tensors with gradients; cavpl, theta_open and zoffset only move
    the cavity's edge (a mask) and have none."""
    dev = device or (mass.device if torch.is_tensor(mass) else torch.device("cpu"))
    rr, tt, _ = _mesh(r_au, theta, phi, dev)
    mass, rcent, cavpl, cavrfact, theta_open, zoffset = (
        _t(v, dev) for v in (mass, rcent, cavpl, cavrfact, theta_open, zoffset))
    rin, rout = rmin * AU, rmax * AU
    m = mass * M_sun
    rc = rcent * AU
    z0 = zoffset * AU
    th_o = theta_open * math.pi / 180.0
    cava = (rout * torch.sin(th_o / 2) / AU / torch.tan(th_o / 2) - z0 / AU) * \
        (rout * torch.sin(th_o / 2) / AU) ** -cavpl
    mu = torch.cos(tt)
    RR = rr * torch.sin(tt)
    zz = rr * torch.cos(tt)
    x = rr / rc
    mid = torch.abs(mu) < 1.0e-10
    mu0 = streamline_mu0(x, mu)
    mu0 = torch.where(mid, torch.ones_like(mu0), mu0)   # midplane: replaced below
    rho = x ** (-1.5) * (1 + mu / mu0) ** (-0.5) * (mu / mu0 + 2 * mu0 ** 2 / x) ** (-1)
    # midplane limits, evaluated only where they apply (no NaN in the unused branch)
    in1, in2 = mid & (rr < rc), mid & (rr > rc)
    xs = torch.where(in1, x, torch.full_like(x, 0.5))
    xl = torch.where(in2, x, torch.full_like(x, 2.0))
    rho = torch.where(in1, xs ** (-0.5) * (1.0 - xs) ** (-1) / 2.0, rho)
    rho = torch.where(in2, (2.0 * xl - 1) ** (-0.5) * (xl - 1.0) ** (-1), rho)
    rho = torch.where((rr >= rout) ^ (rr <= rin), torch.zeros_like(rho), rho)
    cav = torch.abs(zz) / AU - z0 / AU - cava * (RR / AU) ** cavpl > 0.0
    rho = torch.where(cav, rho * cavrfact, rho)
    inner = torch.trapezoid(rho * rr ** 2 * torch.sin(tt), tt, dim=1)
    total = torch.trapezoid(inner, rr[:, 0, :], dim=0)
    th = _t(theta, dev)
    c = 2.0 if float(th.max()) > pi_pdspy / 2 else 4.0
    mdot = m / (c * pi_pdspy * total)[0]
    return rho * mdot
