"""Rotating-collapse (Ulrich) envelope with a conical outflow cavity.

Restates pdspy/modeling/UlrichEnvelopeExtended.py:37-110: the streamline origin mu0 of
every cell solves mu0^3 - mu0 (1 - r/Rc) - mu r/Rc = 0 with scipy's brenth on [-1, 1]
(as the reference does), rho ~ (r/Rc)^-1.5 (1 + mu/mu0)^-0.5 (mu/mu0 + 2 mu0^2 Rc/r)^-1,
the midplane limits of the reference, zero density outside [rmin, rmax], the cavity
|z| - z0 - a R^cavpl > 0 scaled by cavrfact, and the mass normalisation by nested
trapezoids over theta and r.
"""
import numpy
from scipy.optimize import brenth

from ..constants import AU, M_sun, pi_pdspy


class UlrichEnvelopeExtended:
    def __init__(self, mass=1.0e-3, rmin=0.1, rmax=1000, rcent=30, cavpl=1.0, cavrfact=0.2,
                 theta_open=1., zoffset=1., dust=None, **ignored):
        self.mass = mass
        self.rmin = rmin
        self.rmax = rmax
        self.rcent = rcent
        self.cavpl = cavpl
        self.cavrfact = cavrfact
        self.theta_open = theta_open
        self.zoffset = zoffset
        if dust is not None:
            self.dust = dust

    def density(self, r, theta, phi):
        rin = self.rmin * AU
        rout = self.rmax * AU
        mass = self.mass * M_sun
        rcent = self.rcent * AU
        cavz0 = self.zoffset * AU
        cavpl = self.cavpl
        cavrfact = self.cavrfact
        theta_open = self.theta_open * numpy.pi / 180.
        cava = (rout * numpy.sin(theta_open / 2) / AU / numpy.tan(theta_open / 2) - cavz0 / AU) * \
            (rout * numpy.sin(theta_open / 2) / AU)**-cavpl
        theta = numpy.asarray(theta)
        rr, tt, pp = numpy.meshgrid(numpy.asarray(r) * AU, theta, phi, indexing='ij')
        mu = numpy.cos(tt)
        RR = rr * numpy.sin(tt)
        zz = rr * numpy.cos(tt)

        def func(mu0, r, mu, R_c):
            return mu0**3 - mu0 * (1 - r / R_c) - mu * (r / R_c)

        mu0 = mu * 0.
        for ir in range(rr.shape[0]):
            for it in range(rr.shape[1]):
                mu0[ir, it, 0] = brenth(func, -1.0, 1.0, args=(rr[ir, it, 0], mu[ir, it, 0], rcent))
        if mu0.shape[2] > 1:
            mu0[:, :, 1:] = mu0[:, :, 0:1]
        rho0 = 1.0
        with numpy.errstate(all="ignore"):
            rho = rho0 * (rr / rcent)**(-1.5) * (1 + mu / mu0)**(-0.5) * \
                (mu / mu0 + 2 * mu0**2 * rcent / rr)**(-1)
            mid1 = (numpy.abs(mu) < 1.0e-10) & (rr < rcent)
            rho[mid1] = rho0 * (rr[mid1] / rcent)**(-0.5) * (1. - rr[mid1] / rcent)**(-1) / 2.
            mid2 = (numpy.abs(mu) < 1.0e-10) & (rr > rcent)
            rho[mid2] = rho0 * (2. * rr[mid2] / rcent - 1)**(-0.5) * (rr[mid2] / rcent - 1.)**(-1)
        rho[(rr >= rout) ^ (rr <= rin)] = 0e0
        rho[numpy.abs(zz) / AU - cavz0 / AU - cava * (RR / AU)**cavpl > 0.0] *= cavrfact
        inner = numpy.trapezoid(rho * rr**2 * numpy.sin(tt), tt, axis=1)
        if theta.max() > pi_pdspy / 2:
            mdot = mass / (2 * pi_pdspy * numpy.trapezoid(inner, rr[:, 0, :], axis=0))[0]
        else:
            mdot = mass / (4 * pi_pdspy * numpy.trapezoid(inner, rr[:, 0, :], axis=0))[0]
        rho *= mdot
        return rho
