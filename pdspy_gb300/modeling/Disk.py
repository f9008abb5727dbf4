"""Power-law disk density; restates pdspy/modeling/Disk.py:48-135.

rho(r, theta, phi) = Sigma(R) / (sqrt(2 pi) h(R)) exp(-z^2 / 2 h^2) with
Sigma ~ R^-gamma (gamma = plrho - plh) between rmin and rmax, h = h0 AU (R/AU)^plh, and
Sigma rescaled so that 2 pi int R Sigma dR (trapezoid over 1000 log radii) equals the
disk mass -- the same normalisation, constants and masks as the reference, so the
density fields agree to rounding.
"""
import numpy

from ..constants import AU, M_sun, pi_pdspy


class Disk:
    def __init__(self, mass=1.0e-3, rmin=0.1, rmax=300, plrho=2.37, h0=0.1, plh=58. / 45.,
                 dust=None, **ignored):
        self.mass = mass
        self.rmin = rmin
        self.rmax = rmax
        self.plrho = plrho
        self.h0 = h0
        self.plh = plh
        if dust is not None:
            self.dust = dust

    def density(self, x1, x2, x3, coordsys="spherical", normalize=True):
        if coordsys != "spherical":
            raise ValueError("only spherical coordinates are supported")
        rt, tt, pp = numpy.meshgrid(numpy.asarray(x1) * AU, x2, x3, indexing='ij')
        rr = rt * numpy.sin(tt)
        zz = rt * numpy.cos(tt)
        Sigma = self.surface_density(rr / AU, normalize=normalize)
        h = self.scale_height(rr / AU)
        return Sigma / (numpy.sqrt(2 * numpy.pi) * h) * numpy.exp(-0.5 * (zz / h)**2)

    def surface_density(self, r, normalize=True):
        rin = self.rmin * AU
        rout = self.rmax * AU
        mass = self.mass * M_sun
        gamma = self.plrho - self.plh
        Sigma0 = (2 - gamma) * mass / (2 * pi_pdspy * (1 * AU)**(gamma)) / \
            (rout**(-gamma + 2) - rin**(-gamma + 2))
        r = numpy.asarray(r, dtype=numpy.float64)
        Sigma = Sigma0 * r**(-gamma)
        Sigma[(r >= rout / AU) ^ (r <= rin / AU)] = 0e0
        if (r > 0).any() and (r == 0).any():
            dr = r[r > 0].min()
            Sigma[r == 0] = Sigma0 * (0.7 * dr)**(-gamma)
        if normalize:
            r_high = numpy.logspace(numpy.log10(self.rmin), numpy.log10(self.rmax), 1000)
            Sigma_high = self.surface_density(r_high, normalize=False)
            scale = mass / (2 * numpy.pi * numpy.trapezoid(r_high * AU * Sigma_high, r_high * AU))
            Sigma *= scale
        return Sigma

    def scale_height(self, r):
        return self.h0 * AU * r**self.plh
