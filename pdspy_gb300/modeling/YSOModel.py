"""Young-stellar-object builder; mirrors the parts of pdspy/modeling/YSOModel.py on the
thermal/imaging path: add_star (:29-31), set_spherical_grid (:47-63), add_disk
(:69-115, dust density only) and add_ulrichextended_envelope (:595-651, dust density
only)."""
import numpy

from .Disk import Disk
from .Model import Model
from .Star import Star
from .UlrichEnvelopeExtended import UlrichEnvelopeExtended


class YSOModel(Model):
    def add_star(self, mass=0.5, luminosity=1, temperature=4000.):
        self.grid.add_star(Star(mass=mass, luminosity=luminosity, temperature=temperature))

    def set_spherical_grid(self, rmin, rmax, nr, ntheta, nphi, log=True, code="radmc3d"):
        if log:
            r = numpy.logspace(numpy.log10(rmin), numpy.log10(rmax), nr)
        else:
            r = numpy.linspace(rmin, rmax, nr)
        if code == "hyperion":
            r = numpy.hstack([0.0, r])
            theta = numpy.linspace(0.0, numpy.pi, ntheta)
        else:
            theta = numpy.linspace(0.0, numpy.pi / 2, ntheta)
        phi = numpy.linspace(0.0, 2 * numpy.pi, nphi)
        self.grid.set_spherical_grid(r, theta, phi)

    def add_disk(self, mass=1.0e-3, rmin=0.1, rmax=300, plrho=2.37, h0=0.1, plh=58. / 45.,
                 dust=None, **ignored):
        self.disk = Disk(mass=mass, rmin=rmin, rmax=rmax, plrho=plrho, h0=h0, plh=plh, dust=dust)
        if dust is not None:
            self.grid.add_density(self.disk.density(self.grid.r, self.grid.theta, self.grid.phi),
                                  dust)

    def add_ulrichextended_envelope(self, mass=1.0e-3, rmin=0.1, rmax=1000, rcent=300, cavpl=1.0,
                                    cavrfact=0.2, theta_open=45., zoffset=1., dust=None,
                                    rcent_ne_rdisk=False, **ignored):
        if not rcent_ne_rdisk and hasattr(self, 'disk'):
            rcent = self.disk.rmax
        self.envelope = UlrichEnvelopeExtended(mass=mass, rmin=rmin, rmax=rmax, rcent=rcent,
                                               cavpl=cavpl, cavrfact=cavrfact,
                                               theta_open=theta_open, zoffset=zoffset, dust=dust)
        if dust is not None:
            self.grid.add_density(self.envelope.density(self.grid.r, self.grid.theta,
                                                        self.grid.phi), dust)
