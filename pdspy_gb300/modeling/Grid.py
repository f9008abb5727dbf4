"""Grid state container; mirrors pdspy/modeling/Grid.py:7-87."""
import numpy


class Grid:
    def __init__(self):
        self.density = []
        self.dust = []
        self.temperature = []
        self.stars = []

    def add_density(self, density, dust):
        self.density.append(density)
        self.dust.append(dust)

    def add_star(self, star):
        self.stars.append(star)

    def add_temperature(self, temperature):
        self.temperature.append(temperature)

    def set_spherical_grid(self, w1, w2, w3):
        self.coordsystem = "spherical"
        w1, w2, w3 = numpy.asarray(w1), numpy.asarray(w2), numpy.asarray(w3)
        self.r = 0.5 * (w1[0:w1.size - 1] + w1[1:w1.size])
        self.theta = 0.5 * (w2[0:w2.size - 1] + w2[1:w2.size])
        self.phi = 0.5 * (w3[0:w3.size - 1] + w3[1:w3.size])
        self.w1 = w1
        self.w2 = w2
        self.w3 = w3

    def set_wavelength_grid(self, lmin, lmax, nlam, log=False):
        if log:
            self.lam = numpy.logspace(numpy.log10(lmin), numpy.log10(lmax), nlam)
        else:
            self.lam = numpy.linspace(lmin, lmax, nlam)
