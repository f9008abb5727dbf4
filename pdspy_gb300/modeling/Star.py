"""Blackbody point star; mirrors pdspy/modeling/Star.py:7-16."""
import numpy

from ..constants import L_sun, R_sun, sigma


class Star:
    def __init__(self, mass=0.5, luminosity=1.0, temperature=4000., x=0.0, y=0.0, z=0.0):
        self.mass = mass
        self.luminosity = luminosity
        self.temperature = temperature
        self.radius = (luminosity * L_sun / (4 * numpy.pi * sigma * temperature**4))**(1. / 2) / R_sun
        self.x = x
        self.y = y
        self.z = z
