"""Dust opacity object; mirrors pdspy/dust/Dust.py:181-188 (set_properties).

``lam`` is in cm, ``kabs``/``ksca`` in cm^2/g.  An optional ``g`` array (Henyey-Greenstein
asymmetry) is used by the GPU transport; pdspy never passes g to RADMC-3D (its dustkappa
files are iformat 2, pdspy/radmc3d/write.py:316-342), which corresponds to g = 0.
"""
from .constants import c


class Dust:
    def set_properties(self, lam, kabs, ksca, g=None):
        self.lam = lam
        self.nu = c / self.lam
        self.kabs = kabs
        self.ksca = ksca
        self.kext = self.kabs + self.ksca
        self.albedo = self.ksca / self.kext
        if g is not None:
            self.g = g
