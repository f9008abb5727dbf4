"""Generic model; mirrors pdspy/modeling/Model.py with a "gb300" code path.

``run_thermal``, ``run_scattering``, ``run_image``, ``run_sed`` and ``run_visibilities``
keep the reference's signatures and string dispatch on ``code`` (Model.py:69-72,
:275-278, :345-348, :600-603, :672-675).  ``code="gb300"`` (the
default here) runs the CUDA backend; "radmc3d" and "hyperion" name external programs
that are not part of this package and raise NotImplementedError.
"""
from .Grid import Grid


class Model:
    def __init__(self):
        self.grid = Grid()
        self.images = {}
        self.spectra = {}
        self.visibilities = {}

    def set_camera_wavelength(self, lam):
        self.camera_wavelength = lam

    def run_thermal(self, nphot=1e6, code="gb300", **keywords):
        if code == "gb300":
            from ..thermal import run_thermal
            return run_thermal(self, nphot=nphot, **keywords)
        raise NotImplementedError("code=%r is an external program; use code='gb300'" % code)

    def run_scattering(self, nphot=1e6, code="gb300", **keywords):
        if code == "gb300":
            from ..scatter import run_scattering
            return run_scattering(self, nphot=nphot, **keywords)
        raise NotImplementedError("code=%r is an external program; use code='gb300'" % code)

    def run_image(self, name=None, nphot=1e6, code="gb300", **keywords):
        if code == "gb300":
            from ..image import run_image
            return run_image(self, name=name, nphot=nphot, **keywords)
        raise NotImplementedError("code=%r is an external program; use code='gb300'" % code)

    def run_sed(self, name=None, nphot=1e6, code="gb300", **keywords):
        if code == "gb300":
            from ..image import run_sed
            return run_sed(self, name=name, nphot=nphot, **keywords)
        raise NotImplementedError("code=%r is an external program; use code='gb300'" % code)

    def run_visibilities(self, name=None, nphot=1e6, code="gb300", **keywords):
        if code == "gb300":
            from ..image import run_visibilities
            return run_visibilities(self, name=name, nphot=nphot, **keywords)
        raise NotImplementedError("code=%r is an external program; use code='gb300'" % code)
