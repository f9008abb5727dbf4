"""Host-side mirror of pdspy.modeling for the GB300 backend.

The classes keep pdspy's names, arguments and array conventions (pdspy/modeling/Model.py,
Grid.py, YSOModel.py, Star.py, Disk.py, UlrichEnvelopeExtended.py) so that scripts written
against pdspy's Model API run unchanged; ``run_thermal``/``run_scattering``/``run_image``/
``run_sed`` dispatch ``code="gb300"`` to the CUDA backend.
"""
from .Grid import Grid
from .Star import Star
from .Disk import Disk
from .UlrichEnvelopeExtended import UlrichEnvelopeExtended
from .Model import Model
from .YSOModel import YSOModel
