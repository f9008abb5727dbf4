"""GB300-native backend for pdspy's thermal Monte Carlo and ray-traced images.

Entry points mirror pdspy's Model API: ``modeling.Model.run_thermal(code="gb300")``,
``run_scattering``, ``run_image`` and ``run_sed``; visibilities (``vis``: direct sum and
galario-style gridded sampling), chi^2 gradients (``adjoint``), device density builders
(``builders``) and the batched MCMC log-probability (``fitting``) build on them.  The
device work runs in the CUDA library built in-tree (``pdspy_gb300/_build/libpdgpu.so``)
behind the C ABI of ``include/pdgpu.h``.
"""
from . import constants
from .dust import Dust

__all__ = ["constants", "Dust"]
