"""Scattering kernels of homogeneous scatterers (acc/kernels)."""

from .kernels import (ConstantQEKernel, E_Q_Kernel,  # noqa: F401
                      IsotropicKernel, Peak, PowderDiffraction,
                      SimplePowderDiffractionKernel, SQEGridKernel,
                      coefficient_from_cross_section)
from .expression import compile_expression  # noqa: F401
