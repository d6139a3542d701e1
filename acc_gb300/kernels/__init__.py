"""Scattering kernels of homogeneous scatterers (acc/kernels)."""

from .kernels import (CompositeKernel, ConstantQEKernel,  # noqa: F401
                      DGSSXResKernel, E_Q_Kernel,
                      IsotropicKernel, Peak, PowderDiffraction,
                      SANS2D_ongrid_Kernel, SimplePowderDiffractionKernel,
                      SQEGridKernel,
                      coefficient_from_cross_section)
from .expression import compile_expression  # noqa: F401
