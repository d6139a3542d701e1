"""Scattering kernels of homogeneous scatterers (acc/kernels)."""

from .kernels import (IsotropicKernel, Peak, PowderDiffraction,  # noqa: F401
                      SimplePowderDiffractionKernel, SQEGridKernel,
                      coefficient_from_cross_section)
