"""IsotropicBox (acc/components/samples/isotropic_box.py:17-98): a box of
xwidth x yheight x zthickness scattering isotropically, mu the absorption
coefficient at 2200 m/s and sigma the scattering coefficient (1/m).  Its
propagate is the homogeneous single scatterer's on a box with the isotropic
kernel: the same draws (one for the depth, two for the direction), the
weight sigma * L * exp(-(mu 2200/v + sigma) d) and the exit attenuation;
the reference moves to the box's surface and then to the scattering point
in two steps, here in one (the same point up to rounding)."""

from ...geometry import Block
from ...kernels import IsotropicKernel
from .homogeneous_single_scatterer import factory

category = 'samples'


def IsotropicBox(name, xwidth, yheight, zthickness, mu, sigma):
    """The box sample (an HSS component instance)."""
    cls = factory(Block(xwidth, yheight, zthickness),
                  IsotropicKernel(mu, sigma))
    return cls(name)
