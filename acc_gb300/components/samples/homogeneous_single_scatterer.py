"""Homogeneous single scatterer: a shape filled with one scattering kernel
(acc/components/samples/homogeneous_single_scatterer.py:26-102).

    HSSbase = factory(shape=Sphere(0.01), kernel=IsotropicKernel(mu, sigma))
    class HSS(HSSbase): pass
    sample = HSS('sample')
"""

from ... import _native as nat
from ...geometry.shapes import pack_shape
from ..ComponentBase import set_param
from .SampleBase import SampleBase

category = 'samples'


def factory(shape, kernel):
    """A component class scattering with `kernel` inside `shape`."""

    class HomogeneousSingleScatterer(SampleBase):
        opcode = nat.OP_HSS

        def __init__(self, name):
            self.name = name
            self.shape = shape
            self.kernel = kernel
            self.propagate_params = ()

        def pack(self, c, binder):
            c.opcode = self.opcode
            pack_shape(self.shape, c, set_param)
            c.ip[1] = self.kernel.kind
            self.kernel.pack(self, c, binder, set_param)

    return HomogeneousSingleScatterer
