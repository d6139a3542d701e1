"""Homogeneous multiple scatterer: a shape filled with one scattering
kernel, with multiple scattering inside it
(acc/components/samples/homogeneous_multiple_scatterer.py:22-342).

    HMSbase = factory(shape=HollowCylinder(0.01, 0.02, 0.06), kernel=...,
                      max_ms_loops=2, max_ms_loops_path1=5,
                      max_scattered_neutrons=16)
    class HMS(HMSbase): pass
    sample = HMS('sample')

Each incident neutron leaves as up to max_scattered_neutrons output
neutrons; the components after the sample run on each of them.
"""

from ... import _native as nat
from ...geometry.shapes import pack_shape
from ..ComponentBase import set_param
from .SampleBase import SampleBase

category = 'samples'


def factory(shape, kernel, max_scattered_neutrons=10, max_ms_loops=3,
            max_ms_loops_path1=2, minimum_neutron_event_probability=1e-20):
    """A component class scattering with `kernel` inside `shape`, with up to
    max_ms_loops loops among re-entries and max_ms_loops_path1 loops on the
    first passage (homogeneous_multiple_scatterer.py:22-45)."""
    # as asserted by the reference (:46): the worst case must fit
    assert max_scattered_neutrons > max_ms_loops * (max_ms_loops_path1 + 1)
    if not 1 <= max_scattered_neutrons <= nat.MCV_MS_MAX_SCATTERED:
        raise ValueError(
            f"max_scattered_neutrons must be 1..{nat.MCV_MS_MAX_SCATTERED}")

    class HomogeneousMultipleScatterer(SampleBase):
        opcode = nat.OP_HMS
        is_multiplescattering = True
        NUM_MULTIPLE_SCATTER = max_scattered_neutrons

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
            c.ip[6] = int(max_scattered_neutrons)
            c.ip[7] = int(max_ms_loops) | (int(max_ms_loops_path1) << 16)
            set_param(c, 14, float(minimum_neutron_event_probability))

    HomogeneousMultipleScatterer.max_scattered_neutrons = \
        max_scattered_neutrons
    HomogeneousMultipleScatterer.max_ms_loops = max_ms_loops
    HomogeneousMultipleScatterer.max_ms_loops_path1 = max_ms_loops_path1
    HomogeneousMultipleScatterer.minimum_neutron_event_probability = \
        minimum_neutron_event_probability
    return HomogeneousMultipleScatterer
