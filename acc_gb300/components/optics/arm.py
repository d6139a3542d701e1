"""Arm: a placeholder component that leaves the neutron unchanged
(acc/components/optics/arm.py:14-43)."""

from ... import _native as nat
from ..ComponentBase import ComponentBase

category = 'optics'


class Arm(ComponentBase):
    opcode = nat.OP_ARM

    def __init__(self, name, **kwargs):
        self.name = name
        self.propagate_params = ()
