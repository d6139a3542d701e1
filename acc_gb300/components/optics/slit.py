"""Slit: absorb neutrons that miss a rectangular or round opening at z=0
(acc/components/optics/slit.py:17-108)."""

from ... import _native as nat
from ..ComponentBase import ComponentBase, set_param

category = 'optics'


class Slit(ComponentBase):
    opcode = nat.OP_SLIT

    def __init__(self, name, xmin=0, xmax=0, ymin=0, ymax=0, radius=0, cut=0,
                 width=0, height=0, **kwargs):
        """Opening at z=0: xmin..xmax x ymin..ymax (or width x height
        centred), or a disc of `radius`; weights below `cut` are absorbed."""
        self.name = name
        if width > 0:
            xmax = width / 2
            xmin = -xmax
        if height > 0:
            ymax = height / 2
            ymin = -ymax
        if not (xmin or xmax or ymin or ymax or radius):
            raise ValueError(f"a {self._kind} must have some extent")
        self.propagate_params = (
            (float(xmin), float(xmax), float(ymin), float(ymax),
             float(radius) * float(radius), float(cut)),)

    _kind = "slit"

    def pack(self, c, binder):
        c.opcode = self.opcode
        for k, v in enumerate(self.propagate_params[0]):
            set_param(c, k, v)
