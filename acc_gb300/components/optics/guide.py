"""Guide: straight or linearly tapered four-mirror guide
(acc/components/optics/guide.py:21-162)."""

from ... import _native as nat
from ..ComponentBase import ComponentBase, set_param

category = 'optics'
max_bounces = nat.MCV_MAX_BOUNCES


class Guide(ComponentBase):
    opcode = nat.OP_GUIDE

    def __init__(self, name, w1, h1, w2, h2, l, R0=0.99, Qc=0.0219,
                 alpha=6.07, m=2, W=0.003, **kwargs):
        """Guide centred on the z axis with its entrance at z=0: entry
        w1 x h1, exit w2 x h2, length l (m); supermirror R0, Qc (1/A),
        alpha (A), m, W (1/A)."""
        self.name = name
        ww = .5 * (w2 - w1)
        hh = .5 * (h2 - h1)
        hw1 = 0.5 * w1
        hh1 = 0.5 * h1
        self.propagate_params = (
            float(ww), float(hh), float(hw1), float(hh1), float(l),
            float(R0), float(Qc), float(alpha), float(m), float(W),
        )

    def pack(self, c, binder):
        c.opcode = self.opcode
        for k, v in enumerate(self.propagate_params):
            set_param(c, k, v)
