"""Source_simple (acc/components/sources/source_simple.py:44-162)."""

import math

from ... import _native as nat
from ..ComponentBase import set_param
from .SourceBase import SourceBase

category = 'sources'


class Source_simple(SourceBase):
    opcode = nat.OP_SOURCE_SIMPLE

    def __init__(self, name, radius=0.05, height=0, width=0, dist=10.0,
                 xw=0.1, yh=0.1, E0=60, dE=10, Lambda0=0, dLambda=0, flux=1,
                 gauss=0, N=1, **kwargs):
        """Disc (radius) or rectangle (width x height) source at z=0 aimed at
        an xw x yh target a distance `dist` down the z axis, with a flat
        energy (E0 +- dE, meV) or wavelength (Lambda0 +- dLambda, A)
        distribution.  `gauss` is accepted and ignored, as in the reference
        (source_simple.py:52,153-158)."""
        self.name = name
        if radius != 0 and height == 0 and width == 0:
            square = False
            srcArea = math.pi * radius * radius
        elif radius == 0 and height != 0 and width != 0:
            square = True
            srcArea = width * height
        else:
            raise RuntimeError(
                f"Source_simple: confused! Both radius ({radius}) and "
                f"width({width})/height({height}) are specified")
        pmul = flux * 1e4 * srcArea / N
        if srcArea <= 0 or dist < 0 or xw < 0 or yh < 0:
            raise RuntimeError("bad source geometry")
        if Lambda0 == 0 and dLambda == 0 and (E0 <= 0 or dE < 0 or E0 - dE <= 0):
            raise RuntimeError("bad energy distribution spec")
        if E0 == 0 and dE == 0 and (Lambda0 <= 0 or dLambda < 0
                                    or Lambda0 - dLambda <= 0):
            raise RuntimeError("bad wavelength distribution spec")
        wl_distr = Lambda0 != 0
        self.propagate_params = (
            square, width, height, radius,
            wl_distr, Lambda0, dLambda, E0, dE,
            xw, yh, dist, pmul,
        )

    def nominal_weight(self):
        """The weight of a neutron aimed at the target's centre:
        pmul * xw * yh / dist^2 (propagate, source_simple.py:143-161)."""
        xw, yh, dist, pmul = self.propagate_params[9:13]
        if dist <= 0 or xw <= 0 or yh <= 0:
            return None
        return pmul * xw * yh / (dist * dist)

    def pack(self, c, binder):
        (square, width, height, radius, wl_distr, Lambda0, dLambda, E0, dE,
         xw, yh, dist, pmul) = self.propagate_params
        c.opcode = self.opcode
        c.ip[0] = int(bool(square))
        c.ip[1] = int(bool(wl_distr))
        for k, v in enumerate((width, height, radius, Lambda0, dLambda, E0,
                               dE, xw, yh, dist, pmul)):
            set_param(c, k, v)
