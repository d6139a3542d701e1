"""PosDiv_monitor: x versus horizontal divergence
(acc/components/monitors/posdiv_monitor.py)."""

import numpy as np

from ... import _native as nat
from ..ComponentBase import set_param
from .MonitorBase import MonitorBase

category = 'monitors'


class PosDiv_monitor(MonitorBase):
    opcode = nat.OP_POSDIV_MONITOR

    def __init__(self, name, xmin=0., xmax=0., ymin=0., ymax=0., xwidth=0.,
                 yheight=0., maxdiv=2., npos=20, ndiv=20,
                 filename="posdiv.h5", **kwargs):
        self.name = name
        self.filename = filename
        if xwidth > 0:
            xmax = xwidth / 2
            xmin = -xmax
        if yheight > 0:
            ymax = yheight / 2
            ymin = -ymax
        assert xmin < xmax
        assert ymin < ymax
        npos, ndiv = int(npos), int(ndiv)
        dx = (xmax - xmin) / npos
        self.x_centers = np.arange(xmin + dx / 2, xmax, dx)[:npos]
        ddiv = 2 * maxdiv / ndiv
        self.div_centers = np.arange(-maxdiv + ddiv / 2, maxdiv, ddiv)[:ndiv]
        self.hist_shape = (npos, ndiv)
        self.propagate_params = (np.array([xmin, xmax, ymin, ymax, maxdiv]),
                                 npos, ndiv)

    def pack(self, c, binder):
        limits, npos, ndiv = self.propagate_params
        c.opcode = self.opcode
        c.ip[0], c.ip[1] = npos, ndiv
        for k, v in enumerate(limits):
            set_param(c, k, v)
        self.pack_tally(c, binder)

    def histogram_name(self):
        return 'Idiv_x'

    def axes(self):
        return [('x', self.x_centers, 'm'), ('div', self.div_centers, 'deg')]
