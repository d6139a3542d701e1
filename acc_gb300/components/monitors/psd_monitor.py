"""PSD_monitor: x-y histogram at z=0 (acc/components/monitors/psd_monitor.py)."""

import numpy as np

from ... import _native as nat
from ..ComponentBase import set_param
from .MonitorBase import MonitorBase, centers

category = 'monitors'


class PSD_monitor(MonitorBase):
    opcode = nat.OP_PSD_MONITOR

    def __init__(self, name, xmin=0., xmax=0., ymin=0., ymax=0., xwidth=0.,
                 yheight=0., nx=100, ny=100, filename="psd.h5", **kwargs):
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
        self.x_centers = centers(xmin, xmax, nx)
        self.y_centers = centers(ymin, ymax, ny)
        self.hist_shape = (int(nx), int(ny))
        self.propagate_params = (np.array([xmin, xmax, ymin, ymax]), int(nx),
                                 int(ny))

    def pack(self, c, binder):
        limits, nx, ny = self.propagate_params
        c.opcode = self.opcode
        c.ip[0], c.ip[1] = nx, ny
        for k, v in enumerate(limits):
            set_param(c, k, v)
        self.pack_tally(c, binder)

    def histogram_name(self):
        return 'Iyx'

    def axes(self):
        return [('x', self.x_centers, 'm'), ('y', self.y_centers, 'm')]
