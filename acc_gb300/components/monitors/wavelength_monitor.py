"""Wavelength_monitor (acc/components/monitors/wavelength_monitor.py)."""

import numpy as np

from ... import _native as nat
from ..ComponentBase import set_param
from .MonitorBase import MonitorBase, centers

category = 'monitors'


class Wavelength_monitor(MonitorBase):
    opcode = nat.OP_WAVELENGTH_MONITOR

    def __init__(self, name, xmin=0., xmax=0., ymin=0., ymax=0., xwidth=0.,
                 yheight=0., Lmin=0., Lmax=10., nchan=200, filename="IL.h5",
                 **kwargs):
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
        self.L_centers = centers(Lmin, Lmax, nchan)
        self.hist_shape = (int(nchan),)
        self.propagate_params = (np.array([xmin, xmax, ymin, ymax, Lmin, Lmax]),
                                 int(nchan))

    def pack(self, c, binder):
        limits, nchan = self.propagate_params
        c.opcode = self.opcode
        c.ip[0] = nchan
        for k, v in enumerate(limits):
            set_param(c, k, v)
        self.pack_tally(c, binder)

    def histogram_name(self):
        return 'I(wavelength)'

    def axes(self):
        return [('wavelength', self.L_centers, 'angstrom')]
