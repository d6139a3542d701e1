"""Energy_monitor: the wavelength monitor binned in E = v^2 VS2E (meV).
No reference counterpart; modelled on
acc/components/monitors/wavelength_monitor.py:52-74."""

import numpy as np

from ... import _native as nat
from ..ComponentBase import set_param
from .MonitorBase import MonitorBase, centers

category = 'monitors'


class Energy_monitor(MonitorBase):
    opcode = nat.OP_ENERGY_MONITOR

    def __init__(self, name, xmin=0., xmax=0., ymin=0., ymax=0., xwidth=0.,
                 yheight=0., Emin=0., Emax=100., nchan=200, filename="IE.h5",
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
        assert Emin < Emax
        self.E_centers = centers(Emin, Emax, nchan)
        self.hist_shape = (int(nchan),)
        self.propagate_params = (np.array([xmin, xmax, ymin, ymax, Emin, Emax]),
                                 int(nchan))

    def pack(self, c, binder):
        limits, nchan = self.propagate_params
        c.opcode = self.opcode
        c.ip[0] = nchan
        for k, v in enumerate(limits):
            set_param(c, k, v)
        self.pack_tally(c, binder)

    def histogram_name(self):
        return 'I(energy)'

    def axes(self):
        return [('energy', self.E_centers, 'meV')]
