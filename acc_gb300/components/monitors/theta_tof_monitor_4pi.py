"""ThetaTOF_monitor_4Pi: a spherical shell around the sample binned by the
polar angle from +z (0..180 deg) and time of flight.  No reference
counterpart; the sphere crossing of
acc/components/monitors/psd_monitor_4pi.py:56-66."""

import numpy as np

from ... import _native as nat
from ..ComponentBase import set_param
from .MonitorBase import MonitorBase, centers

category = 'monitors'


class ThetaTOF_monitor_4Pi(MonitorBase):
    opcode = nat.OP_THETA_TOF_4PI

    def __init__(self, name, radius=3., ntheta=180, ntof=200, tofmin=0.,
                 tofmax=0.01, filename="theta_tof.h5", **kwargs):
        self.name = name
        self.radius = float(radius)
        self.filename = filename
        assert tofmin < tofmax
        self.theta_centers = centers(0., 180., int(ntheta))
        self.tof_centers = centers(tofmin, tofmax, int(ntof))
        self.hist_shape = (int(ntheta), int(ntof))
        self.propagate_params = (self.radius, float(tofmin), float(tofmax),
                                 int(ntheta), int(ntof))

    def pack(self, c, binder):
        r, t0, t1, nth, nt = self.propagate_params
        c.opcode = self.opcode
        c.ip[0], c.ip[1] = nth, nt
        for k, v in enumerate((r, t0, t1)):
            set_param(c, k, v)
        self.pack_tally(c, binder)

    def histogram_name(self):
        return 'I_theta_tof'

    def axes(self):
        return [('theta', self.theta_centers, 'deg'),
                ('tof', self.tof_centers, 's')]
