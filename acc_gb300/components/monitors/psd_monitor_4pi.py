"""PSD_monitor_4Pi: phi x theta on a sphere
(acc/components/monitors/psd_monitor_4pi.py)."""

import math

import numpy as np

from ... import _native as nat
from ..ComponentBase import set_param
from .MonitorBase import MonitorBase

category = 'monitors'


class PSD_monitor_4Pi(MonitorBase):
    opcode = nat.OP_PSD_MONITOR_4PI

    def __init__(self, name, radius=1., nphi=90, ntheta=90,
                 filename="psd_monitor_4pi.h5", **kwargs):
        self.name = name
        self.radius = float(radius)
        self.filename = filename
        thetamin, thetamax = -math.pi / 2, math.pi / 2
        phimin, phimax = -math.pi, math.pi
        dphi = (phimax - phimin) / nphi
        self.phi_centers = np.arange(phimin + dphi / 2, phimax, dphi)[:nphi]
        dtheta = (thetamax - thetamin) / ntheta
        self.theta_centers = np.arange(-thetamax + dtheta / 2, thetamax,
                                       dtheta)[:ntheta]
        self.hist_shape = (int(nphi), int(ntheta))
        self.propagate_params = (
            np.array([phimin, phimax, thetamin, thetamax]), self.radius,
            int(nphi), int(ntheta))

    def pack(self, c, binder):
        c.opcode = self.opcode
        c.ip[0], c.ip[1] = self.hist_shape
        set_param(c, 0, self.radius)
        self.pack_tally(c, binder)

    def histogram_name(self):
        return 'I_thetaphi'

    def axes(self):
        return [('phi', self.phi_centers, 'radian'),
                ('theta', self.theta_centers, 'radian')]
