"""Detectors on a vertical cylinder (axis y) centred on the sample.  No
reference counterpart.

CylinderIQE_detector bins I(Q, E) where the neutron crosses the cylinder,
with Q and E computed as IQE_monitor does (iqe_monitor.py:96-110).
BankedCylinder_detector splits the cylinder into azimuthal banks of tubes
(pixels along the height) and bins time of flight per pixel.
"""

import math

import numpy as np

from ... import _native as nat
from ..ComponentBase import set_param
from .MonitorBase import MonitorBase, centers

category = 'monitors'


class CylinderIQE_detector(MonitorBase):
    opcode = nat.OP_CYL_IQE_DETECTOR

    def __init__(self, name, radius=3., height=2., Ei=60., Qmin=0., Qmax=10.,
                 nQ=100, Emin=-50., Emax=55., nE=100, filename="cyl_iqe.h5",
                 **kwargs):
        self.name = name
        self.filename = filename
        self.Ei = Ei
        self.Q_centers = centers(Qmin, Qmax, int(nQ))
        self.E_centers = centers(Emin, Emax, int(nE))
        self.hist_shape = (int(nQ), int(nE))
        self.propagate_params = (float(radius), float(height), float(Ei),
                                 float(Qmin), float(Qmax), float(Emin),
                                 float(Emax))

    def pack(self, c, binder):
        c.opcode = self.opcode
        c.ip[0], c.ip[1] = self.hist_shape
        for k, v in enumerate(self.propagate_params):
            set_param(c, k, v)
        self.pack_tally(c, binder)

    def histogram_name(self):
        return 'IQE'

    def axes(self):
        return [('Q', self.Q_centers, '1./angstrom'),
                ('E', self.E_centers, 'meV')]


class BankedCylinder_detector(MonitorBase):
    """Banks are azimuthal windows of phi = atan2(x, z):
    [a0 + b (w + g), a0 + b (w + g) + w), b = 0..nbanks-1."""
    opcode = nat.OP_BANKED_DETECTOR

    def __init__(self, name, radius=3., height=1., nbanks=8, ntubes=128,
                 npixels=256, bank_angle0=10., bank_width=15., bank_gap=5.,
                 tofmin=0., tofmax=0.02, ntof=1000, filename="banked.h5",
                 **kwargs):
        self.name = name
        self.filename = filename
        self.shape4 = (int(nbanks), int(ntubes), int(npixels), int(ntof))
        self.hist_shape = (int(nbanks) * int(ntubes) * int(npixels), int(ntof))
        self.tof_centers = centers(tofmin, tofmax, int(ntof))
        self.propagate_params = (
            float(radius), float(height), math.radians(bank_angle0),
            math.radians(bank_width), math.radians(bank_gap), float(tofmin),
            float(tofmax))

    def pack(self, c, binder):
        c.opcode = self.opcode
        for k, v in enumerate(self.shape4):
            c.ip[k] = v
        for k, v in enumerate(self.propagate_params):
            set_param(c, k, v)
        self.pack_tally(c, binder)

    def histogram_name(self):
        return 'I_pixel_tof'

    def axes(self):
        return [('pixel', np.arange(self.hist_shape[0]), ''),
                ('tof', self.tof_centers, 's')]
