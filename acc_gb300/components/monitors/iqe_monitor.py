"""IQE_monitor: I(Q, E) of scattered neutrons at the sample position, with
angular acceptance (acc/components/monitors/iqe_monitor.py:14-174)."""

import numpy as np

from ... import _native as nat
from ...conversion import e2v
from ..ComponentBase import set_param
from .MonitorBase import MonitorBase, centers

category = 'monitors'


class IQE_monitor(MonitorBase):
    opcode = nat.OP_IQE_MONITOR

    def __init__(self, name, Ei=60., Qmin=0., Qmax=10., nQ=100, Emin=-45.,
                 Emax=45., nE=90, max_angle_in_plane=120,
                 min_angle_in_plane=0, max_angle_out_of_plane=30,
                 min_angle_out_of_plane=-30, filename="iqe.h5", **kwargs):
        self.name = name
        self.filename = filename
        self.Ei = Ei
        self.nQ, self.Qmin, self.Qmax = int(nQ), Qmin, Qmax
        self.nE, self.Emin, self.Emax = int(nE), Emin, Emax
        self.Q_centers = centers(Qmin, Qmax, self.nQ)
        self.E_centers = centers(Emin, Emax, self.nE)
        self.hist_shape = (self.nQ, self.nE)
        self.propagate_params = (
            np.array([Ei, Qmin, Qmax, Emin, Emax, max_angle_in_plane,
                      min_angle_in_plane, max_angle_out_of_plane,
                      min_angle_out_of_plane]), self.nQ, self.nE)

    def copy(self):
        p, nQ, nE = self.propagate_params
        return self.__class__(
            self.name, Ei=p[0], Qmin=p[1], Qmax=p[2], nQ=nQ, Emin=p[3],
            Emax=p[4], nE=nE, max_angle_in_plane=p[5], min_angle_in_plane=p[6],
            max_angle_out_of_plane=p[7], min_angle_out_of_plane=p[8],
            filename=self.filename)

    def pack(self, c, binder):
        p, nQ, nE = self.propagate_params
        c.opcode = self.opcode
        c.ip[0], c.ip[1] = nQ, nE
        for k, v in enumerate(p):
            set_param(c, k, v)
        self.pack_tally(c, binder)

    def axes(self):
        return [('Q', self.Q_centers, '1./angstrom'),
                ('E', self.E_centers, 'meV')]

    def histogram_name(self):
        return 'IQE'

    def _getHistogram(self, scale_factor=1.):
        return MonitorBase.getHistogram(self, scale_factor)

    def getHistogram(self, scale_factor=1., normalization_count=None):
        """I(Q,E) divided by the Monte-Carlo solid-angle normaliser of
        getNormalization (iqe_monitor.py:115-174)."""
        h = self._getHistogram(scale_factor)
        n = getNormalization(self, N=normalization_count, epsilon=1e-7)
        return h / n


def makeNeutrons(Ei, Emin, Emax, N, rng=None):
    """4pi neutrons with a uniform energy transfer (iqe_monitor.py:146-174)."""
    rng = rng or np.random.default_rng(0)
    E = Emin + rng.random(N) * (Emax - Emin)
    Ef = Ei - E
    vi = e2v(Ei)
    vf = np.sqrt(np.clip(Ef, 0, None)) * (e2v(1.0))
    cos_t = rng.random(N) * 2 - 1
    sin_t = np.sin(np.arccos(cos_t))
    phi = rng.random(N) * 2 * np.pi
    n = np.zeros((N, 10))
    n[:, 3] = vf * sin_t * np.cos(phi)
    n[:, 4] = vf * sin_t * np.sin(phi)
    n[:, 5] = vf * cos_t
    n[:, 9] = vf / vi
    return n


def getNormalization(monitor, N=None, epsilon=1e-7):
    if N is None:
        N = monitor.nQ * monitor.nE * 10000
    mcopy = monitor.copy()
    rng = np.random.default_rng(0)
    done, chunk = 0, int(2e7)
    while done < N:
        n = min(N - done, chunk)
        mcopy.process(makeNeutrons(monitor.Ei, monitor.Emin, monitor.Emax, n,
                                   rng))
        done += n
    h = mcopy._getHistogram(1.)
    h.data[h.data < epsilon] = 1
    return h
