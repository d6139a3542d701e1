"""SNS moderator source (acc/components/sources/SNS_source.py:20-207): the
energy and emission time of each neutron are drawn from a moderator file's
tabulated spectrum and pulse shapes.

The host set-up restates acc/components/sources/_SNS_source_utils.py:
the file's two sections are read, the cumulative probabilities P(E) and,
for every energy, P(t) are integrated from quadratic interpolants
(scipy.integrate.quad), and the GPU draws E and t by inverting them
(mcv_component layout: include/acc_gb300.h, SNS_SOURCE).
"""

import math
import warnings

import numpy as np

from ... import _native as nat
from ..ComponentBase import set_param
from .SourceBase import SourceBase

category = 'sources'


def sns_source_load(filename, xcol=0, ycol=2):
    """The moderator file (_SNS_source_utils.py:12-57): section 1, one row
    per energy (eV) with the spectrum in column `ycol`, ends at the first
    blank line; section 2 holds one block per energy of rows (t in us, E,
    brightness, error), blocks separated by blank lines, '#' lines are
    comments.  Returns (E, I(E), veclen, t, I[E][t])."""
    with open(filename, "rt") as stream:
        first_block = []
        while True:
            line = stream.readline()
            if line.startswith("#"):
                continue
            if len(line.strip()) != 0:
                first_block.append(list(map(float, line.split())))
            else:
                break
        first_block = np.array(first_block)
        xvec = first_block[:, xcol]
        yvec = first_block[:, ycol]
        idx1 = first_block.shape[0]
        idx2 = idx1 // 2
        while idx2 < idx1 and yvec[idx2] > 0:
            idx2 += 1
        veclen = idx2 if idx2 < idx1 else idx1 - 2
        while True:
            line = stream.readline()
            if not (line.startswith("#") or len(line.strip()) == 0):
                break
        mat = []
        while len(line):
            block = []
            while len(line.strip()) != 0:
                block.append([float(t) for t in line.split()])
                line = stream.readline()
            mat.append(block)
            while len(line) and len(line.strip()) == 0:
                line = stream.readline()
        mat = np.array(mat)
    nE, nt, _ = mat.shape
    if nE != len(xvec):
        raise RuntimeError(f"{filename}: {nE} pulse shapes for {len(xvec)} "
                           "energies")
    for i in range(nt):
        if not np.allclose(mat[:, i, 1], xvec):
            raise RuntimeError(f"{filename}: energies of section 2 differ")
    tvec = mat[0, :, 0]
    for i in range(nE):
        if not np.allclose(mat[i, :, 0], tvec):
            raise RuntimeError(f"{filename}: times of section 2 differ")
    return (np.ascontiguousarray(xvec), np.ascontiguousarray(yvec), veclen,
            np.ascontiguousarray(tvec), np.ascontiguousarray(mat[:, :, 2]))


def Pcalc(func, llim, hlim, xvec, Prob, veclen):
    """Cumulative probability of I(x) on the points of xvec between llim
    and hlim, normalised to 1 (_SNS_source_utils.py:129-177); 0 below,
    1 above.  Returns the index range (start, stop) it filled."""
    import scipy.integrate as si
    idx1 = 0
    while xvec[idx1] <= llim:
        Prob[idx1] = 0
        idx1 += 1
    if idx1 < 1:
        raise RuntimeError("Error: lower energy limit is out of bounds\n")
    idxstart = idx1
    Prob[idx1], _ = si.quad(func, llim, xvec[idx1])
    idx1 += 1
    while xvec[idx1] <= hlim:
        part, _ = si.quad(func, xvec[idx1 - 1], xvec[idx1])
        Prob[idx1] = Prob[idx1 - 1] + part
        idx1 += 1
    idxstop = idx1
    while idx1 < veclen:
        Prob[idx1] = 1
        idx1 += 1
    norm = Prob[idxstop - 1]
    if norm > 0:
        for i in range(idxstart, idxstop):
            Prob[i] /= norm
    return idxstart, idxstop


def init(Emin, Emax, datafile):
    """_SNS_source_utils.init (:187-223): Emin, Emax in meV.  Returns
    (INorm2, Es, Pvec, ts, Ptmat, EPmin, EPmax, (Eidx_start, Eidx_stop),
    (tidx_start, tidx_stop))."""
    import scipy.integrate as si
    import scipy.interpolate as sinterp
    inxvec, inyvec, xylength, tvec, mat = sns_source_load(datafile, 0, 2)
    nE, nt = mat.shape
    llim, hlim = inxvec[1], inxvec[xylength]
    I_E = sinterp.interp1d(inxvec, inyvec, kind="quadratic")
    INorm2, _ = si.quad(I_E, Emin / 1000.0, Emax / 1000.0)
    Pvec = np.zeros(nE)
    idxstart, idxstop = Pcalc(I_E, llim, hlim, inxvec, Pvec, xylength)
    Ptmat = np.zeros((nE, nt))
    ltlim, htlim = 0.1, 1.8e3
    for iE in range(nE):
        I_t = sinterp.interp1d(tvec, mat[iE], kind="quadratic")
        tidxstart, tidxstop = Pcalc(I_t, ltlim, htlim, tvec, Ptmat[iE], nt)
    f = sinterp.interp1d(inxvec, Pvec, kind="quadratic")
    EPmax = float(f(Emax / 1000.0))
    EPmin = float(f(Emin / 1000.0))
    return (INorm2, inxvec, Pvec, tvec, Ptmat, EPmin, EPmax,
            (idxstart, idxstop), (tidxstart, tidxstop))


class SNS_source(SourceBase):
    opcode = nat.OP_SNS_SOURCE

    def __init__(self, name, filename, Emin, Emax, xwidth, yheight, dist,
                 focus_xw, focus_yh, Anorm=0.01, radius=-1.0):
        """Moderator face xwidth x yheight (or a disc of `radius` when
        either is <= 0) aimed at a focus_xw x focus_yh window `dist` m
        away; energies in [Emin, Emax] meV from `filename`."""
        self.name = name
        self.Emin, self.Emax = Emin, Emax
        (self.INorm2, Es, Pvec, ts, Ptmat, EPmin, EPmax, Eidx_range,
         tidx_range) = init(Emin, Emax, filename)
        if xwidth <= 0 or yheight <= 0:
            warnings.warn("Either xwidth or yheight is invalid. will assume "
                          "a circle")
            self.square = False
            if not radius > 0:
                raise ValueError(f"radius is invalid: {radius}")
            srcArea = math.pi * radius * radius
        else:
            self.square = True
            srcArea = xwidth * yheight
        self.p_in = focus_xw * focus_yh / dist / dist * srcArea / Anorm
        self._prob = self.p_in * self.INorm2
        self.xwidth, self.yheight, self.radius = xwidth, yheight, radius
        self.dist, self.focus_xw, self.focus_yh = dist, focus_xw, focus_yh
        self.Anorm = Anorm
        self.tables = (Es, Pvec, ts, Ptmat)
        self.propagate_params = (
            self.square, xwidth, yheight, radius, focus_xw, focus_yh, dist,
            EPmin, EPmax, Es, Eidx_range[0], Eidx_range[1], Pvec, ts,
            tidx_range[0], tidx_range[1], Ptmat, self._prob)

    def nominal_weight(self):
        """Every neutron carries the same weight (propagate, :205-206)."""
        return self._prob

    def pack(self, c, binder):
        (square, xwidth, yheight, radius, focus_xw, focus_yh, dist, EPmin,
         EPmax, Es, Eidx_start, Eidx_stop, Pvec, ts, tidx_start, tidx_stop,
         Ptmat, prob) = self.propagate_params
        c.opcode = self.opcode
        c.ip[0] = int(bool(square))
        c.ip[1], c.ip[2] = len(Es), len(ts)
        c.ip[3], c.ip[4] = int(Eidx_start), int(Eidx_stop)
        c.ip[5], c.ip[6] = int(tidx_start), int(tidx_stop)
        for k, v in enumerate((xwidth, yheight, radius, focus_xw, focus_yh,
                               dist, EPmin, EPmax, prob)):
            set_param(c, k, v)
        flat = np.concatenate([Es, Pvec, ts, np.asarray(Ptmat).reshape(-1)])
        c.table = binder.table(self, "moderator", flat, np.float64)
        c.table_len = flat.size
