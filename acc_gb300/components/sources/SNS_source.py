"""SNS moderator source (acc/components/sources/SNS_source.py:20-207): the
energy and emission time of each neutron are drawn from a moderator file's
tabulated spectrum and pulse shapes.

The host set-up restates acc/components/sources/_SNS_source_utils.py:
the file's two sections are read, the cumulative probabilities P(E) and,
for every energy, P(t) are integrated from quadratic interpolants
(scipy.integrate.quad), and the GPU draws E and t by inverting them
(mcv_component layout: include/acc_gb300.h, SNS_SOURCE).
"""

import gzip
import math
import warnings

import numpy as np

from ... import _native as nat
from ..ComponentBase import set_param
from .SourceBase import SourceBase

category = 'sources'


def sts_params_load(stream):
    """The STS file's section 0 (_SNS_source_utils.py:62-78): one number
    per line (first token) up to '## section 0 end'; the last must be the
    check value 12345678.  Returns (PPower, Freq, MRadius, MOffangle,
    PHeight, PWidth, TRadius)."""
    params = []
    while True:
        line = stream.readline()
        if not line:
            raise RuntimeError("no '## section 0 end' line")
        if line.startswith("## section 0 end"):
            break
        if line.startswith("#"):
            continue
        if len(line.strip()) != 0:
            params.append(float(line.strip().split()[0]))
    if not params or params[-1] != 12345678.0:
        raise RuntimeError("ERROR: Inconsistent parameter data set. Expected "
                           "check string 12345678, got "
                           f"{params[-1] if params else None}")
    return np.array(params[:-1])


def sns_source_load(filename, xcol=0, ycol=2, sts=False):
    """The moderator file (_SNS_source_utils.py:12-57): section 1, one row
    per energy (eV) with the spectrum in column `ycol`, ends at the first
    blank line; section 2 holds one block per energy of rows (t in us, E,
    brightness, error), blocks separated by blank lines, '#' lines are
    comments.  Returns (E, I(E), veclen, t, I[E][t]), and the STS
    parameters first when `sts` (the file then opens with section 0).  A
    name ending in .gz is read through gzip."""
    params = None
    opener = gzip.open if str(filename).endswith(".gz") else open
    with opener(filename, "rt") as stream:
        if sts:
            params = sts_params_load(stream)
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
    out = (np.ascontiguousarray(xvec), np.ascontiguousarray(yvec), veclen,
           np.ascontiguousarray(tvec), np.ascontiguousarray(mat[:, :, 2]))
    return out + (params,) if sts else out


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


def init(Emin, Emax, datafile, sts_load=False):
    """_SNS_source_utils.init (:187-223): Emin, Emax in meV.  Returns
    (INorm2, Es, Pvec, ts, Ptmat, EPmin, EPmax, (Eidx_start, Eidx_stop),
    (tidx_start, tidx_stop)), and the STS parameters last when
    `sts_load`."""
    import scipy.integrate as si
    import scipy.interpolate as sinterp
    loaded = sns_source_load(datafile, 0, 2, sts=sts_load)
    inxvec, inyvec, xylength, tvec, mat = loaded[:5]
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
    out = (INorm2, inxvec, Pvec, tvec, Ptmat, EPmin, EPmax,
           (idxstart, idxstop), (tidxstart, tidxstop))
    return out + (loaded[5],) if sts_load else out


# ------------------------------------------------- FP32 sampling tables
# The FP64 kernels invert the cumulative tables per neutron with the
# reference's zero_find (SNS_source.py:77-96).  The FP32 kernels read
# inverse tables instead, computed here once with the same zero_find:
#   E(u) at SNS_E_NODES + 1 evenly spaced u, linearly interpolated;
#   for every energy row r, t_r(u) at SNS_T_NODES + 1 evenly spaced u over
#   the row's t window, and the row's probability mass in that window.
# A neutron's t comes from the two rows that bracket its E, mixed with the
# reference's weights wl, 1 - wl: the row is picked with probability
# proportional to its weight times its mass and the uniform rescaled into
# it, which samples the mixture the reference inverts.  Draws of u outside
# [u_lo, u_hi], where zero_find's bracket leaves the table, go to the FP64
# sampler, so the reference's values there are kept.
SNS_E_NODES = nat.MCV_SNS_E_NODES
SNS_T_NODES = nat.MCV_SNS_T_NODES
ZERO_FIND_EXPAND_MAX, ZERO_FIND_BISECT_MAX = 64, 200


def _quadfuncint(xdes, vecx, rows, vecy):
    """quadfuncint (SNS_source.py:66-75) for arrays of xdes; vecy[rows]
    gives each element's table (rows None: one table).  The index is the
    first in [1, len) not below xdes, clamped to the last point; index -1
    wraps to the last point (numba's indexing)."""
    n = len(vecx)
    idx = np.searchsorted(vecx[1:], xdes, side="left") + 1
    idx = np.minimum(idx, n - 1)
    i0 = idx - 2
    i0 = np.where(i0 < 0, i0 + n, i0)
    if rows is None:
        y0, y1, y2 = vecy[i0], vecy[idx - 1], vecy[idx]
    else:
        y0, y1, y2 = vecy[rows, i0], vecy[rows, idx - 1], vecy[rows, idx]
    x1, x2, x3 = vecx[i0], vecx[idx - 1], vecx[idx]
    with np.errstate(all="ignore"):
        t1 = ((xdes - x2) * (xdes - x3) * y0) / ((x1 - x2) * (x1 - x3))
        t2 = ((xdes - x1) * (xdes - x3) * y1) / ((x2 - x1) * (x2 - x3))
        t3 = ((xdes - x1) * (xdes - x2) * y2) / ((x3 - x1) * (x3 - x2))
        val = t1 + t2 + t3
    return np.where(vecx[idx] == xdes, y2, val)


def zero_find(vecx, vecy, yval, xmin, xmax, tol, rows=None):
    """zero_find (SNS_source.py:77-96) for an array of targets yval, with
    its loops bounded as the kernels bound them (64 expansions, 200
    bisections)."""
    yval = np.asarray(yval, dtype=np.float64)
    F = lambda x, sel: _quadfuncint(  # noqa: E731
        x, vecx, None if rows is None else rows[sel], vecy) - yval[sel]
    allsel = np.arange(yval.size)
    xl = np.full(yval.shape, float(xmin))
    with np.errstate(all="ignore"):
        xh = np.power(10.0, np.log10(xmin) + yval * (np.log10(xmax)
                                                     - np.log10(xmin)))
        f = F(xl, allsel)
        fmid = F(xh, allsel)
        for _ in range(ZERO_FIND_EXPAND_MAX):
            m = np.where(fmid * f >= 0.0)[0]
            if m.size == 0:
                break
            xh[m] = xh[m] + (xh[m] - xl[m]) * 2.0
            fmid[m] = F(xh[m], m)
        dx = xh - xl
        rtb = xl.copy()
        act = np.where(np.abs(F(rtb, allsel)) > tol)[0]
        for _ in range(ZERO_FIND_BISECT_MAX):
            if act.size == 0:
                break
            dx[act] *= 0.5
            xmid = rtb[act] + dx[act]
            fm = F(xmid, act)
            up = fm < 0
            rtb[act[up]] = xmid[up]
            act = act[np.abs(F(rtb[act], act)) > tol]
    return rtb


# an FP32 kernel's uniform is k * 2^-24, k < 2^24 (PhiloxStream::next)
UNIFORM_STEPS = 1 << 24
# at most this many tail energies (float32) a source
SNS_TAIL_MAX = nat.MCV_SNS_TAIL_MAX
# largest relative error of the FP32 energy table's linear interpolation at
# an interval's midpoint; coarser end intervals take per-draw tail energies
SNS_INTERP_TOL = 2e-5


def fp32_tables(Es, Pvec, ts, Ptmat, EPmin, EPmax, Eidx, tidx):
    """(ftable float32 array, u_lo, u_hi, n_lo, n_hi): the inverse tables
    the FP32 kernels sample (layout in include/acc_gb300.h, SNS_SOURCE);
    n_lo and n_hi count the tail energies of the draws below u_lo and
    above u_hi."""
    Es = np.asarray(Es, dtype=np.float64)
    ts = np.asarray(ts, dtype=np.float64)
    Pvec = np.asarray(Pvec, dtype=np.float64)
    Ptmat = np.asarray(Ptmat, dtype=np.float64)
    nE = len(Es)
    u = np.arange(SNS_E_NODES + 1) / SNS_E_NODES
    randp = EPmin + u * (EPmax - EPmin)
    xmin, xmax = Es[Eidx[0]], Es[Eidx[1]]
    Einv = zero_find(Es, Pvec, randp, xmin, xmax, 1e-7)
    # the regular range: zero_find's bracket starts with the target above
    # the cumulative probability at xmin, and the nodes lie in [xmin, xmax]
    # and increase (the table's cumulative column drops to 0 past the
    # file's usable rows, so the top is found from the nodes themselves)
    ok = (randp > Pvec[Eidx[0]] + 1e-7) & (Einv >= xmin) & (Einv <= xmax)
    # the longest run of regular nodes, each not below the one before
    link = ok[1:] & ok[:-1] & (np.diff(Einv) >= 0)
    best, start, lo, hi = 0, 0, 1, 0
    for kk in range(1, len(u) + 1):
        if kk == len(u) or not link[kk - 1]:
            if ok[start] and kk - start > best:
                best, lo, hi = kk - start, start, kk - 1
            start = kk
    if best >= 2:
        # intervals at the ends of the range whose linear interpolation
        # misses zero_find's energy at their midpoint by more than
        # SNS_INTERP_TOL (the inverse spectrum bends sharply at its ends,
        # e.g. VERDI's 0.1 meV lower limit) go to the per-draw tail table
        # while it has room
        um = (u[lo:hi] + u[lo + 1:hi + 1]) / 2
        Em = zero_find(Es, Pvec, EPmin + um * (EPmax - EPmin), xmin, xmax,
                       1e-7)
        bad = (np.abs((Einv[lo:hi] + Einv[lo + 1:hi + 1]) / 2 - Em)
               > SNS_INTERP_TOL * np.abs(Em))
        room = SNS_TAIL_MAX // (UNIFORM_STEPS // SNS_E_NODES) - 1
        while room > 0 and hi - lo > 2 and bad[0]:
            lo, bad, room = lo + 1, bad[1:], room - 1
        while room > 0 and hi - lo > 2 and bad[-1]:
            hi, bad, room = hi - 1, bad[:-1], room - 1
        u_lo, u_hi = u[lo], u[hi]
    else:
        u_lo, u_hi = 1.0, 0.0  # every draw takes the FP64 sampler
    t0, t1 = tidx[0], tidx[1] - 1
    mass = Ptmat[:, t1] - Ptmat[:, t0]
    ut = np.arange(SNS_T_NODES + 1) / SNS_T_NODES
    rows = np.repeat(np.arange(nE), SNS_T_NODES + 1)
    targ = (Ptmat[rows, t0] + np.tile(ut, nE) * mass[rows])
    Tinv = zero_find(ts, Ptmat, targ, ts[t0], ts[t1], 1e-5, rows=rows)
    # the draws outside [u_lo, u_hi]: an FP32 uniform is k * 2^-24, so
    # each such draw is one of a few thousand k, whose energies zero_find
    # gives here once (the kernels index them by k instead of running the
    # FP64 sampler); none when there are too many
    n_lo = int(np.ceil(u_lo * UNIFORM_STEPS))
    first_hi = int(np.floor(u_hi * UNIFORM_STEPS)) + 1
    n_hi = max(0, UNIFORM_STEPS - first_hi)
    if n_lo + n_hi > SNS_TAIL_MAX:
        n_lo = n_hi = 0
    lo_k = np.arange(n_lo, dtype=np.float64)
    hi_k = np.arange(first_hi, first_hi + n_hi, dtype=np.float64)
    uk = np.concatenate([lo_k, hi_k]) / UNIFORM_STEPS
    Etail = zero_find(Es, Pvec, EPmin + uk * (EPmax - EPmin), xmin, xmax,
                      1e-7) if len(uk) else uk
    ftab = np.concatenate([Einv, Es, np.maximum(mass, 0.0), Tinv, Etail])
    return (ftab.astype(np.float32), float(u_lo), float(u_hi), len(lo_k),
            len(hi_k))


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
        if getattr(self, "_fp32", None) is None:
            self._fp32 = fp32_tables(Es, Pvec, ts, Ptmat, EPmin, EPmax,
                                     (Eidx_start, Eidx_stop),
                                     (tidx_start, tidx_stop))
        ftab, u_lo, u_hi, n_lo, n_hi = self._fp32
        c.ftable = binder.table(self, "moderator_f32", ftab, np.float32)
        set_param(c, 16, u_lo)
        set_param(c, 17, u_hi)
        set_param(c, 18, n_lo)
        set_param(c, 19, n_hi)
        self.pack_geometry(c)

    def pack_geometry(self, c):
        c.ip[7] = 0


class STS_source(SNS_source):
    """STS moderator source (acc/components/sources/STS_source.py:107-284):
    the SNS source's energy and time draws, on a cylindrical moderator
    whose radius, port size and flight angle come from the file's
    section 0."""

    def __init__(self, name, filename, Emin, Emax, xwidth, yheight, dist,
                 focus_xw, focus_yh, PPower=0.0, frequency=0.0,
                 MOffangle=-1000.0, dmode=1.0, radius=0.0):
        self.name = name
        self.Emin, self.Emax = Emin, Emax
        (self.INorm2, Es, Pvec, ts, Ptmat, EPmin, EPmax, Eidx_range,
         tidx_range, sts_params) = init(Emin, Emax, filename, sts_load=True)
        self.xwidth, self.yheight, self.radius = xwidth, yheight, radius
        self.PPower, self.frequency = PPower, frequency
        (self.PPower0, self.Freq0, self.MRadius0, MOffangle0, PHeight,
         PWidth, TRadius) = sts_params
        # the file's flight angle is used (:134-138)
        self.MOffangle = MOffangle0
        if MOffangle != MOffangle0 and MOffangle > -1000.0:
            warnings.warn("Requested MOffangle different from value in "
                          "source file")
        self.MOffangle_rad = math.pi / 180.0 * self.MOffangle
        self.tanMOa = 1.0
        # the reference sets the cylinder only for square ports (:160-175)
        self.cylx = self.cylz = self.cylphi1 = self.cylphi2 = 0.0
        if TRadius > 0.0:
            Anorm = np.pi * TRadius * TRadius
            if self.radius > TRadius or self.radius <= 0.0:
                self.radius = TRadius
                warnings.warn("radius not set or requested is larger than "
                              "TRadius. Setting radius=TRadius.")
            self.square = False
            srcArea = np.pi * self.radius * self.radius
            self.tanMOa = math.tan(self.MOffangle_rad)
        else:
            Anorm = PWidth * PHeight
            if self.xwidth > PWidth or self.xwidth <= 0.0:
                self.xwidth = PWidth
                warnings.warn("xwidth not set or requested larger than "
                              "PWidth. Setting xwidth=PWidth")
            if self.yheight > PHeight or self.yheight <= 0.0:
                self.yheight = PHeight
                warnings.warn("yheight not set or requested larger than "
                              "PHeight. Setting yheight=PHeight")
            self.square = True
            srcArea = self.xwidth * self.yheight
            MR = self.MRadius0
            self.cylz = -MR * math.cos(self.MOffangle_rad)
            self.cylx = -MR * math.sin(self.MOffangle_rad)
            arg = math.sqrt(MR * MR - (self.xwidth / 2.0 - self.cylx) ** 2) \
                + self.cylz
            self.cylphi1 = 2.0 * math.asin(
                math.sqrt(arg * arg + 0.25 * self.xwidth * self.xwidth)
                / 2.0 / MR)
            arg = math.sqrt(MR * MR - (-self.xwidth / 2.0 - self.cylx) ** 2) \
                + self.cylz
            self.cylphi2 = 2.0 * math.asin(
                math.sqrt(arg * arg + 0.25 * self.xwidth * self.xwidth)
                / 2.0 / MR)
        self.p_in = focus_xw * focus_yh / (dist * dist) * srcArea / Anorm
        if self.PPower > 0.0:
            self.p_in *= self.PPower / self.PPower0
        if self.frequency > 0.0:
            self.p_in *= self.Freq0 / self.frequency
        self.dmode = dmode == 1.0
        self._prob = self.p_in * self.INorm2
        self.dist, self.focus_xw, self.focus_yh = dist, focus_xw, focus_yh
        self.Anorm = Anorm
        self.tables = (Es, Pvec, ts, Ptmat)
        # as the reference, the sampling uses the requested xwidth, yheight
        # and radius (:203-206), the area the adjusted ones
        self.propagate_params = (
            self.square, xwidth, yheight, radius, focus_xw, focus_yh, dist,
            EPmin, EPmax, Es, Eidx_range[0], Eidx_range[1], Pvec, ts,
            tidx_range[0], tidx_range[1], Ptmat, self._prob)

    def pack_geometry(self, c):
        c.ip[7] = 1 | (2 if self.dmode else 0)
        for k, v in enumerate((self.tanMOa, self.cylx, self.cylz,
                               self.cylphi1, self.cylphi2, self.MRadius0,
                               self.MOffangle_rad)):
            set_param(c, 9 + k, v)
