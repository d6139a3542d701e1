"""Kernel descriptions packed into an HSS component.

mu (absorption) and sigma (scattering) are coefficients in 1/m; mu is the
value at 2200 m/s and scales as 1/v (acc/kernels/__init__.py:149-161).
"""

from collections import namedtuple
from math import pi

import numpy as np

from .. import _native as nat
from ..conversion import K2V, V2K


def coefficient_from_cross_section(number_density, cross_section_barn):
    """n [1/A^3] x sigma [barn] -> 1/m (1 barn/A^3 = 100 /m)."""
    return float(number_density) * float(cross_section_barn) * 100.0


class IsotropicKernel:
    """isotropic.S (acc/kernels/isotropic.py:5-21) with p *= sigma
    (acc/kernels/__init__.py:36-44)."""
    kind = nat.KERNEL_ISOTROPIC

    def __init__(self, absorption_coefficient, scattering_coefficient):
        self.absorption_coefficient = float(absorption_coefficient)
        self.scattering_coefficient = float(scattering_coefficient)

    def pack(self, comp, c, binder, set_param):
        set_param(c, 8, self.absorption_coefficient)
        set_param(c, 9, self.scattering_coefficient)


Peak = namedtuple("Peak", "q F_squared multiplicity DebyeWaller_factor "
                  "intrinsic_line_width")


class PowderDiffraction:
    """Peak tables of acc/kernels/powderdiffr.py:112-155: per peak
    my_s_v2 = 4 pi^3 pack DW / V / V2K^2 * mult F^2 / q * XsectionFactor,
    q_v = q K2V, w_v = intrinsic line width; peaks sorted by q."""

    def __init__(self, peaks, unitcell_volume, absorption_cross_section,
                 incoherent_cross_section, coherent_cross_section, pack=1.,
                 XsectionFactor=100., d_phi=0):
        n = len(peaks)
        q_v = np.zeros(n)
        w_v = np.zeros(n)
        my_s_v2 = np.zeros(n)
        for i, pk in enumerate(peaks):
            dw = pk.DebyeWaller_factor
            dw = dw if dw > 0 else 1.0
            my_s_v2[i] = 4 * pi * pi * pi * pack * dw / unitcell_volume / (V2K * V2K)
            my_s_v2[i] *= (pk.multiplicity * pk.F_squared / pk.q) * XsectionFactor
            q_v[i] = pk.q * K2V
            w_v[i] = pk.intrinsic_line_width
            if i > 0:
                assert q_v[i - 1] <= q_v[i], "peaks must be sorted by q"
        self.absorption_cross_section = pack * absorption_cross_section
        self.absorption_coeff = absorption_cross_section / unitcell_volume * 100
        self.incoherent_cross_section = incoherent_cross_section
        self.coherent_cross_section = coherent_cross_section
        self.Npeaks = n
        self.q_v, self.w_v, self.my_s_v2 = q_v, w_v, my_s_v2
        self.d_phi = d_phi
        self.unitcell_volume = unitcell_volume

    def table(self):
        """rows {q_v, w_v, my_s_v2, cumulative my_s_v2} (float64)."""
        return np.stack([self.q_v, self.w_v, self.my_s_v2,
                         np.cumsum(self.my_s_v2)], axis=1)


class SimplePowderDiffractionKernel:
    """powderdiffr.scatter / scattering_coefficient
    (acc/kernels/powderdiffr.py:10-109); mu defaults to the kernel's
    absorption cross section over the unit cell."""
    kind = nat.KERNEL_POWDER

    def __init__(self, peaks, unitcell_volume, absorption_cross_section=0.,
                 incoherent_cross_section=0., coherent_cross_section=0.,
                 d_phi=0, pack=1., absorption_coefficient=None):
        self.peaks = sorted(peaks, key=lambda p: p.q)
        self.unitcell_volume = float(unitcell_volume)
        self.pd = PowderDiffraction(
            self.peaks, self.unitcell_volume, absorption_cross_section,
            incoherent_cross_section, coherent_cross_section, pack=pack,
            d_phi=d_phi)
        self.absorption_coefficient = (
            self.pd.absorption_coeff if absorption_coefficient is None
            else float(absorption_coefficient))

    def pack(self, comp, c, binder, set_param):
        tab = self.pd.table()
        set_param(c, 8, self.absorption_coefficient)
        set_param(c, 9, 0.0)
        set_param(c, 10, self.unitcell_volume)
        set_param(c, 11, self.pd.d_phi)
        c.ip[4] = self.pd.Npeaks
        c.table = binder.table(comp, "powder", tab, np.float64)
        c.ftable = binder.table(comp, "powder_f32", tab, np.float32)
        c.table_len = tab.size


class SQEGridKernel:
    """Gridded S(Q,E) kernel: S sampled on nQ x nE nodes spanning
    [Qmin, Qmax] x [Emin, Emax], bilinear in between; (Q, E) drawn uniformly
    over that box with the kinematics of acc/kernels/E_Q.py:37-99.
    No reference counterpart."""
    kind = nat.KERNEL_SQE_GRID

    def __init__(self, S, Qmin, Qmax, Emin, Emax, absorption_coefficient,
                 scattering_coefficient):
        S = np.ascontiguousarray(S, dtype=np.float32)
        if S.ndim != 2 or S.shape[0] < 2 or S.shape[1] < 2:
            raise ValueError("S must be a (nQ >= 2, nE >= 2) array")
        self.S = S
        self.Qmin, self.Qmax = float(Qmin), float(Qmax)
        self.Emin, self.Emax = float(Emin), float(Emax)
        self.absorption_coefficient = float(absorption_coefficient)
        self.scattering_coefficient = float(scattering_coefficient)

    def pack(self, comp, c, binder, set_param):
        set_param(c, 8, self.absorption_coefficient)
        set_param(c, 9, self.scattering_coefficient)
        for k, v in enumerate((self.Qmin, self.Qmax, self.Emin, self.Emax)):
            set_param(c, 10 + k, v)
        c.ip[4], c.ip[5] = self.S.shape
        p = binder.table(comp, "sqe", self.S, np.float32)
        c.table = p
        c.ftable = p
        c.table_len = self.S.size


class ConstantQEKernel:
    """constant_qe.S (acc/kernels/constant_qe.py:15-67) with p *= sigma
    (acc/kernels/__init__.py:76-88): every scattered neutron takes the
    momentum transfer Q (1/A) and the energy transfer E (meV), at a
    uniform azimuth about its incident direction.  A neutron that cannot
    make that transfer is absorbed."""
    kind = nat.KERNEL_CONSTANT_QE

    def __init__(self, Q, E, absorption_coefficient, scattering_coefficient):
        self.Q, self.E = float(Q), float(E)
        self.absorption_coefficient = float(absorption_coefficient)
        self.scattering_coefficient = float(scattering_coefficient)

    def pack(self, comp, c, binder, set_param):
        set_param(c, 8, self.absorption_coefficient)
        set_param(c, 9, self.scattering_coefficient)
        set_param(c, 10, self.Q)
        set_param(c, 11, self.E)


class E_Q_Kernel:
    """The makeS kernel of acc/kernels/E_Q.py:16-117 with p *= sigma
    (acc/kernels/__init__.py:90-105): an analytic dispersion E(Q) and
    intensity S(Q), both Python expressions in Q (1/A) with the names of
    the math module ("^" is "**"), Q drawn on [Qmin, Qmax) with up to
    max_iter tries.  The expressions are compiled to postfix programs on
    the host (expression.compile_expression)."""
    kind = nat.KERNEL_E_Q

    def __init__(self, E_Q, S_Q, Qmin, Qmax, absorption_coefficient,
                 scattering_coefficient, max_iter=100):
        from .expression import compile_expression
        self.E_Q, self.S_Q = str(E_Q), str(S_Q)
        self.Qmin, self.Qmax = float(Qmin), float(Qmax)
        self.max_iter = int(max_iter)
        if self.max_iter < 1:
            raise ValueError("max_iter must be >= 1")
        self.absorption_coefficient = float(absorption_coefficient)
        self.scattering_coefficient = float(scattering_coefficient)
        self.E_prog = compile_expression(self.E_Q)
        self.S_prog = compile_expression(self.S_Q)

    def E_depends_on_Q(self):
        """Whether the E(Q) program reads Q."""
        from .expression import Q_
        return bool(np.any(np.asarray(self.E_prog)[:, 0] == Q_))

    def program(self):
        """{opcode, argument} rows: the E(Q) program, then the S(Q) one."""
        return np.concatenate([self.E_prog, self.S_prog])

    def pack(self, comp, c, binder, set_param):
        set_param(c, 8, self.absorption_coefficient)
        set_param(c, 9, self.scattering_coefficient)
        set_param(c, 10, self.Qmin)
        set_param(c, 11, self.Qmax)
        set_param(c, 12, float(self.max_iter))
        # 1 when E(Q) does not read Q: the device evaluates it once per
        # scatter instead of once per try (same values, same draws)
        set_param(c, 13, 0.0 if self.E_depends_on_Q() else 1.0)
        c.ip[4], c.ip[5] = len(self.E_prog), len(self.S_prog)
        flat = np.ascontiguousarray(self.program().reshape(-1))
        c.table = binder.table(comp, "expr", flat, np.float64)
        c.ftable = binder.table(comp, "expr_f32", flat, np.float32)
        c.table_len = flat.size


class CompositeKernel:
    """The composite kernel of acc/kernels/composite.py:7-127 (rendered by
    acc/kernels/__init__.py:24-34): `elements` (1..16 kernels, none of them
    composite) with weights (each element's `weight`, 1 when it has none),
    normalised to sum 1.  A scattering picks element i with probability
    w_i, lets it scatter and divides p by w_i.  The scattering coefficient
    is the sum of the elements' (divided by N when `average`), the
    absorption coefficient their mean.  Its elements take the chain slots
    after the sample (include/acc_gb300.h, COMPOSITE)."""
    kind = nat.KERNEL_COMPOSITE

    def __init__(self, elements, weights=None, average=False):
        elements = list(elements)
        if not 1 <= len(elements) <= nat.MCV_COMPOSITE_MAX:
            raise ValueError(f"a composite kernel holds 1.."
                             f"{nat.MCV_COMPOSITE_MAX} elements")
        if any(isinstance(e, CompositeKernel) for e in elements):
            raise ValueError("composite kernels do not nest")
        if weights is None:
            weights = [float(getattr(e, "weight", 1.0)) for e in elements]
        weights = np.asarray(weights, dtype=np.float64)
        if weights.shape != (len(elements),) or not np.all(weights > 0):
            raise ValueError("one positive weight per element")
        self.elements = elements
        self.weights = weights / weights.sum()
        self.average = bool(average)
        self.n_slots = len(elements)

    def pack(self, comp, c, binder, set_param):
        c.ip[4] = len(self.elements)
        # mu, sigma and the speed-dependence flag follow in pack_elements,
        # once the elements' own slots are packed

    def pack_elements(self, c, slots, binder, set_param):
        n = len(self.elements)
        scale = 1.0 / n if self.average else 1.0
        cum, mu, sigma, speed = 0.0, 0.0, 0.0, False
        for i, (e, w, cs) in enumerate(zip(self.elements, self.weights,
                                           slots)):
            cs.opcode = nat.OP_KERNEL_ELEMENT
            cs.ip[1] = e.kind
            # the element is the owner of its tables (one set per element)
            e.pack(e, cs, binder, set_param)
            cum = 1.0 if i == n - 1 else cum + float(w)
            set_param(cs, 22, float(w))
            set_param(cs, 23, cum)
            mu += cs.dp[8]
            if e.kind == nat.KERNEL_POWDER:
                speed = True
            else:
                sigma += cs.dp[9]
        set_param(c, 8, mu / n)
        set_param(c, 9, sigma * scale)
        set_param(c, 10, scale)
        c.ip[5] = 1 if speed else 0


class SANS2D_ongrid_Kernel:
    """acc/kernels/SANS2D_ongrid.py:16-78 with p *= sigma
    (acc/kernels/__init__.py:107-122): small-angle scattering from
    S(Qx, Qy) on a grid.  `S_QxQy` is the reference's image, indexed
    (y, x) (a .npy path or an array); the kernel stores its transpose.
    (Qx, Qy) is drawn uniformly over the box and S interpolated bilinearly
    on cells of width (Qmax - Qmin) / n."""
    kind = nat.KERNEL_SANS2D

    def __init__(self, S_QxQy, Qx_min, Qx_max, Qy_min, Qy_max,
                 absorption_coefficient, scattering_coefficient):
        if isinstance(S_QxQy, str):
            S_QxQy = np.load(S_QxQy)
        img = np.asarray(S_QxQy, dtype=np.float64)
        if img.ndim != 2 or min(img.shape) < 2:
            raise ValueError("S_QxQy must be a (ny >= 2, nx >= 2) image")
        self.S_QxQy = img
        self.S = np.ascontiguousarray(img.T)  # [nx][ny]
        self.Qx_min, self.Qx_max = float(Qx_min), float(Qx_max)
        self.Qy_min, self.Qy_max = float(Qy_min), float(Qy_max)
        self.absorption_coefficient = float(absorption_coefficient)
        self.scattering_coefficient = float(scattering_coefficient)

    def pack(self, comp, c, binder, set_param):
        set_param(c, 8, self.absorption_coefficient)
        set_param(c, 9, self.scattering_coefficient)
        for k, v in enumerate((self.Qx_min, self.Qx_max, self.Qy_min,
                               self.Qy_max)):
            set_param(c, 10 + k, v)
        c.ip[4], c.ip[5] = self.S.shape
        c.table = binder.table(comp, "sans2d", self.S, np.float64)
        c.ftable = binder.table(comp, "sans2d_f32", self.S, np.float32)
        c.table_len = self.S.size


class DGSSXResKernel:
    """acc/kernels/DGSSXResKernel.py:19-98 with p *= sigma
    (acc/kernels/__init__.py:124-146): every neutron scatters towards a
    target disc of `target_radius` (m) at `target_position` (m, the
    sample's frame), arriving at a time of flight uniform in
    tof_at_target +- dtof / 2 (s) -- the resolution kernel of a
    single-crystal direct-geometry spectrometer."""
    kind = nat.KERNEL_DGSSXRES

    def __init__(self, target_position, target_radius, tof_at_target, dtof,
                 absorption_coefficient, scattering_coefficient):
        self.target_position = tuple(float(v) for v in target_position)
        self.target_radius = float(target_radius)
        self.tof_at_target = float(tof_at_target)
        self.dtof = float(dtof)
        self.absorption_coefficient = float(absorption_coefficient)
        self.scattering_coefficient = float(scattering_coefficient)

    def pack(self, comp, c, binder, set_param):
        set_param(c, 8, self.absorption_coefficient)
        set_param(c, 9, self.scattering_coefficient)
        for k, v in enumerate(self.target_position):
            set_param(c, 15 + k, v)
        set_param(c, 18, self.target_radius)
        set_param(c, 19, self.tof_at_target)
        set_param(c, 20, self.dtof)
