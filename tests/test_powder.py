"""Powder diffraction (acc/kernels/powderdiffr.py) on the CPU: the peak
tables against values worked out here by hand for the reference's Al
sample, and the oracle's scatter against the Bragg condition.

The Al sample is the reference's
tests/components/samples/sampleassemblies/Al-simplepowderdiffractionkernel
(peaks.py): a = 4.04932 A, 4 atoms, peaks (q = 1.92 /A, F^2 = 0, mult 12)
and (q = 3.1353 /A, F^2 = 3.3, mult 8), Debye-Waller factor 0 (read as 1),
cross sections 4 x (1.495 coh, 0.0082 inc, 0.231 abs) barn.
"""

import math

import numpy as np

from acc_gb300.components.samples.homogeneous_single_scatterer import factory
from acc_gb300.conversion import K2V, SE2V, V2K
from acc_gb300.geometry import Sphere
from acc_gb300.kernels import Peak, PowderDiffraction, \
    SimplePowderDiffractionKernel
from acc_gb300.memory import HostBinder

A = 4.049320
V = A ** 3
AL = [Peak(q=1.9200, F_squared=0.0, multiplicity=12,
           DebyeWaller_factor=0, intrinsic_line_width=0),
      Peak(q=3.1353, F_squared=3.3, multiplicity=8,
           DebyeWaller_factor=0, intrinsic_line_width=0)]


def test_al_peak_table_by_hand():
    pd = PowderDiffraction(AL, V, 4 * 0.231, 4 * 0.0082, 4 * 1.495)
    # my_s_v2 = 4 pi^3 * pack * DW / V / V2K^2 * mult * F^2 / q * 100
    # (powderdiffr.py:129-131) with pack = 1, DW = 1 (a zero factor reads
    # as 1, :127-128)
    # 4.04932^3 = 66.39667 A^3; 4 pi^3 = 124.02511; V2K^2 = 2.5225490e-6
    assert abs(V - 66.39667) < 1e-5
    pref = 124.02511 / 66.39667 / 2.5225490e-6
    assert abs(pref / 740497.5 - 1) < 1e-6
    # peak 2: 740497.5 * 8 * 3.3 / 3.1353 * 100 = 6.235172e8 (m/s)^2 barn
    assert pd.my_s_v2[0] == 0.0
    assert abs(pd.my_s_v2[1] / 6.235172e8 - 1) < 1e-6
    # q_v = q K2V with K2V = 1/V2K = 629.62237 m/s per 1/A (:134)
    np.testing.assert_allclose(pd.q_v, [1.92 * 629.62237, 3.1353 * 629.62237],
                               rtol=1e-8)
    # absorption coefficient: sigma_abs / V * 100 = 0.924 / 66.39667 * 100
    # = 1.391636 /m (:148)
    assert abs(pd.absorption_coeff / 1.391636 - 1) < 1e-6
    assert pd.Npeaks == 2 and list(pd.w_v) == [0.0, 0.0]


def _scatter(comp_struct, v, seed, index):
    from oracle import binding as O
    n = np.array([0, 0, 0, 0, 0, v, 0, 0, 0, 1.0])
    return O.kernel_scatter_one(comp_struct, n, seed=seed, index=index)


def _powder_struct(peaks, vol):
    ker = SimplePowderDiffractionKernel(peaks, vol,
                                        absorption_cross_section=0.924)
    H = factory(Sphere(0.01), ker)("s")
    b = HostBinder()
    return H.to_struct(b), b, ker


def test_oracle_scatter_obeys_bragg():
    """For config 5's 50 peaks and incident speeds over 5-100 meV: |v| is
    preserved, the turn between incident and outgoing velocity is 2 theta
    of a reachable peak, theta = asin(q_v / (2 v)), and the weight factor
    is Nreach * my_s_v2 / v^2 / V_uc of that peak (powderdiffr.py:27-109;
    Nreach counts the peaks with q_v <= 2 v, less one when all are
    reachable: the reference's loop leaves its index at Npeaks - 1)."""
    import acc_gb300.instruments as I
    peaks = I.powder_peaks()
    c, b, ker = _powder_struct(peaks, 66.4)
    pd = ker.pd
    rng = np.random.default_rng(4)
    checked = 0
    for i in range(400):
        v = SE2V * math.sqrt(rng.uniform(5, 100))
        out = _scatter(c, v, seed=3, index=i)
        vout = out[3:6]
        assert abs(np.linalg.norm(vout) / v - 1) < 1e-13
        turn = math.acos(np.clip(vout[2] / np.linalg.norm(vout), -1, 1))
        reach = pd.q_v <= 2 * v
        nreach = int(reach.sum())
        if nreach == pd.Npeaks:
            nreach -= 1
        nreach = max(nreach, 1)
        thetas = np.arcsin(np.clip(pd.q_v[:nreach] / (2 * v), -1, 1))
        k = int(np.argmin(np.abs(2 * thetas - turn)))
        assert abs(2 * thetas[k] - turn) < 1e-7, (i, turn, 2 * thetas[k])
        expect = nreach * pd.my_s_v2[k] / v ** 2 / 66.4
        assert abs(out[9] / expect - 1) < 1e-12
        checked += 1
    assert checked == 400


def test_oracle_scatter_below_first_peak_absorbs():
    """v < q_v[0] / 2: the neutron is absorbed (powderdiffr.py:33-35)."""
    c, b, ker = _powder_struct(AL, V)
    v = 0.99 * ker.pd.q_v[0] / 2
    out = _scatter(c, v, seed=1, index=0)
    assert out[9] == -1
    assert np.allclose(out[3:6], [0, 0, v])
    # Al: a neutron reaching both peaks picks peak 0 only (the quirk), with
    # F^2 = 0 there, so its weight becomes 0
    v = 1.01 * ker.pd.q_v[1] / 2
    out = _scatter(c, v, seed=1, index=1)
    assert out[9] == 0.0
    assert abs(V2K * K2V - 1) < 1e-15
