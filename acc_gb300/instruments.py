"""Example instruments: the workloads the engine is benchmarked and tested on.

sphere_theta_tof   disc source -> isotropic sphere -> 4pi theta x tof shell
guide_chain        disc source -> 10 m guide -> 5 m tapered guide ->
                   100x100 PSD + 200-bin energy monitor
sqe_hollow_cylinder  60 meV beam -> hollow cylinder with a gridded S(Q,E)
                   -> 3 m cylinder detector binned in I(Q,E)
powder_banked      guide chain -> powder cylinder -> banked cylinder detector
constant_qe_box    70 meV beam -> Al block with the constant-(Q, E) kernel ->
                   I(Q, E) monitor
e_q_box            70 meV beam -> Al block with an analytic E(Q) dispersion
                   -> I(Q, E) monitor
un_ms              500 meV beam -> UN cylinder, multiple scattering with a
                   composite of 8 E(Q) kernels -> I(Q, E) monitor
verdi              the VERDI instrument (SNS source, elliptic guides)
sans2d_grid        10 A beam -> thin Al plate with S(Qx, Qy) on a 1475 x
                   1100 grid -> PSD 10 m downstream
saved_guide_chain  guide_chain saving the neutrons at the guide exit (.mcv);
                   guide_exit_replay replays them onto the same monitors

Numbers that the workload descriptions leave open are fixed here once
(source distance, gaps between components, detector heights, number
densities) and documented beside each builder.
"""

import math
import os

import numpy as np

from .components.monitors.cylinder_detectors import (BankedCylinder_detector,
                                                     CylinderIQE_detector)
from .components.monitors.energy_monitor import Energy_monitor
from .components.monitors.iqe_monitor import IQE_monitor
from .components.monitors.psd_monitor import PSD_monitor
from .components.monitors.psd_monitor_4pi import PSD_monitor_4Pi
from .components.monitors.theta_tof_monitor_4pi import ThetaTOF_monitor_4Pi
from .components.optics.guide import Guide
from .components.samples.homogeneous_single_scatterer import factory
from .components.sources.source_simple import Source_simple
from .geometry import Block, Cylinder, Difference, HollowCylinder, Sphere
from .instrument import instrument
from .kernels import (CompositeKernel, ConstantQEKernel, DGSSXResKernel,
                      E_Q_Kernel,
                      IsotropicKernel, Peak, SANS2D_ongrid_Kernel,
                      SimplePowderDiffractionKernel, SQEGridKernel,
                      coefficient_from_cross_section)

COATING = dict(R0=0.99, Qc=0.0219, alpha=3.0, m=3.0, W=0.003)

# the moderator files of the reference's tests
# (tests/components/sources), shipped gzip-compressed in acc_gb300/data
DATA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data")
SNS_MODERATOR = "source_rot2_cdr_cyl_3x3_20190417.dat"
STS_MODERATOR = "BL20-CY-123D-STS-Min-2G-source_mctal-195_sp.dat"


def shipped_moderator(name):
    """Path of a moderator file shipped with the package (SNS_MODERATOR:
    the SNS moderator VERDI reads, VERDI_base.py:17; STS_MODERATOR: the
    cylindrical STS moderator of test_STS_source.py)."""
    path = os.path.join(DATA, name + ".gz")
    if not os.path.exists(path):
        raise FileNotFoundError(
            f"{path} is missing: acc_gb300/data/copy_moderators.py copies "
            "it from the mcvine/acc source tree")
    return path


def sphere_theta_tof(ntheta=180, ntof=200):
    """Disc source (r = 5 cm) aimed at a 1 x 1 cm target 5 m away, E uniform
    in 50-70 meV; isotropic sphere r = 1 cm at the target with
    sigma_s = sigma_a = 5 b and n = 0.05 /A^3 (25 /m each, absorption at
    2200 m/s); 4pi shell of radius 3 m around the sample binned
    theta 0-180 deg x tof 0-10 ms."""
    ins = instrument("sphere_theta_tof")
    src = Source_simple("source", radius=0.05, dist=5.0, xw=0.01, yh=0.01,
                        E0=60.0, dE=10.0)
    mu = coefficient_from_cross_section(0.05, 5.0)
    sigma = coefficient_from_cross_section(0.05, 5.0)
    HSS = factory(Sphere(0.01), IsotropicKernel(mu, sigma))
    mon = ThetaTOF_monitor_4Pi("theta_tof", radius=3.0, ntheta=ntheta,
                               ntof=ntof, tofmin=0.0, tofmax=0.01,
                               filename="theta_tof.h5")
    ins.append(src, position=(0, 0, 0))
    ins.append(HSS("sample"), position=(0, 0, 5.0))
    ins.append(mon, position=(0, 0, 5.0))
    return ins


def guide_chain(extra=None):
    """Disc source (r = 5 cm, E uniform 5-100 meV) aimed at the 5 x 5 cm
    entrance of a 10 m straight guide 1 m away; a 5 m guide tapering
    5 x 5 cm -> 2 x 2 cm follows after a 1 mm gap (coating m=3, R0=0.99,
    Qc=0.0219 /A, alpha=3, W=0.003 /A); 1 mm after its exit a 100 x 100
    PSD over +-3 cm and a 200-bin energy monitor over 0-100 meV (same
    +-3 cm aperture).  `extra` components are appended at the exit."""
    ins = instrument("guide_chain")
    src = Source_simple("source", radius=0.05, dist=1.0, xw=0.05, yh=0.05,
                        E0=52.5, dE=47.5)
    g1 = Guide("guide1", w1=0.05, h1=0.05, w2=0.05, h2=0.05, l=10.0,
               **COATING)
    g2 = Guide("guide2", w1=0.05, h1=0.05, w2=0.02, h2=0.02, l=5.0, **COATING)
    psd = PSD_monitor("psd", xmin=-0.03, xmax=0.03, ymin=-0.03, ymax=0.03,
                      nx=100, ny=100, filename="psd.h5")
    emon = Energy_monitor("energy", xmin=-0.03, xmax=0.03, ymin=-0.03,
                          ymax=0.03, Emin=0.0, Emax=100.0, nchan=200,
                          filename="energy.h5")
    ins.append(src, position=(0, 0, 0))
    ins.append(g1, position=(0, 0, 1.0))
    ins.append(g2, position=(0, 0, 11.001))
    z = 16.002
    ins.append(psd, position=(0, 0, z))
    ins.append(emon, position=(0, 0, z))
    for c in extra or ():
        ins.append(c, position=(0, 0, z))
    return ins


def sqe_table(nQ=200, nE=200, Qmin=0.0, Qmax=10.0, Emin=-50.0, Emax=55.0):
    """Gaussian ridge of width 2 meV at E = 30 |sin(Q/2)| meV times
    exp(-0.01 Q^2) on nQ x nE nodes spanning the box."""
    Q = np.linspace(Qmin, Qmax, nQ)[:, None]
    E = np.linspace(Emin, Emax, nE)[None, :]
    S = np.exp(-(E - 30 * np.abs(np.sin(Q / 2))) ** 2 / (2 * 2.0 ** 2)) * \
        np.exp(-0.01 * Q ** 2)
    return S.astype(np.float32)


def sqe_hollow_cylinder(S=None, sigma_abs_barn=2.0, number_density=0.05,
                        sigma_s_barn=5.0, nQ=100, nE=100):
    """1 x 1 cm source, monochromatic 60 meV, aimed at a 1 x 1 cm target
    5 m away; hollow cylinder r 1.0-1.2 cm, height 5 cm, axis vertical,
    sigma_abs = 2 b, sigma_s = 5 b at 0.05 /A^3; S(Q,E) from `sqe_table`
    over Q 0-10 /A, E -50..55 meV; a vertical detector cylinder of radius
    3 m and height 2 m binned 100 x 100 in I(Q, E)."""
    ins = instrument("sqe_hollow_cylinder")
    src = Source_simple("source", radius=0, width=0.01, height=0.01, dist=5.0,
                        xw=0.01, yh=0.01, E0=60.0, dE=0.0)
    if S is None:
        S = sqe_table()
    ker = SQEGridKernel(S, 0.0, 10.0, -50.0, 55.0,
                        coefficient_from_cross_section(number_density,
                                                       sigma_abs_barn),
                        coefficient_from_cross_section(number_density,
                                                       sigma_s_barn))
    HSS = factory(HollowCylinder(0.010, 0.012, 0.05), ker)
    det = CylinderIQE_detector("iqe", radius=3.0, height=2.0, Ei=60.0,
                               Qmin=0.0, Qmax=10.0, nQ=nQ, Emin=-50.0,
                               Emax=55.0, nE=nE, filename="iqe.h5")
    ins.append(src, position=(0, 0, 0))
    # the cylinder's axis is local z; orientation (90, 0, 0) turns it vertical
    ins.append(HSS("sample"), position=(0, 0, 5.0), orientation=(90, 0, 0))
    ins.append(det, position=(0, 0, 5.0))
    return ins


def powder_peaks(npeaks=50, seed=0):
    """npeaks peaks with d uniform in 0.5-4 A, F^2 lognormal(0, 1),
    multiplicity from {2,4,6,8,12,24}, Debye-Waller exp(-0.005/d^2)."""
    rng = np.random.default_rng(seed)
    d = rng.uniform(0.5, 4.0, npeaks)
    F2 = rng.lognormal(0.0, 1.0, npeaks)
    mult = rng.choice([2, 4, 6, 8, 12, 24], npeaks)
    peaks = [Peak(q=2 * math.pi / di, F_squared=f, multiplicity=int(m),
                  DebyeWaller_factor=math.exp(-0.005 / di ** 2),
                  intrinsic_line_width=0.0)
             for di, f, m in zip(d, F2, mult)]
    return sorted(peaks, key=lambda p: p.q)


def powder_banked(peaks=None, unitcell_volume=66.4, nbanks=8, ntubes=128,
                  npixels=256, ntof=1000):
    """The guide chain feeding a powder cylinder (r = 0.5 cm, h = 4 cm,
    axis vertical) 0.5 m past the guide exit, and a banked vertical
    cylinder detector of radius 3 m and height 1 m around it: 8 banks of
    15 deg separated by 5 deg gaps from 10 deg, 128 tubes x 256 pixels,
    tof 0-20 ms in 1000 bins."""
    ins = guide_chain()
    peaks = powder_peaks() if peaks is None else peaks
    ker = SimplePowderDiffractionKernel(peaks, unitcell_volume,
                                        absorption_cross_section=0.23,
                                        incoherent_cross_section=0.0,
                                        coherent_cross_section=1.5)
    HSS = factory(Cylinder(0.005, 0.04), ker)
    det = BankedCylinder_detector("banked", radius=3.0, height=1.0,
                                  nbanks=nbanks, ntubes=ntubes,
                                  npixels=npixels, bank_angle0=10.0,
                                  bank_width=15.0, bank_gap=5.0, tofmin=0.0,
                                  tofmax=0.02, ntof=ntof,
                                  filename="banked.h5")
    z = 16.002 + 0.5
    ins.append(HSS("sample"), position=(0, 0, z), orientation=(90, 0, 0))
    ins.append(det, position=(0, 0, z))
    return ins


def synthetic_moderator_file(path=None, nE=60, nt=50, sts=False):
    """Write a moderator file in the format SNS_source reads
    (acc/components/sources/_SNS_source_utils.py:12-57) with a synthetic
    spectrum and pulse shapes (no measured data) and return its path (a
    temporary file when `path` is None):

      f(E) = E / kT^2 exp(-E / kT) + 0.02 / E   (Maxwellian at kT = 25 meV
                                                 with an epithermal tail)
      I(t, E) = (t / tau) exp(-t / tau),  tau = 20 us + 40 us sqrt(kT / E)

    on nE log-spaced energies in [1e-4, 10] eV and nt log-spaced times in
    [0.05, 3000] us.  `sts`: with the STS file's section 0 first (power
    700 kW, 15 Hz, moderator radius 3 cm, flight angle 5 deg, port 3 x
    3 cm, no disk)."""
    import tempfile
    if path is None:
        fd, path = tempfile.mkstemp(suffix=".dat", prefix="moderator_")
        os.close(fd)
    kT = 0.025
    E = np.logspace(-4, 1, nE)
    lam = 9.044567 / np.sqrt(E * 1000.0)
    fE = E / kT ** 2 * np.exp(-E / kT) + 0.02 / E
    t = np.logspace(np.log10(0.05), np.log10(3000.0), nt)
    lines = ["## synthetic moderator file (acc_gb300.instruments)"]
    if sts:
        lines += ["## section 0: PPower, Freq, MRadius, MOffangle, PHeight,"
                  " PWidth, TRadius, check", "  700.0", "  15.0", "  0.03",
                  "  5.0", "  0.03", "  0.03", "  0.0", "  12345678.0",
                  "## section 0 end"]
    lines += ["## section 1: E, wavelength, f(E), err, f(l), err"]
    for e, l, f in zip(E, lam, fE):
        lines.append(f"  {e:.6e}   {l:.6e}   {f:.6e}   {0.01 * f:.6e}"
                     f"   {f:.6e}   {0.01 * f:.6e}")
    lines += ["", "", "## section1end", "## section 2: t, E, I, err"]
    for e in E:
        tau = 20.0 + 40.0 * np.sqrt(kT / e)
        I = (t / tau) * np.exp(-t / tau)
        for tt, ii in zip(t, I):
            lines.append(f"  {tt:.6e}   {e:.6e}   {ii:.6e}   {0.01 * ii:.6e}")
        lines.append("")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")
    return path


def sns_source_chain(filename=None, Emin=5., Emax=20.):
    """An SNS moderator source (3 x 3 cm face, energies Emin-Emax meV from
    `filename`) aimed at a 3 x 3 cm
    window 5 m away, where a PSD (100 x 100 over +-3 cm) and an energy
    monitor (100 bins over 0-25 meV) sit: the reference's SNS source test
    set-up (tests/components/sources/test_SNS_source.py:12-15), on the
    reference's SNS moderator file when `filename` is None."""
    from .components.sources.SNS_source import SNS_source
    if filename is None:
        filename = shipped_moderator(SNS_MODERATOR)
    ins = instrument("sns_source_chain")
    src = SNS_source("src", filename, Emin, Emax, 0.03, 0.03, 5., .03, .03)
    psd = PSD_monitor("psd", xmin=-0.03, xmax=0.03, ymin=-0.03, ymax=0.03,
                      nx=100, ny=100, filename="psd.h5")
    emon = Energy_monitor("energy", xmin=-0.03, xmax=0.03, ymin=-0.03,
                          ymax=0.03, Emin=0.0, Emax=25.0, nchan=100,
                          filename="energy.h5")
    ins.append(src, position=(0, 0, 0))
    ins.append(psd, position=(0, 0, 5.0))
    ins.append(emon, position=(0, 0, 5.0))
    return ins


def sts_source_chain(filename=None, Emin=5., Emax=20., dmode=1.0):
    """An STS moderator source (the sns_source_chain set-up on the
    cylindrical moderator of an STS file; the reference's STS file when
    `filename` is None)."""
    from .components.sources.SNS_source import STS_source
    if filename is None:
        filename = shipped_moderator(STS_MODERATOR)
    ins = instrument("sts_source_chain")
    src = STS_source("src", filename, Emin, Emax, 0.03, 0.03, 5., .03, .03,
                     dmode=dmode)
    psd = PSD_monitor("psd", xmin=-0.03, xmax=0.03, ymin=-0.03, ymax=0.03,
                      nx=100, ny=100, filename="psd.h5")
    emon = Energy_monitor("energy", xmin=-0.03, xmax=0.03, ymin=-0.03,
                          ymax=0.03, Emin=0.0, Emax=25.0, nchan=100,
                          filename="energy.h5")
    ins.append(src, position=(0, 0, 0))
    ins.append(psd, position=(0, 0, 5.0))
    ins.append(emon, position=(0, 0, 5.0))
    return ins


def stored_neutrons(n=10007, seed=11):
    """n seeded neutrons (x y z vx vy vz sx sy t p rows) leaving z=0 within
    +-2 cm at about 2000 m/s along z, 1 ms, weights in [1e-4, 1e-3]."""
    rng = np.random.default_rng(seed)
    a = np.zeros((n, 10))
    a[:, 0:2] = rng.uniform(-0.02, 0.02, (n, 2))
    a[:, 3:5] = rng.normal(0.0, 10.0, (n, 2))
    a[:, 5] = rng.uniform(1500.0, 2500.0, n)
    a[:, 8] = 1e-3
    a[:, 9] = rng.uniform(1e-4, 1e-3, n)
    return a


def storage_chain(neutrons=None):
    """Stored neutrons (stored_neutrons() by default) replayed through a
    1 cm isotropic sphere 1 m downstream onto a 4pi theta x tof shell
    (NeutronFromStorage, neutronfromstorage.py:42-82)."""
    from .components.sources.neutronfromstorage import NeutronFromStorage
    if neutrons is None:
        neutrons = stored_neutrons()
    ins = instrument("storage_chain")
    sample = factory(Sphere(0.01), IsotropicKernel(25.0, 25.0))
    mon = ThetaTOF_monitor_4Pi("theta_tof", radius=3.0, ntheta=180, ntof=200,
                               tofmin=0.0, tofmax=0.01,
                               filename="theta_tof.h5")
    ins.append(NeutronFromStorage("src", neutrons=neutrons),
               position=(0, 0, 0))
    ins.append(sample("sample"), position=(0, 0, 1.0))
    ins.append(mon, position=(0, 0, 1.0))
    return ins


def saved_guide_chain(path="after_guide2.mcv", capacity=None):
    """guide_chain with a NeutronToStorage at the guide's exit plane, where
    the reference's instrument factory saves `after_<component>.mcv`
    (acc/test/instrument_factory.py:109-113)."""
    from .components.monitors.neutron_to_storage import NeutronToStorage
    return guide_chain(extra=[NeutronToStorage("after_guide2", path=path,
                                               capacity=capacity)])


def guide_exit_replay(neutrons):
    """Neutrons saved at the guide exit (saved_guide_chain; a .mcv path or
    an (N, 10) array) replayed onto guide_chain's PSD and energy monitors,
    in the same frame."""
    from .components.sources.neutronfromstorage import NeutronFromStorage
    src = (NeutronFromStorage("src", path=neutrons)
           if isinstance(neutrons, (str, os.PathLike))
           else NeutronFromStorage("src", neutrons=neutrons))
    ref = guide_chain()
    psd, emon = ref.components[3], ref.components[4]
    ins = instrument("guide_exit_replay")
    ins.append(src, position=(0, 0, 0))
    ins.append(psd, position=(0, 0, 0))
    ins.append(emon, position=(0, 0, 0))
    return ins


def elliptic_segments(nseg=100, w_in=0.05, w_mid=0.08, w_out=0.04,
                      h_in=0.05, h_mid=0.07, h_out=0.04):
    """(h1, h2, w1, w2) of `nseg` equal segments approximating a guide whose
    width and height follow half-ellipses through the entrance, middle and
    exit openings (a synthetic profile for tests and benchmarks)."""
    z = np.linspace(0.0, 1.0, nseg + 1)

    def profile(a_in, a_mid, a_out):
        # ellipse through (0, a_in), (0.5, a_mid), (1, a_out) in its
        # semi-axis form a(z) = a_mid * sqrt(1 - ((z - 0.5) / b)^2) + skew
        lin = a_in + (a_out - a_in) * z
        bulge = (a_mid - 0.5 * (a_in + a_out)) * np.sqrt(
            np.clip(1 - (2 * z - 1) ** 2, 0, None))
        return lin + bulge

    w, h = profile(w_in, w_mid, w_out), profile(h_in, h_mid, h_out)
    return h[:-1], h[1:], w[:-1], w[1:]


def tapered_guide_chain(nseg=100, length=10.99, mx=6., my=6.):
    """A 3 x 3 cm source (10 +- 9.5 A) 2 m before the 5 x 5 cm entrance of
    a segmented tapered guide of `length` m (elliptic profile, see
    elliptic_segments), a position-divergence monitor 1 mm after its exit
    (as the reference's acc_tapered_guide_instrument.py, with a synthetic
    profile in place of its segment file)."""
    from .components.monitors.posdiv_monitor import PosDiv_monitor
    from .components.optics.guide_tapering import Guide as TaperedGuide
    ins = instrument("tapered_guide_chain")
    src = Source_simple("source", radius=0., width=0.03, height=0.03,
                        dist=2.0, xw=0.05, yh=0.05, Lambda0=10.,
                        dLambda=9.5)
    guide = TaperedGuide("guide", l=length, mx=mx, my=my,
                         segments=elliptic_segments(nseg))
    mon = PosDiv_monitor("Ixdivx", npos=250, ndiv=250, xwidth=0.25,
                         yheight=0.25, maxdiv=0.5, filename="Ixdivx.h5")
    ins.append(src, position=(0, 0, 0))
    ins.append(guide, position=(0, 0, 2.0))
    ins.append(mon, position=(0, 0, 2.0 + length + 1e-3))
    return ins


def ms_hollow_cylinder(max_scattered_neutrons=16, max_ms_loops=2,
                       max_ms_loops_path1=5):
    """Multiple scattering: a 1 x 1 cm source 1 m from an 8 x 8 mm target,
    wavelength 10 +- 9.5 A, onto an isotropic hollow cylinder 2 m
    downstream (radii 1 and 2 cm, heights 7 and 6 cm, axis vertical,
    absorption and scattering 10/m), with a 4pi PSD of radius 1 m (90 x 90)
    around it: the test instrument of the reference's multiple scatterer
    (tests/components/samples/acc_ss_test_instrument.py,
    HMS_isotropic_hollowcylinder.py, test_homogeneous_multiple_scatterer.py
    :15-31)."""
    from .components.samples.homogeneous_multiple_scatterer import \
        factory as ms_factory
    ins = instrument("ms_hollow_cylinder")
    src = Source_simple("src", radius=0., width=0.01, height=0.01, dist=1.,
                        xw=0.008, yh=0.008, Lambda0=10., dLambda=9.5,
                        E0=0., dE=0.0, flux=1, gauss=0)
    shape = Difference(Cylinder(0.02, 0.06), Cylinder(0.01, 0.07))
    HMS = ms_factory(shape, IsotropicKernel(10., 10.),
                     max_scattered_neutrons=max_scattered_neutrons,
                     max_ms_loops=max_ms_loops,
                     max_ms_loops_path1=max_ms_loops_path1)
    mon = PSD_monitor_4Pi("psd_4pi", radius=1., nphi=90, ntheta=90,
                          filename="psd_4pi.h5")
    ins.append(src, position=(0, 0, 0))
    ins.append(HMS("sample"), position=(0, 0, 2.0), orientation=(90, 0, 0))
    ins.append(mon, position=(0, 0, 2.0))
    return ins


def sphere_variants(nvariants=64, seed=0, nmin=1e6, nmax=1e8, emin=20.0,
                    emax=500.0):
    """`nvariants` copies of the sphere_theta_tof chain, each with a
    monochromatic source at Ei log-uniform in [emin, emax] meV, a neutron
    count log-uniform in [nmin, nmax] and its own seed and histogram.
    Returns (instruments, counts, seeds)."""
    rng = np.random.default_rng(seed)
    Ei = np.exp(rng.uniform(np.log(emin), np.log(emax), nvariants))
    counts = np.exp(rng.uniform(np.log(nmin), np.log(nmax), nvariants))
    counts = [int(c) for c in counts]
    seeds = [int(s) for s in rng.integers(1, 2 ** 62, nvariants)]
    out = []
    for e in Ei:
        ins = sphere_theta_tof()
        src = ins.components[0]
        sp = list(src.propagate_params)
        sp[7], sp[8] = float(e), 0.0  # E0, dE
        src.propagate_params = tuple(sp)
        out.append(ins)
    return out, counts, seeds


# fcc Al, a = 4.04 A, 4 atoms per cell (the sample of the reference's
# constant-(Q, E) and E(Q) box tests); tabulated free-atom cross sections
# absorption 0.231 b (2200 m/s), coherent 1.495 b, incoherent 0.0082 b
AL_NUMBER_DENSITY = 4 / 4.04 ** 3
AL_MU = coefficient_from_cross_section(AL_NUMBER_DENSITY, 0.231)
AL_SIGMA = coefficient_from_cross_section(AL_NUMBER_DENSITY, 1.495 + 0.0082)


def _al_box(name, kernel):
    """The instrument of the reference's box tests
    (tests/components/samples/acc_ss_test_instrument.py:6-33 with the
    source and monitor of test_fccAl_E_Q_kernel.py:28-55): 1 x 1 cm source,
    70 +- 0.1 meV, aimed at 8 x 8 mm 1 m away; 6 x 10 x 1 cm block
    (width x height x thickness along the beam) 2 m downstream; I(Q, E)
    monitor at the sample, Q 0-8 /A x 160, E -60..60 meV x 120, all
    directions."""
    ins = instrument(name)
    src = Source_simple("src", radius=0.0, width=0.01, height=0.01, dist=1.0,
                        xw=0.008, yh=0.008, E0=70.0, dE=0.1, Lambda0=0.0,
                        dLambda=0.0)
    HSS = factory(Block(0.06, 0.10, 0.01), kernel)
    mon = IQE_monitor("iqe_monitor", Ei=70.0, Qmin=0.0, Qmax=8.0, nQ=160,
                      Emin=-60.0, Emax=60.0, nE=120,
                      min_angle_in_plane=0.0, max_angle_in_plane=359.0,
                      min_angle_out_of_plane=-90.0,
                      max_angle_out_of_plane=90.0)
    ins.append(src, position=(0, 0, 0))
    ins.append(HSS("sample"), position=(0, 0, 2.0))
    ins.append(mon, position=(0, 0, 2.0))
    return ins


def constant_qe_box(Q=3.0, E=30.0):
    """Al block scattering every neutron to Q = 3 /A, E = 30 meV
    (sampleassemblies/Al-constantqekernel/Al-scatterer.xml:7-8)."""
    return _al_box("constant_qe_box",
                   ConstantQEKernel(Q, E, AL_MU, AL_SIGMA))


def e_q_box(E_Q="30+20*sin(Q)", S_Q="1", Qmin=0.0, Qmax=10.0):
    """Al block with the dispersion E = 30 + 20 sin(Q) meV, S = 1 over
    Q 0-10 /A (sampleassemblies/Al-E_Q_kernel/Al-scatterer.xml:7-12)."""
    return _al_box("e_q_box",
                   E_Q_Kernel(E_Q, S_Q, Qmin, Qmax, AL_MU, AL_SIGMA))


# ---------------------------------------------------------------- VERDI
def ellipse_half_opening(z, a, b):
    """Half opening of an ellipse with semi-minor axis a and semi-major
    axis b, at distance z along the major axis from its vertex:
    a sqrt(z/b (2 - z/b)) (acc/test/ellipse.py:148-162)."""
    z = np.asarray(z, dtype=np.float64)
    return a * np.sqrt(z / b * (2 - z / b))


def shield_vertex(a, b, z_src, src_size, z_guide_start, z_guide_end,
                  z_target, target_size):
    """Where the ray from the source's lower edge to the guide exit's upper
    edge crosses the ray from the guide entrance's upper edge to the
    target's lower edge: the tip (x, z) of the shield that blocks the
    direct line of sight of a single-wall elliptic mirror
    (SingleWall.calc_shield_xz, acc/test/ellipse.py:37-54)."""
    x_end = float(ellipse_half_opening(z_guide_end - z_src, a, b))
    x_src = -src_size / 2.
    k1 = (x_end - x_src) / (z_guide_end - z_src)
    b1 = x_src - k1 * z_src
    x_start = float(ellipse_half_opening(z_guide_start - z_src, a, b))
    x_tgt = -target_size / 2.
    k2 = (x_tgt - x_start) / (z_target - z_guide_start)
    b2 = x_tgt - k2 * z_target
    z = (b2 - b1) / (k1 - k2)
    return k1 * z + b1, z


def elliptic_guide_segments(z_center, z_start, z_exit, nseg, major, minor):
    """(h1, h2, w1, w2) of `nseg` equal segments from z_start to z_exit of
    an elliptic guide (both axes of the opening on the same ellipse,
    centre at z_center), as the segment files of
    acc/test/ellipse.py:101-145 list them; the tapered guide's loader then
    drops the last one, as the reference's does."""
    b, a = major / 2., minor / 2.
    zs, step = np.linspace(z_start, z_exit, nseg, retstep=True,
                           endpoint=False)
    zs = zs - (z_center - b)
    h1 = 2 * ellipse_half_opening(zs, a, b)
    h2 = 2 * ellipse_half_opening(zs + step, a, b)
    return h1, h2, h1.copy(), h2.copy()


def verdi(moderator_file=None, guide_mvalue=6., sample_width=0.005,
          sample_height=0.005, source_width=0.03, source_height=0.03,
          secsource_size=0.02, xDivergence=2, yDivergence=2,
          guide1_start=6.35, guide1_len=10.99 + 9.56,
          ellipse1_major_axis_len=31.75, ellipse1_minor_axis_len=0.21,
          guide2_start=35.05, guide2_len=2.44 + 1.01,
          ellipse2_major_axis_len=40.0 - 31.75, ellipse2_minor_axis_len=0.1,
          guide_n_segments=500, Emin=0.1, Emax=1000.):
    """The VERDI instrument of tests/instruments/VERDI/VERDI_base.py:14-339
    (the reference's largest acc instrument, timed in its walltime.txt):
    SNS moderator -> two elliptic mirrors, each cut in two tapered guides of
    499 segments with a two-plate shield between them -> secondary-source
    slit -> sample mask, with wavelength, position-divergence and PSD
    monitors along the way (26 components, 4 of them arms).

    `moderator_file`: a moderator file in the SNS format; VERDI's own
    (source_rot2_cdr_cyl_3x3_20190417.dat, VERDI_base.py:17) when None."""
    from .components.monitors.posdiv_monitor import PosDiv_monitor
    from .components.monitors.wavelength_monitor import Wavelength_monitor
    from .components.optics.arm import Arm
    from .components.optics.beamstop import Beamstop
    from .components.optics.guide_tapering import Guide as TaperedGuide
    from .components.optics.slit import Slit
    from .components.sources.SNS_source import SNS_source
    if moderator_file is None:
        moderator_file = shipped_moderator(SNS_MODERATOR)
    # first mirror and its shield (VERDI_base.py:37-49)
    a1, b1 = ellipse1_minor_axis_len / 2, ellipse1_major_axis_len / 2
    shield1_x, shield1_z = shield_vertex(
        a1, b1, 0., source_width, guide1_start, guide1_start + guide1_len,
        ellipse1_major_axis_len, secsource_size)
    guide11_len = shield1_z - guide1_start
    guide12_len = guide1_len - guide11_len
    focus = float(ellipse_half_opening(guide1_start, a1, b1)) * 2
    focus_dist = guide1_start * .99
    # second mirror, looked at backwards from the sample (:51-67)
    a2, b2 = ellipse2_minor_axis_len / 2, ellipse2_major_axis_len / 2
    z_gs = (ellipse1_major_axis_len + ellipse2_major_axis_len - guide2_start
            - guide2_len)
    shield2_x, shield2_z = shield_vertex(
        a2, b2, 0., sample_width, z_gs, z_gs + guide2_len,
        ellipse2_major_axis_len, secsource_size)
    guide22_len = shield2_z - z_gs
    guide21_len = guide2_len - guide22_len
    guide21_start = ellipse1_major_axis_len + (ellipse2_major_axis_len
                                               - z_gs - guide2_len)
    # segment profiles (:69-93)
    c1 = ellipse1_major_axis_len / 2.
    g11 = elliptic_guide_segments(c1, guide1_start, guide1_start + guide11_len,
                                  guide_n_segments, ellipse1_major_axis_len,
                                  ellipse1_minor_axis_len)
    g12 = elliptic_guide_segments(c1, guide1_start + guide11_len,
                                  guide1_start + guide1_len, guide_n_segments,
                                  ellipse1_major_axis_len,
                                  ellipse1_minor_axis_len)
    c2 = ellipse1_major_axis_len + ellipse2_major_axis_len / 2
    g21 = elliptic_guide_segments(c2, guide21_start,
                                  guide21_start + guide21_len,
                                  guide_n_segments, ellipse2_major_axis_len,
                                  ellipse2_minor_axis_len)
    g22 = elliptic_guide_segments(c2, guide21_start + guide21_len,
                                  guide21_start + guide2_len,
                                  guide_n_segments, ellipse2_major_axis_len,
                                  ellipse2_minor_axis_len)

    def segs(g):  # the loader drops the last segment of a file
        return tuple(v[:-1] for v in g)

    m = guide_mvalue
    ins = instrument("verdi")
    origin = Arm("origin")
    ins.append(origin, position=(0, 0, 0))
    moderator = SNS_source("moderator", moderator_file, Emin, Emax,
                           source_width, source_height, focus_dist, focus,
                           focus, Anorm=0.0009)
    ins.append(moderator, position=(0, 0, 0), relativeTo=origin)
    mod_w, mod_h = source_width * 1.1, source_height * 1.1
    ins.append(Wavelength_monitor("ModeratorSpectrumL", Lmin=0, Lmax=20,
                                  nchan=100, xwidth=mod_w, yheight=mod_h,
                                  filename="moderator_L.h5"),
               position=(0, 0, 1e-5), relativeTo=moderator)
    ins.append(PosDiv_monitor("ModeratorDivergence_xpos", maxdiv=xDivergence,
                              ndiv=1000, npos=100, xwidth=mod_w,
                              yheight=mod_h, filename="moderator_divXpos.h5"),
               position=(0, 0, 2e-5), relativeTo=moderator)
    ins.append(PosDiv_monitor("ModeratorDivergence_ypos", maxdiv=yDivergence,
                              ndiv=1000, npos=100, xwidth=mod_w,
                              yheight=mod_h, filename="moderator_divYpos.h5"),
               position=(0, 0, 3e-5), orientation=(0, 0, 90),
               relativeTo=moderator)
    g1_1 = TaperedGuide("Guide1_1", l=guide11_len, mx=m, my=m,
                        segments=segs(g11))
    ins.append(g1_1, position=(0, 0, guide1_start), relativeTo=moderator)
    ins.append(Beamstop("Shield1_1", xmin=-0.5, xmax=shield1_x, ymin=-0.5,
                        ymax=0.5),
               position=(0, 0, guide11_len + 1e-6), relativeTo=g1_1)
    ins.append(Beamstop("Shield1_2", xmin=-0.5, xmax=0.5, ymin=-0.5,
                        ymax=shield1_x),
               position=(0, 0, guide11_len + 2e-6), relativeTo=g1_1)
    ins.append(TaperedGuide("Guide1_2", l=guide12_len, mx=m, my=m,
                            segments=segs(g12)),
               position=(0, 0, guide11_len + 4e-6), relativeTo=g1_1)
    sec = Arm("SecSource")
    ins.append(sec, position=(0, 0, ellipse1_major_axis_len),
               relativeTo=origin)
    ins.append(PosDiv_monitor("secsrc_divxpos", maxdiv=xDivergence,
                              ndiv=1000, npos=100, xwidth=0.15, yheight=0.15,
                              filename="secsrc_divXpos.h5"),
               position=(0, 0, 1e-7), relativeTo=sec)
    ins.append(PosDiv_monitor("secsrc_divypos", maxdiv=yDivergence,
                              ndiv=1000, npos=100, xwidth=0.15, yheight=0.15,
                              filename="secsrc_divYpos.h5"),
               position=(0, 0, 2e-7), orientation=(0, 0, 90), relativeTo=sec)
    slit = Slit("SecSourceSlit", xmin=-0.01, xmax=0.013, ymin=-0.01,
                ymax=0.013)
    ins.append(slit, position=(0, 0, 1e-5), relativeTo=sec)
    ins.append(Wavelength_monitor("secsrc_IL", Lmin=0, Lmax=20, nchan=100,
                                  xwidth=0.026, yheight=0.026,
                                  filename="secsrc_L.h5"),
               position=(0, 0, 1e-6), relativeTo=slit)
    g2_1 = TaperedGuide("Guide2_1", l=guide21_len, mx=m, my=m,
                        segments=segs(g21))
    ins.append(g2_1, position=(0.0016, 0.0016, guide21_start),
               relativeTo=moderator)
    ins.append(Beamstop("Shield2_1", xmin=-shield2_x, xmax=0.5, ymin=-0.5,
                        ymax=0.5),
               position=(0, 0, guide21_len + 1e-6), relativeTo=g2_1)
    ins.append(Beamstop("Shield2_2", xmin=-0.5, xmax=0.5, ymin=-shield2_x,
                        ymax=0.5),
               position=(0, 0, guide21_len + 2e-6), relativeTo=g2_1)
    ins.append(TaperedGuide("Guide2_2", l=guide22_len, mx=m, my=m,
                            segments=segs(g22)),
               position=(0, 0, guide21_len + 4e-6), relativeTo=g2_1)
    sample = Arm("sampleMantid")
    ins.append(sample, position=(0.001, 0.001, 40.0), relativeTo=origin)
    ins.append(Wavelength_monitor("sample0_IL", Lmin=0, Lmax=20, nchan=100,
                                  xwidth=sample_width, yheight=sample_height,
                                  filename="sample0_L.h5"),
               position=(0, 0, 0), relativeTo=sample)
    pack = Arm("brilliancePack")
    ins.append(pack, position=(0, 0, 0), relativeTo=sample)
    ins.append(Slit("Mask", width=sample_width, height=sample_height),
               position=(0, 0, 0), relativeTo=pack)
    ins.append(PSD_monitor("imagePlate", nx=500, ny=500,
                           xwidth=3 * sample_width,
                           yheight=3 * sample_height, filename="sample_xy.h5"),
               position=(0, 0, 1e-5), relativeTo=pack)
    ins.append(Wavelength_monitor("sampleSpectrumL", Lmin=0, Lmax=20,
                                  nchan=100, xwidth=sample_width,
                                  yheight=sample_height, filename="sample_L.h5"),
               position=(0, 0, 2e-5), relativeTo=pack)
    ins.append(PosDiv_monitor("Divergence_xpos", maxdiv=xDivergence,
                              ndiv=1000, npos=100, xwidth=sample_width,
                              yheight=sample_height,
                              filename="sample_divXpos.h5"),
               position=(0, 0, 3e-5), relativeTo=pack)
    ins.append(PosDiv_monitor("Divergence_ypos", maxdiv=yDivergence,
                              ndiv=1000, npos=100, xwidth=sample_width,
                              yheight=sample_height,
                              filename="sample_divYpos.h5"),
               position=(0, 0, 4e-5), orientation=(0, 0, 90),
               relativeTo=pack)
    return ins


# ------------------------------------------------------------------- UN
def un_kernel(n_levels=8, Qmax=35.0, mu=32.395, sigma=69.847, dE=50.0,
              a=0.00276):
    """The UN sample's kernel (tests/kernels/UN/UN-scatterer.xml): an
    averaged composite of E(Q) kernels, level n at E = n dE (meV) with
    S(Q) = (a Q^2)^n / n! exp(-a Q^2) (S = 1 for n = 0: the elastic line),
    Q 0-35 /A, absorption 32.395 /m and scattering 69.847 /m each."""
    elements = []
    for k in range(n_levels):
        if k == 0:
            S_Q = "1"
        elif k == 1:
            S_Q = f"Q*Q*{a} * exp(-{a} * Q*Q)"
        else:
            S_Q = f"1./{math.factorial(k)} * ({a}*Q*Q)^{k} * exp(-{a} * Q*Q)"
        elements.append(E_Q_Kernel(f"{k * dE:g}", S_Q, 0.0, Qmax, mu, sigma))
    return CompositeKernel(elements, average=True)


def un_ms(Ei=500.0, max_scattered_neutrons=33, max_ms_loops=1,
          max_ms_loops_path1=5, kernel=None, multiple_scattering=True):
    """The UN multiple-scattering benchmark
    (tests/components/samples/UN_test_instrument.py, UN_HMS.py,
    test_ms_UN.py): a 1 x 1 cm source aimed at 8 x 8 mm 1 m away, Ei = 500
    meV +- 1%; the UN cylinder (radius 5.6419 mm, height 1 cm, axis
    vertical) 1.1 m downstream, scattering through un_kernel() with up to
    33 outputs per neutron (1 loop among re-entries, 5 on the first
    passage); an I(Q, E) monitor at the sample, Q 0-30 /A x 150, E -100 to
    400 meV x 100, 10-135 deg in plane, +-26 deg out of it.  `kernel`
    replaces the sample's kernel; multiple_scattering=False scatters once
    (the reference's UN_HSS.py)."""
    from .components.samples.homogeneous_multiple_scatterer import \
        factory as ms_factory
    ins = instrument("un_ms")
    src = Source_simple("src", radius=0.0, width=0.01, height=0.01, dist=1.0,
                        xw=0.008, yh=0.008, E0=Ei, dE=0.01 * Ei, Lambda0=0.0,
                        dLambda=0.0)
    kernel = un_kernel() if kernel is None else kernel
    if multiple_scattering:
        HMS = ms_factory(Cylinder(0.0056419, 0.01), kernel,
                         max_scattered_neutrons=max_scattered_neutrons,
                         max_ms_loops=max_ms_loops,
                         max_ms_loops_path1=max_ms_loops_path1)
    else:  # the single-scattering variant (UN_HSS.py)
        HMS = factory(Cylinder(0.0056419, 0.01), kernel)
    mon = IQE_monitor("iqe_monitor", Ei=Ei, Qmin=0.0, Qmax=30.0, nQ=150,
                      Emin=-100.0, Emax=400.0, nE=100,
                      min_angle_in_plane=10.0, max_angle_in_plane=135.0,
                      min_angle_out_of_plane=-26.0,
                      max_angle_out_of_plane=26.0)
    sample = HMS("sample")
    ins.append(src, position=(0, 0, 0))
    # the cylinder's axis is local z; orientation (90, 0, 0) turns it vertical
    ins.append(sample, position=(0, 0, 1.1), orientation=(90, 0, 0))
    ins.append(mon, position=(0, 0, 0), relativeTo=sample)
    return ins


def composite_box():
    """The Al box of the reference's box tests (_al_box) with a composite
    kernel of three kinds, weights 2 : 1 : 1: the E(Q) dispersion of
    e_q_box, the constant (Q, E) = (2 /A, 15 meV) transfer and isotropic
    elastic scattering, each with Al's coefficients."""
    return _al_box("composite_box", CompositeKernel(
        [E_Q_Kernel("30+20*sin(Q)", "1", 0.0, 10.0, AL_MU, AL_SIGMA),
         ConstantQEKernel(2.0, 15.0, AL_MU, AL_SIGMA),
         IsotropicKernel(AL_MU, AL_SIGMA)], weights=[2, 1, 1]))


# ----------------------------------------------------------------- SANS
def sans2d_image(nx=1475, ny=1100, Qx_max=0.0047176, Qy_max=0.0035176):
    """The synthetic S(Qx, Qy) of the reference's SANS test data
    (tests/components/samples/make_sans2d_data.py:5-31):
    sin(3000 Q)^2 exp(-300 Q) at cell centres over +-Qx_max x +-Qy_max,
    as an image indexed (y, x)."""
    dQx, dQy = 2 * Qx_max / nx, 2 * Qy_max / ny
    Qx = -Qx_max + dQx * (np.arange(nx) + 0.5)
    Qy = -Qy_max + dQy * (np.arange(ny) + 0.5)
    X, Y = np.meshgrid(Qx, Qy)
    Q = np.sqrt(X * X + Y * Y)
    return np.sin(Q * 3000) ** 2 * np.exp(-Q * 300)


def sans2d_grid(image=None):
    """The reference's SANS test instrument
    (tests/components/samples/sans2d_grid_instrument.py:9-37,
    sampleassemblies/sans2d): a 0.3 x 0.3 mm source aimed at a 0.3 x 0.3 mm
    window 9.9 m away, 10 +- 0.65 A; a 3 x 3 cm Al plate 0.2 mm thick at
    10 m, scattering through S(Qx, Qy) on a 1475 x 1100 grid over
    +-0.0047 x +-0.0035 /A; a PSD 250 x 250 over +-7.5 cm 10 m further."""
    if image is None:
        image = sans2d_image()
    ins = instrument("sans2d_grid")
    src = Source_simple("source", radius=0.0, height=0.0003, width=0.0003,
                        dist=9.9, xw=0.0003, yh=0.0003, E0=0.0, dE=0.0,
                        Lambda0=10.0, dLambda=0.65)
    ker = SANS2D_ongrid_Kernel(image, -0.0047176, 0.0047176, -0.0035176,
                               0.0035176, AL_MU, AL_SIGMA)
    HSS = factory(Block(0.03, 0.03, 0.0002), ker)
    mon = PSD_monitor("Ixy", nx=250, ny=250, xmin=-0.075, xmax=0.075,
                      ymin=-0.075, ymax=0.075, filename="Ixy.h5")
    sample = HSS("sample")
    ins.append(src, position=(0, 0, 0))
    ins.append(sample, position=(0, 0, 10.0))
    ins.append(mon, position=(0, 0, 10.0), relativeTo=sample)
    return ins


def dgssxres_box(target=(3.0, 0.0, 0.0), radius=0.025, tof=0.003,
                 dtof=1e-5):
    """The Al box of the reference's box tests (_al_box's source and
    sample) with the DGSSXRes kernel (sampleassemblies/Al-DGSSXResKernel:
    a target 3 m to the side; here a 2.5 cm target radius and a 10 us
    window around 3 ms, which the kernel test uses), and a 4pi theta x tof
    shell of radius 3 m around the sample, binned 180 x 200 over 0-180 deg
    x tof +- 10 us."""
    ins = instrument("dgssxres_box")
    src = Source_simple("src", radius=0.0, width=0.01, height=0.01, dist=1.0,
                        xw=0.008, yh=0.008, E0=70.0, dE=0.1, Lambda0=0.0,
                        dLambda=0.0)
    HSS = factory(Block(0.06, 0.10, 0.01),
                  DGSSXResKernel(target, radius, tof, dtof, AL_MU, AL_SIGMA))
    mon = ThetaTOF_monitor_4Pi("theta_tof", radius=3.0, ntheta=180, ntof=200,
                               tofmin=tof - 1e-5, tofmax=tof + 1e-5,
                               filename="theta_tof.h5")
    ins.append(src, position=(0, 0, 0))
    ins.append(HSS("sample"), position=(0, 0, 2.0))
    ins.append(mon, position=(0, 0, 2.0))
    return ins


# ------------------------------------------------------------ mesh guide
def anyshape_guide_chain(w1=0.035, h1=0.035, w2=0.035, h2=0.035, l=10.0,
                         mesh_file=None, gravity=False):
    """The reference's mesh-guide test instrument
    (tests/components/optics/guide_anyshape_example1_instrument.py with
    acc/test/instrument_factory.py): a 3 x 3 cm source (10 +- 9.5 A) aimed
    at 3.5 x 3.5 cm 0.9 m away; a guide of l = 10 m read from an OFF mesh
    (a w1 x h1 -> w2 x h2 channel written to `mesh_file`, a temporary file
    when None) 1 m downstream, coating R0 0.99, Qc 0.0219, alpha 6.07,
    m 3, W 0.003; 1 m after its exit a PSD (250 x 250 over 10 x 10 cm) and
    position-divergence monitors in x and y (250 x 250).  `gravity`: the
    guide_anyshape_gravity form, g along -y."""
    import tempfile
    from .components.monitors.posdiv_monitor import PosDiv_monitor
    from .components.optics.guide_anyshape import (Guide_anyshape,
                                                   Guide_anyshape_gravity,
                                                   box_guide_mesh, write_off)
    if mesh_file is None:
        fd, mesh_file = tempfile.mkstemp(suffix=".off", prefix="guide_")
        os.close(fd)
    write_off(mesh_file, *box_guide_mesh(w1, h1, w2, h2, l))
    ins = instrument("anyshape_guide_chain")
    src = Source_simple("source", radius=0.0, width=0.03, height=0.03,
                        dist=0.9, xw=0.035, yh=0.035, Lambda0=10.0,
                        dLambda=9.5)
    G = Guide_anyshape_gravity if gravity else Guide_anyshape
    guide = G("guide", R0=0.99, Qc=0.0219, alpha=6.07, m=3, W=0.003,
              geometry=mesh_file)
    z = 2 * 1.0 + l
    ins.append(src, position=(0, 0, 0))
    ins.append(guide, position=(0, 0, 1.0))
    ins.append(PSD_monitor("Ixy", nx=250, ny=250, xwidth=0.1, yheight=0.1,
                           filename="Ixy.h5"), position=(0, 0, z))
    ins.append(PosDiv_monitor("Ixdivx", npos=250, ndiv=250, xwidth=0.1,
                              yheight=0.1, filename="Ixdivx.h5"),
               position=(0, 0, z))
    ins.append(PosDiv_monitor("Ixdivy", npos=250, ndiv=250, xwidth=0.1,
                              yheight=0.1, filename="Ixdivy.h5"),
               position=(0, 0, z), orientation=(0, 0, 90))
    return ins
