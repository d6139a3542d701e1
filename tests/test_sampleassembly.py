"""Sample assemblies (acc/components/samples/__init__.py:1-48): the
reference's sample-assembly fixtures (tests/golden/sampleassemblies, copied
from its tests/components/samples/sampleassemblies) read into shapes and
kernels, and sample scripts written the way the reference's
HSS_isotropic_sphere.py / UN_HSS.py are (loadFirstHomogeneousScatterer ->
factory) run through run_script on the oracle (CPU) and on the GPU."""

import math
import os

import numpy as np
import pytest

from acc_gb300 import kernels as K
from acc_gb300 import sampleassembly as SA
from acc_gb300.components.samples import (getAbsScttCoeffs,
                                          loadFirstHomogeneousScatterer)
from acc_gb300.geometry import Block, Cylinder, Difference, Sphere

HERE = os.path.dirname(os.path.abspath(__file__))
SAMPLES = os.path.join(HERE, "golden", "sampleassemblies")


def assembly(name):
    return os.path.join(SAMPLES, name, "sampleassembly.xml")


def test_unit_expressions():
    m, s = SA.UNITS["m"], SA.UNITS["s"]
    assert SA.quantity("1*cm", m) == pytest.approx(0.01)
    assert SA.quantity("10./m", 1 / m) == pytest.approx(10.0)
    assert SA.quantity("32.395/meter", 1 / m) == pytest.approx(32.395)
    assert SA.quantity("3/angstrom", 1 / SA.UNITS["angstrom"]) == \
        pytest.approx(3.0)
    assert SA.quantity("30*meV", SA.UNITS["meV"]) == 30.0
    assert SA.quantity("2.*millisecond + 1.*millisecond", s) == \
        pytest.approx(0.003)
    assert SA.quantity("3.*meter,0.*meter,0.*meter", m) == (3.0, 0.0, 0.0)
    assert SA.quantity("1e-20") == 1e-20
    with pytest.raises(ValueError):
        SA.quantity("furlong")
    with pytest.raises(ValueError):
        SA.quantity("__import__('os')")


def test_isotropic_sphere_assembly():
    hs = loadFirstHomogeneousScatterer(assembly("isotropic_sphere"))
    assert isinstance(hs.shape(), Sphere) and hs.shape().radius == 0.01
    k = hs.kernel()
    assert isinstance(k, K.IsotropicKernel)
    assert getAbsScttCoeffs(k) == (10.0, 10.0)


def test_hollow_cylinder_and_box_assemblies():
    hs = loadFirstHomogeneousScatterer(assembly("isotropic_hollowcylinder"))
    s = hs.shape()
    assert isinstance(s, Difference)
    assert (s.op1.radius, s.op1.height) == pytest.approx((0.02, 0.06))
    assert (s.op2.radius, s.op2.height) == pytest.approx((0.01, 0.07))
    b = loadFirstHomogeneousScatterer(assembly("isotropic_box")).shape()
    assert isinstance(b, Block)
    assert (b.width, b.height, b.thickness) == pytest.approx((.01,) * 3)


def test_coefficients_from_the_unit_cell():
    """The Al E(Q) and constant-(Q, E) kernels carry no coefficients: they
    come from Al.xyz (4 Al atoms in a 4.04 A cube): mu = 4 x 0.231 b /
    65.939 A^3 x 100 = 1.40129 /m, sigma = 4 x (1.495 + 0.0082) b / 65.939
    A^3 x 100 = 9.11869 /m."""
    for name in ("Al-E_Q_kernel", "Al-constantqekernel"):
        hs = loadFirstHomogeneousScatterer(assembly(name))
        assert isinstance(hs.shape(), Block)
        assert hs.cell.volume == pytest.approx(4.04 ** 3)
        mu, sigma = getAbsScttCoeffs(hs.kernel())
        assert mu == pytest.approx(1.40129, rel=1e-5)
        assert sigma == pytest.approx(9.11869, rel=1e-5)
    k = loadFirstHomogeneousScatterer(assembly("Al-E_Q_kernel")).kernel()
    assert (k.E_Q, k.S_Q, k.Qmin, k.Qmax) == ("30+20*sin(Q)", "1", 0.0, 10.0)
    k = loadFirstHomogeneousScatterer(assembly("Al-constantqekernel")).kernel()
    assert (k.Q, k.E) == (3.0, 30.0)


def test_un_assembly_is_the_un_kernel():
    """UN: a cylinder r = 0.56419 cm, h = 1 cm with an averaged container of
    eight E(Q) kernels; packed, it is the kernel the UN benchmark builds
    (instruments.un_kernel)."""
    from acc_gb300 import instruments
    from acc_gb300.components.samples.homogeneous_single_scatterer import \
        factory
    from acc_gb300.engine import build_chain
    from acc_gb300.memory import HostBinder
    hs = loadFirstHomogeneousScatterer(assembly("UN"))
    s = hs.shape()
    assert isinstance(s, Cylinder)
    assert (s.radius, s.height) == pytest.approx((0.0056419, 0.01))
    k = hs.kernel()
    assert isinstance(k, K.CompositeKernel) and len(k.elements) == 8
    ref = instruments.un_kernel()
    for a, b in zip(k.elements, ref.elements):
        np.testing.assert_array_equal(a.program(), b.program())
        assert (a.Qmin, a.Qmax, a.absorption_coefficient,
                a.scattering_coefficient) == (b.Qmin, b.Qmax,
                                              b.absorption_coefficient,
                                              b.scattering_coefficient)
    c1 = build_chain([factory(s, k)("u")], binder=HostBinder())
    c2 = build_chain([factory(s, ref)("u")], binder=HostBinder())
    for i in range(c1.ncomp):
        assert list(c1.comp[i].ip) == list(c2.comp[i].ip)
        assert list(c1.comp[i].dp) == list(c2.comp[i].dp)


def test_powder_assembly_reads_the_laz_file():
    """The Al powder scatterer lists a peaks.py kernel and then a .laz
    kernel; the last one is the scatterer's: 26 reflections of the .laz
    table, q = 2 pi / d, F^2 = |F|^2, multiplicity from its MULT column, in
    the 4.04932 A cell, cross sections 4 x the per-atom header values."""
    hs = loadFirstHomogeneousScatterer(
        assembly("Al-simplepowderdiffractionkernel"))
    k = hs.kernel()
    assert isinstance(k, K.SimplePowderDiffractionKernel)
    assert isinstance(hs.shape(), Sphere) and hs.shape().radius == 0.003
    assert len(k.peaks) == 26
    assert k.unitcell_volume == pytest.approx(4.049320 ** 3)
    p0 = k.peaks[0]
    assert p0.q == pytest.approx(2 * math.pi / 2.3379)
    assert p0.F_squared == pytest.approx(1.3 ** 2)
    assert p0.multiplicity == 8
    assert k.pd.absorption_cross_section == pytest.approx(4 * 0.231)
    assert k.absorption_coefficient == pytest.approx(
        4 * 0.231 / 4.049320 ** 3 * 100)
    # the peaks.py form of the same sample (the first kernel of the file)
    peaks, vol, xs = SA.read_peaks_py(os.path.join(
        SAMPLES, "Al-simplepowderdiffractionkernel", "peaks.py"))
    assert [p.q for p in peaks] == [1.92, 3.1353]
    assert vol == pytest.approx(4.049320 ** 3)
    assert xs == pytest.approx((4 * 1.495, 4 * 0.0082, 4 * 0.231))


SAMPLE_SCRIPT = '''
import os
from mcvine.acc.components.samples.homogeneous_single_scatterer import factory
from mcvine.acc.components.samples import loadFirstHomogeneousScatterer
path = {path!r}
hs = loadFirstHomogeneousScatterer(path)
HSSbase = factory(shape=hs.shape(), kernel=hs.kernel())
class HSS(HSSbase): pass
'''

INSTRUMENT_SCRIPT = '''
import mcvine
from mcvine.acc.components.sources.source_simple import Source_simple
from mcvine.acc.components.monitors.psd_monitor_4pi import PSD_monitor_4Pi
from sample_{tag} import HSS

def instrument(Ei=60.0):
    ins = mcvine.instrument()
    ins.append(Source_simple("src", radius=0., width=0.01, height=0.01,
                             dist=1.0, xw=0.008, yh=0.008, E0=Ei, dE=0.1 * Ei),
               position=(0, 0, 0))
    ins.append(HSS("sample"), position=(0, 0, 1.0))
    ins.append(PSD_monitor_4Pi("mon", radius=3., nphi=30, ntheta=30,
                               filename="psd_4pi.h5"), position=(0, 0, 1.0))
    return ins
'''


def write_scripts(tmp_path, tag, name):
    (tmp_path / f"sample_{tag}.py").write_text(
        SAMPLE_SCRIPT.format(path=assembly(name)))
    script = tmp_path / f"instrument_{tag}.py"
    script.write_text(INSTRUMENT_SCRIPT.format(tag=tag))
    return str(script)


SCRIPTS = {"sphere": "isotropic_sphere", "un": "UN",
           "powder": "Al-simplepowderdiffractionkernel",
           "eq": "Al-E_Q_kernel"}


@pytest.mark.parametrize("tag", list(SCRIPTS))
def test_sample_script_runs_on_the_oracle(tmp_path, tag):
    """The scripts load under the mcvine alias and their chain runs on the
    oracle; the sample scatters (the 4pi monitor sees more than the
    transmitted beam's bins)."""
    import sys
    from acc_gb300 import run_script
    sys.path.insert(0, str(tmp_path))
    try:
        ins = run_script.loadInstrument(write_scripts(tmp_path, tag,
                                                      SCRIPTS[tag]))
    finally:
        sys.path.remove(str(tmp_path))
    import sys as _s
    _s.path.insert(0, HERE)
    from helpers import oracle_run
    ot, st, _, _ = oracle_run(ins, 200_000, seed=3)
    assert st["processed"] == 200_000
    (_, h), = ot.items()
    assert (h[0] > 0).sum() > 20


@pytest.mark.gpu
@pytest.mark.parametrize("tag", list(SCRIPTS))
def test_sample_script_runs_through_run_script(tmp_path, tag, engine_lib):
    """run_script.run on the script (FP64, the reference's default) gives
    the oracle's histogram: identical counts, sums within 1e-12 (scaled by
    1/ncount as run_script saves them)."""
    import sys
    from acc_gb300 import run_script
    sys.path.insert(0, HERE)
    from helpers import oracle_run
    n = 200_000
    script = write_scripts(tmp_path, tag, SCRIPTS[tag])
    sys.path.insert(0, str(tmp_path))
    try:
        ins = run_script.run(script, str(tmp_path / "out"), n, _acc_seed=5)
        ref = run_script.loadInstrument(script)
    finally:
        sys.path.remove(str(tmp_path))
    g = ins.components[-1].out.reshape(3, -1)
    ot, _, _, _ = oracle_run(ref, n, seed=5)
    (_, o), = ot.items()
    o = o.reshape(3, -1)
    np.testing.assert_array_equal(g[0], o[0])
    np.testing.assert_allclose(g[1:], o[1:], rtol=1e-12, atol=1e-300)
    assert o[0].sum() > 0
